// Oracle (test infrastructure only): mass properties restated from the
// reference, in its own expression order:
//   model/inertia.cpp:20-73   tetrahedronInertiaTensor (Tonon 2005), unit
//                             density -1 as the reference sets it
//   model/inertia.cpp:75-84   pointInertiaTensor
//   model/mesh.cpp:53-91      initInertiaDataVolume
//   model/mesh.cpp:93-130     initInertiaDataSurface
// The volume model tetrahedralises the mesh with tetgen (absent here); this
// restatement uses the tetrahedra of the faces with the origin instead, each
// ordered (a, c, b, origin) so that an outward face gives the orientation
// whose determinant the reference's density -1 expects, and |det| / 6 as the
// tetrahedron volume (igl::volume).  The divergence theorem makes the sums
// the exact volume integrals of the closed surface.
#pragma once
#include <cmath>
#include <vector>

#include "d2o_geom.hpp"

namespace d2o {

// model/inertia.cpp:20-73 (the long sums left to right, as written there)
inline M3 tetrahedron_inertia(V3 a, V3 b, V3 c, V3 d) {
    const double density = -1.0;
    const double detJ = dot(a - d, cross(b - d, c - d));
    const double A[3] = {a.x, a.y, a.z}, B[3] = {b.x, b.y, b.z}, C[3] = {c.x, c.y, c.z}, D[3] = {d.x, d.y, d.z};
    auto diag = [&](int i, int j) {
        return A[i] * A[i] + A[i] * B[i] + B[i] * B[i] + A[i] * C[i] + B[i] * C[i] + C[i] * C[i] + A[i] * D[i] +
               B[i] * D[i] + C[i] * D[i] + D[i] * D[i] + A[j] * A[j] + A[j] * B[j] + B[j] * B[j] + A[j] * C[j] +
               B[j] * C[j] + C[j] * C[j] + A[j] * D[j] + B[j] * D[j] + C[j] * D[j] + D[j] * D[j];
    };
    auto off = [&](int i, int j) {
        return 2 * A[i] * A[j] + B[i] * A[j] + C[i] * A[j] + D[i] * A[j] + A[i] * B[j] + 2 * B[i] * B[j] +
               C[i] * B[j] + D[i] * B[j] + A[i] * C[j] + B[i] * C[j] + 2 * C[i] * C[j] + D[i] * C[j] + A[i] * D[j] +
               B[i] * D[j] + C[i] * D[j] + 2 * D[i] * D[j];
    };
    const double ixx = density * detJ * diag(1, 2) / 60;
    const double iyy = density * detJ * diag(0, 2) / 60;
    const double izz = density * detJ * diag(0, 1) / 60;
    const double iyz = -density * detJ * off(1, 2) / 120;
    const double ixy = -density * detJ * off(0, 2) / 120;
    const double ixz = -density * detJ * off(0, 1) / 120;
    M3 r;
    const double v[9] = {ixx, ixy, ixz, ixy, iyy, iyz, ixz, iyz, izz};
    for (int k = 0; k < 9; k++) r.m[k / 3][k % 3] = v[k];
    return r;
}

// model/inertia.cpp:75-84
inline M3 point_inertia(V3 p) {
    const double x = p.x, y = p.y, z = p.z;
    M3 r;
    const double v[9] = {y * y + z * z, -x * y, -x * z, -x * y, x * x + z * z, -y * z, -x * z, -y * z, x * x + y * y};
    for (int k = 0; k < 9; k++) r.m[k / 3][k % 3] = v[k];
    return r;
}

struct MassOut {
    double volume = 0;
    V3 com{0, 0, 0};
    M3 unit_inertia{};
};

// model/mesh.cpp:53-91 with the face tetrahedra in place of tetgen's.
inline MassOut mass_volume_model(const std::vector<V3>& V, const std::vector<int>& F) {
    MassOut o;
    const size_t nf = F.size() / 3;
    std::vector<double> vol(nf);
    for (size_t f = 0; f < nf; f++) {
        const V3 a = V[F[3 * f]], b = V[F[3 * f + 1]], c = V[F[3 * f + 2]];
        vol[f] = dot(a, cross(b, c)) / 6.0;  // igl::volume's |det| / 6 for the (a, c, b, 0) tetrahedron
        o.volume += vol[f];
    }
    V3 com{0, 0, 0};
    for (size_t f = 0; f < nf; f++) {
        const V3 a = V[F[3 * f]], b = V[F[3 * f + 1]], c = V[F[3 * f + 2]], d{0, 0, 0};
        com = com + ((((a + c) + b) + d) * vol[f]) / 4.0;
    }
    com = com / o.volume;
    o.com = com;
    for (size_t f = 0; f < nf; f++) {
        const V3 a = V[F[3 * f]] - com, b = V[F[3 * f + 1]] - com, c = V[F[3 * f + 2]] - com, d = V3{0, 0, 0} - com;
        const M3 t = tetrahedron_inertia(a, c, b, d);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) o.unit_inertia.m[i][j] += t.m[i][j];
    }
    return o;
}

// model/mesh.cpp:93-130
inline MassOut mass_surface_model(const std::vector<V3>& V, const std::vector<int>& F, double thickness) {
    MassOut o;
    const size_t nf = F.size() / 3;
    V3 com{0, 0, 0};
    for (size_t f = 0; f < nf; f++) {
        const V3 a = V[F[3 * f]], b = V[F[3 * f + 1]], c = V[F[3 * f + 2]];
        const double t_vol = tri_area(Tri{a, b, c}) * thickness;
        const V3 avg = ((a + b) + c) / 3.0;
        o.volume += t_vol;
        com = com + avg * t_vol;
    }
    o.com = com / o.volume;
    for (size_t f = 0; f < nf; f++) {
        const V3 a = V[F[3 * f]] - o.com, b = V[F[3 * f + 1]] - o.com, c = V[F[3 * f + 2]] - o.com;
        const M3 ia = point_inertia(a), ib = point_inertia(b), ic = point_inertia(c);
        const double t_vol = tri_area(Tri{a, b, c}) * thickness;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) o.unit_inertia.m[i][j] += t_vol * ((ia.m[i][j] + ib.m[i][j]) + ic.m[i][j]) / 3.0;
    }
    return o;
}

}  // namespace d2o
