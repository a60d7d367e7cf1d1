// Mass properties of many meshes on the device: the reference's mesh set-up
// (model/mesh.cpp:53-91 initInertiaDataVolume, :93-130
// initInertiaDataSurface; model/inertia.cpp:20-84) for large mesh sets, such
// as the 16,384 distinct noisy icospheres of the open-box scene.
//
// One thread per mesh, in the operation order of the library's host set-up
// (host/d2g_scene.cpp mass_volume / mass_surface), so a mesh gets the same
// bits on the GPU as on the host:
//   * closed surfaces (volume model): the tetrahedra of the faces with the
//     origin (the reference tetrahedralises with tetgen, absent here; the sum
//     over face tetrahedra is the divergence theorem's exact volume
//     integral): volume, centre of mass, then the unit-density inertia tensor
//     about the centre of mass with tetrahedronInertiaTensor's terms;
//   * thin shells (surface model): triangle area times thickness per face,
//     the centroid-weighted centre of mass, then the point inertia tensors of
//     the three vertices per face;
//   * the inverse of the 3x3 tensor by cofactors.
// Sequential per mesh: the sums keep the host's order (bit-identical), and
// there are as many threads as meshes.
#include "d2g_geom.cuh"
#include "d2g_internal.hpp"

namespace d2g {
namespace {

constexpr int kMassBlock = 64;

__device__ V3 mvert(const double* V, const int32_t* F, int f, int k) {
    const double* p = V + 3 * (size_t)F[3 * (size_t)f + k];
    return mk(p[0], p[1], p[2]);
}

// model/inertia.cpp:20-73 tetrahedronInertiaTensor (Tonon 2005) with the
// reference's placement of the product terms; `sign` carries the orientation.
__device__ void tet_inertia_add(V3 a, V3 b, V3 c, V3 d, double sign, double* I) {
    const double A[3] = {a.x, a.y, a.z}, B[3] = {b.x, b.y, b.z}, C[3] = {c.x, c.y, c.z}, D[3] = {d.x, d.y, d.z};
    const double detJ = dot(a - d, cross(b - d, c - d));
    auto sq = [&](int k) {
        return A[k] * A[k] + A[k] * B[k] + B[k] * B[k] + A[k] * C[k] + B[k] * C[k] + C[k] * C[k] + A[k] * D[k] +
               B[k] * D[k] + C[k] * D[k] + D[k] * D[k];
    };
    auto pr = [&](int i, int j) {
        return 2 * A[i] * A[j] + B[i] * A[j] + C[i] * A[j] + D[i] * A[j] + A[i] * B[j] + 2 * B[i] * B[j] +
               C[i] * B[j] + D[i] * B[j] + A[i] * C[j] + B[i] * C[j] + 2 * C[i] * C[j] + D[i] * C[j] + A[i] * D[j] +
               B[i] * D[j] + C[i] * D[j] + 2 * D[i] * D[j];
    };
    const double ixx = sign * detJ * (sq(1) + sq(2)) / 60;
    const double iyy = sign * detJ * (sq(0) + sq(2)) / 60;
    const double izz = sign * detJ * (sq(0) + sq(1)) / 60;
    const double iyz = -sign * detJ * pr(1, 2) / 120;
    const double ixy = -sign * detJ * pr(0, 2) / 120;
    const double ixz = -sign * detJ * pr(0, 1) / 120;
    const double R[9] = {ixx, ixy, ixz, ixy, iyy, iyz, ixz, iyz, izz};
    for (int k = 0; k < 9; k++) I[k] += R[k];
}

__device__ void inv3_cofactor(const double* m, double* r) {
    const double c00 = m[4] * m[8] - m[5] * m[7];
    const double c01 = m[5] * m[6] - m[3] * m[8];
    const double c02 = m[3] * m[7] - m[4] * m[6];
    const double det = (m[0] * c00 + m[1] * c01) + m[2] * c02;
    const double id = 1.0 / det;
    r[0] = c00 * id;
    r[1] = (m[2] * m[7] - m[1] * m[8]) * id;
    r[2] = (m[1] * m[5] - m[2] * m[4]) * id;
    r[3] = c01 * id;
    r[4] = (m[0] * m[8] - m[2] * m[6]) * id;
    r[5] = (m[2] * m[3] - m[0] * m[5]) * id;
    r[6] = c02 * id;
    r[7] = (m[1] * m[6] - m[0] * m[7]) * id;
    r[8] = (m[0] * m[4] - m[1] * m[3]) * id;
}

__device__ double area3(V3 A, V3 B, V3 C) { return 0.5 * norm(cross(A - C, B - C)); }

// out per mesh (22 doubles): volume, centre of mass (3), unit-density inertia
// tensor about it (9, row major), its inverse (9).
__global__ void __launch_bounds__(kMassBlock) k_mass_props(int n, const double* __restrict__ V,
                                                           const int32_t* __restrict__ F,
                                                           const int32_t* __restrict__ voff,
                                                           const int32_t* __restrict__ foff,
                                                           const uint8_t* __restrict__ surface, double thickness,
                                                           double* __restrict__ out) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    const double* Vm = V + 3 * (size_t)voff[m];
    const int f0 = foff[m], f1 = foff[m + 1];
    double vol = 0.0, I[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, Ii[9];
    V3 com = mk(0, 0, 0);
    if (surface && surface[m]) {
        for (int f = f0; f < f1; f++) {
            const V3 A = mvert(Vm, F, f, 0), B = mvert(Vm, F, f, 1), C = mvert(Vm, F, f, 2);
            const double tv = area3(A, B, C) * thickness;
            vol += tv;
            com = com + (((A + B) + C) * (1.0 / 3.0)) * tv;
        }
        com = com * (1.0 / vol);
        for (int f = f0; f < f1; f++) {
            const V3 A = mvert(Vm, F, f, 0) - com, B = mvert(Vm, F, f, 1) - com, C = mvert(Vm, F, f, 2) - com;
            const double tv = area3(A, B, C) * thickness;
            const V3 P[3] = {A, B, C};
            for (int k = 0; k < 3; k++) {  // model/inertia.cpp:75-84 pointInertiaTensor
                const double x = P[k].x, y = P[k].y, z = P[k].z;
                const double pi[9] = {y * y + z * z, -x * y, -x * z, -x * y, x * x + z * z, -y * z,
                                      -x * z, -y * z, x * x + y * y};
                for (int j = 0; j < 9; j++) I[j] += tv * pi[j] / 3.0;
            }
        }
    } else {
        for (int f = f0; f < f1; f++) {
            const V3 a = mvert(Vm, F, f, 0), b = mvert(Vm, F, f, 1), c = mvert(Vm, F, f, 2);
            const double v = dot(a, cross(b, c)) / 6.0;
            vol += v;
            com = com + ((a + b) + c) * (v / 4.0);
        }
        com = com * (1.0 / vol);
        for (int f = f0; f < f1; f++)
            tet_inertia_add(mvert(Vm, F, f, 0) - com, mvert(Vm, F, f, 1) - com, mvert(Vm, F, f, 2) - com, mk(0, 0, 0),
                            1.0, I);
    }
    inv3_cofactor(I, Ii);
    double* o = out + 22 * (size_t)m;
    o[0] = vol;
    o[1] = com.x;
    o[2] = com.y;
    o[3] = com.z;
    for (int k = 0; k < 9; k++) {
        o[4 + k] = I[k];
        o[13 + k] = Ii[k];
    }
}

}  // namespace

int run_mass_properties(d2g_ctx* ctx, const double* d_V, const int32_t* d_F, const int32_t* d_voff,
                        const int32_t* d_foff, const uint8_t* d_surface, int n_meshes, double thickness,
                        double* d_out) {
    if (n_meshes > 0) {
        k_mass_props<<<(n_meshes + kMassBlock - 1) / kMassBlock, kMassBlock, 0, ctx->stream>>>(
            n_meshes, d_V, d_F, d_voff, d_foff, d_surface, thickness, d_out);
        ctx->eng.launches++;
    }
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

}  // namespace d2g
