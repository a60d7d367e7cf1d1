// Oracle (test infrastructure only): geometry primitives restated from the
// reference's common/ headers, in plain C++ (no Eigen), FP64 throughout except
// where the reference itself computes in float.
//
// Evaluation order is declared here and mirrored by the CUDA kernels so that
// both produce identical bits (compile with -ffp-contract=off):
//   dot(a,b)        = (a.x*b.x + a.y*b.y) + a.z*b.z
//   cross(a,b)      = (a.y*b.z - a.z*b.y, a.z*b.x - a.x*b.z, a.x*b.y - a.y*b.x)
//   M*v (4x4)       = ((m[r][0]*v0 + m[r][1]*v1) + m[r][2]*v2) + m[r][3]*v3
//   (A*B)[i][j]     = ((A[i][0]*B[0][j] + A[i][1]*B[1][j]) + A[i][2]*B[2][j]) + A[i][3]*B[3][j]
//   normalized(v)   = v / sqrt(dot(v,v)) if dot(v,v) > 0 else v   (Eigen >= 3.3 semantics)
//   std::min(a,b)   = (b < a) ? b : a ;  std::max(a,b) = (a < b) ? b : a
#pragma once
#include <cmath>
#include <cstdint>
#include <limits>

#include "d2o_math.hpp"

namespace d2o {

struct V3 {
    double x, y, z;
};

inline V3 v3(double x, double y, double z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, double s) { return V3{a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(double s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
inline V3 operator/(V3 a, double s) { return V3{a.x / s, a.y / s, a.z / s}; }
inline bool operator!=(V3 a, V3 b) { return a.x != b.x || a.y != b.y || a.z != b.z; }
inline double dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
    return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double norm(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 normalized(V3 a) {
    const double z = dot(a, a);
    if (z > 0.0) {
        const double s = std::sqrt(z);
        return V3{a.x / s, a.y / s, a.z / s};
    }
    return a;
}
inline double dmin(double a, double b) { return (b < a) ? b : a; }
inline double dmax(double a, double b) { return (a < b) ? b : a; }
inline double dclamp(double v, double lo, double hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }
// common/basic_utils.h:10-19
inline double clamp01(double t) {
    if (t < 0) return 0;
    if (t > 1) return 1;
    return t;
}
// common/basic_utils.h:22-25, 30-33: A*(1-t) + B*t
inline V3 lerp(V3 A, V3 B, double t) {
    const double u = 1 - t;
    return V3{A.x * u + B.x * t, A.y * u + B.y * t, A.z * u + B.z * t};
}
inline double lerp(double A, double B, double t) { return A * (1 - t) + B * t; }

// ---------------------------------------------------------------- 4x4 ------
struct M4 {
    double m[4][4];
};

inline M4 mat_mul(const M4& A, const M4& B) {
    M4 R;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            R.m[i][j] = ((A.m[i][0] * B.m[0][j] + A.m[i][1] * B.m[1][j]) + A.m[i][2] * B.m[2][j]) +
                        A.m[i][3] * B.m[3][j];
    return R;
}

// Homogeneous multiply then divide by w: common/basic_utils.h:35-40.
inline V3 xform(V3 p, const M4& M) {
    double v[4];
    for (int r = 0; r < 4; r++)
        v[r] = ((M.m[r][0] * p.x + M.m[r][1] * p.y) + M.m[r][2] * p.z) + M.m[r][3] * 1.0;
    return V3{v[0] / v[3], v[1] / v[3], v[2] / v[3]};
}

// (1-t)*S + t*E, element-wise (continuous_comparison.h:58,86).
inline M4 mat_lerp(const M4& S, const M4& E, double t) {
    M4 R;
    const double u = 1 - t;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) R.m[i][j] = u * S.m[i][j] + t * E.m[i][j];
    return R;
}

// General 4x4 inverse by Laplace expansion in complementary 2x2 minors
// (the cofactor method; Eigen's own kernel is not reproducible here).
inline M4 mat_inverse(const M4& M) {
    const double(*a)[4] = M.m;
    const double s0 = a[0][0] * a[1][1] - a[1][0] * a[0][1];
    const double s1 = a[0][0] * a[1][2] - a[1][0] * a[0][2];
    const double s2 = a[0][0] * a[1][3] - a[1][0] * a[0][3];
    const double s3 = a[0][1] * a[1][2] - a[1][1] * a[0][2];
    const double s4 = a[0][1] * a[1][3] - a[1][1] * a[0][3];
    const double s5 = a[0][2] * a[1][3] - a[1][2] * a[0][3];
    const double c5 = a[2][2] * a[3][3] - a[3][2] * a[2][3];
    const double c4 = a[2][1] * a[3][3] - a[3][1] * a[2][3];
    const double c3 = a[2][1] * a[3][2] - a[3][1] * a[2][2];
    const double c2 = a[2][0] * a[3][3] - a[3][0] * a[2][3];
    const double c1 = a[2][0] * a[3][2] - a[3][0] * a[2][2];
    const double c0 = a[2][0] * a[3][1] - a[3][0] * a[2][1];
    const double det = ((((s0 * c5 - s1 * c4) + s2 * c3) + s3 * c2) - s4 * c1) + s5 * c0;
    const double id = 1.0 / det;
    M4 R;
    R.m[0][0] = ((a[1][1] * c5 - a[1][2] * c4) + a[1][3] * c3) * id;
    R.m[0][1] = ((-a[0][1] * c5 + a[0][2] * c4) - a[0][3] * c3) * id;
    R.m[0][2] = ((a[3][1] * s5 - a[3][2] * s4) + a[3][3] * s3) * id;
    R.m[0][3] = ((-a[2][1] * s5 + a[2][2] * s4) - a[2][3] * s3) * id;
    R.m[1][0] = ((-a[1][0] * c5 + a[1][2] * c2) - a[1][3] * c1) * id;
    R.m[1][1] = ((a[0][0] * c5 - a[0][2] * c2) + a[0][3] * c1) * id;
    R.m[1][2] = ((-a[3][0] * s5 + a[3][2] * s2) - a[3][3] * s1) * id;
    R.m[1][3] = ((a[2][0] * s5 - a[2][2] * s2) + a[2][3] * s1) * id;
    R.m[2][0] = ((a[1][0] * c4 - a[1][1] * c2) + a[1][3] * c0) * id;
    R.m[2][1] = ((-a[0][0] * c4 + a[0][1] * c2) - a[0][3] * c0) * id;
    R.m[2][2] = ((a[3][0] * s4 - a[3][1] * s2) + a[3][3] * s0) * id;
    R.m[2][3] = ((-a[2][0] * s4 + a[2][1] * s2) - a[2][3] * s0) * id;
    R.m[3][0] = ((-a[1][0] * c3 + a[1][1] * c1) - a[1][2] * c0) * id;
    R.m[3][1] = ((a[0][0] * c3 - a[0][1] * c1) + a[0][2] * c0) * id;
    R.m[3][2] = ((-a[3][0] * s3 + a[3][1] * s1) - a[3][2] * s0) * id;
    R.m[3][3] = ((a[2][0] * s3 - a[2][1] * s1) + a[2][2] * s0) * id;
    return R;
}

// ---------------------------------------------------------- quaternion -----
struct Quat {
    double w, x, y, z;
};

// Hamilton product a*b.
inline Quat qmul(const Quat& a, const Quat& b) {
    return Quat{((a.w * b.w - a.x * b.x) - a.y * b.y) - a.z * b.z,
                ((a.w * b.x + a.x * b.w) + a.y * b.z) - a.z * b.y,
                ((a.w * b.y + a.y * b.w) + a.z * b.x) - a.x * b.z,
                ((a.w * b.z + a.z * b.w) + a.x * b.y) - a.y * b.x};
}

struct M3 {
    double m[3][3];
};

// Rotation matrix of a (not necessarily unit) quaternion, Eigen's formula.
inline M3 qmat(const Quat& q) {
    const double tx = 2.0 * q.x, ty = 2.0 * q.y, tz = 2.0 * q.z;
    const double twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
    const double txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
    const double tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
    M3 R;
    R.m[0][0] = 1.0 - (tyy + tzz);
    R.m[0][1] = txy - twz;
    R.m[0][2] = txz + twy;
    R.m[1][0] = txy + twz;
    R.m[1][1] = 1.0 - (txx + tzz);
    R.m[1][2] = tyz - twx;
    R.m[2][0] = txz - twy;
    R.m[2][1] = tyz + twx;
    R.m[2][2] = 1.0 - (txx + tyy);
    return R;
}

inline M3 m3_mul(const M3& A, const M3& B) {
    M3 R;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            R.m[i][j] = (A.m[i][0] * B.m[0][j] + A.m[i][1] * B.m[1][j]) + A.m[i][2] * B.m[2][j];
    return R;
}
inline M3 m3_transpose(const M3& A) {
    M3 R;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) R.m[i][j] = A.m[j][i];
    return R;
}
inline V3 m3_vec(const M3& A, V3 v) {
    return V3{(A.m[0][0] * v.x + A.m[0][1] * v.y) + A.m[0][2] * v.z,
              (A.m[1][0] * v.x + A.m[1][1] * v.y) + A.m[1][2] * v.z,
              (A.m[2][0] * v.x + A.m[2][1] * v.y) + A.m[2][2] * v.z};
}
// v^T * A * v evaluated as (v^T*A)*v (strategies/contact_force/sequential_impulses.cpp:144).
inline double quad_form(V3 v, const M3& A) {
    const double r0 = (v.x * A.m[0][0] + v.y * A.m[1][0]) + v.z * A.m[2][0];
    const double r1 = (v.x * A.m[0][1] + v.y * A.m[1][1]) + v.z * A.m[2][1];
    const double r2 = (v.x * A.m[0][2] + v.y * A.m[1][2]) + v.z * A.m[2][2];
    return (r0 * v.x + r1 * v.y) + r2 * v.z;
}

// common/basic_utils.h:79-95 transformationMatrix(quaternion, translation).
inline M4 transformation(const Quat& q, V3 t) {
    const M3 R = qmat(q);
    M4 T;
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) T.m[i][j] = R.m[i][j];
    }
    T.m[0][3] = t.x;
    T.m[1][3] = t.y;
    T.m[2][3] = t.z;
    T.m[3][0] = 0.0;
    T.m[3][1] = 0.0;
    T.m[3][2] = 0.0;
    T.m[3][3] = 1.0;
    return T;
}

// common/basic_utils.cpp:36-44 quaternion exponential of a rotation vector.
inline Quat qexp(V3 d) {
    if (norm(d) == 0.0) return Quat{1.0, 0.0, 0.0, 0.0};
    const double n = norm(d);
    const double s = psin(n);
    const V3 v = V3{(d.x / n) * s, (d.y / n) * s, (d.z / n) * s};
    return Quat{pcos(n), v.x, v.y, v.z};
}

// Euler angles -> quaternion for the known-answer tests only
// (common/basic_utils.h:62-69 eulerAnglesToQuaternion).  Each axis rotation
// is (cos(a/2), sin(a/2)*axis).  The reference's golden matrices and contact
// points (common/test_utils.cpp:57-91, collision_detection/test_comparison.cpp
// :8-62) are reproduced by R = Rz * Ry * Rx, so that composition is used.
inline Quat euler_to_quat(V3 ang) {
    const double hx = 0.5 * ang.x, hy = 0.5 * ang.y, hz = 0.5 * ang.z;
    const Quat qx{pcos(hx), psin(hx) * 1.0, psin(hx) * 0.0, psin(hx) * 0.0};
    const Quat qy{pcos(hy), psin(hy) * 0.0, psin(hy) * 1.0, psin(hy) * 0.0};
    const Quat qz{pcos(hz), psin(hz) * 0.0, psin(hz) * 0.0, psin(hz) * 1.0};
    return qmul(qmul(qz, qy), qx);
}

// Slerp as Eigen's QuaternionBase::slerp (shortest arc, linear fallback when
// the quaternions are within one ulp of parallel).
inline Quat qslerp(const Quat& a, double t, const Quat& b) {
    const double one = 1.0 - std::numeric_limits<double>::epsilon();
    const double d = ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w;
    const double absD = std::fabs(d);
    double scale0, scale1;
    if (absD >= one) {
        scale0 = 1.0 - t;
        scale1 = t;
    } else {
        const double theta = pacos(absD);
        const double sinTheta = psin(theta);
        scale0 = psin((1.0 - t) * theta) / sinTheta;
        scale1 = psin(t * theta) / sinTheta;
    }
    if (d < 0.0) scale1 = -scale1;
    return Quat{scale0 * a.w + scale1 * b.w, scale0 * a.x + scale1 * b.x, scale0 * a.y + scale1 * b.y,
                scale0 * a.z + scale1 * b.z};
}

// ------------------------------------------------------------- triangle ----
struct Tri {
    V3 A, B, C;
};
struct Edge {
    V3 A, B;
};

inline V3 tri_vertex(const Tri& T, int i) { return i == 0 ? T.A : (i == 1 ? T.B : T.C); }
inline Edge tri_edge(const Tri& T, int i) {  // AB, BC, CA
    return i == 0 ? Edge{T.A, T.B} : (i == 1 ? Edge{T.B, T.C} : Edge{T.C, T.A});
}

// common/triangle.h:43-45
inline V3 tri_normal(const Tri& T) { return normalized(cross(T.B - T.A, T.C - T.A)); }
// common/triangle.h:21-23
inline double tri_area(const Tri& T) { return 0.5 * norm(cross(T.A - T.C, T.B - T.C)); }

// common/triangle.h:90-103; dot products in double, the rest in float.
inline void tri_bary(const Tri& T, V3 P, double& u_out, double& v_out, double& w_out) {
    const V3 v0 = T.B - T.A, v1 = T.C - T.A, v2 = P - T.A;
    const float d00 = (float)dot(v0, v0);
    const float d01 = (float)dot(v0, v1);
    const float d11 = (float)dot(v1, v1);
    const float d20 = (float)dot(v2, v0);
    const float d21 = (float)dot(v2, v1);
    const float denom = d00 * d11 - d01 * d01;
    const float v = (d11 * d20 - d01 * d21) / denom;
    const float w = (d00 * d21 - d01 * d20) / denom;
    const float u = (1.0f - v) - w;
    u_out = u;
    v_out = v;
    w_out = w;
}

// common/triangle.h:105-131
inline V3 tri_intersect_segment(const Tri& T, const Edge& E, double& t, bool& t_inf, bool& isInt) {
    const V3 start = E.A;
    const V3 end = E.B;
    const V3 AP = T.A - start;
    const V3 n = tri_normal(T);
    const V3 D = end - start;
    const double p1 = dot(AP, n);
    const double p2 = dot(D, n);
    t_inf = false;
    if (std::fabs(p2) <= std::numeric_limits<double>::epsilon()) {
        t = 0.0;
        t_inf = true;
        isInt = false;
        return V3{0, 0, 0};
    }
    t = p1 / p2;
    if (0.0 < t && t < 1.0) {
        double u, v, w;
        tri_bary(T, start + D * t, u, v, w);
        isInt = 0.0 < u && u < 1.0 && 0.0 < v && v < 1.0 && u + v < 1.0;
        const double s = 1 - t;
        return V3{start.x * s + end.x * t, start.y * s + end.y * t, start.z * s + end.z * t};
    }
    isInt = false;
    return V3{0, 0, 0};
}

// common/triangle.h:133-141
inline V3 tri_project_to_plane(const Tri& T, V3 pt, bool& inTri) {
    const V3 AP = pt - T.A;
    const V3 n = tri_normal(T);
    const V3 onPlane = pt - dot(AP, n) * n;
    double u, v, w;
    tri_bary(T, onPlane, u, v, w);
    inTri = 0 < u && u < 1 && 0 < v && v < 1 && u + v < 1;
    return onPlane;
}

// common/triangle.h:472-487
inline Tri tri_xform(const Tri& T, const M4& M) { return Tri{xform(T.A, M), xform(T.B, M), xform(T.C, M)}; }

// common/edge.h:61-69
inline V3 edge_lerp(const Edge& E, double t) { return lerp(E.A, E.B, t); }
inline V3 edge_constrain(const Edge& E, V3 pos) {
    const V3 ba = E.B - E.A;
    const double t = dot(pos - E.A, ba) / dot(ba, ba);
    return edge_lerp(E, clamp01(t));
}
// common/edge.h:40-59  (this = S, other = E)
inline double edge_closest(const Edge& S, const Edge& E, V3& P_out, V3& Q_out) {
    const V3 segDC = E.B - E.A;
    const double lineDirSqrMag = dot(segDC, segDC);
    const V3 segAC = S.A - E.A;
    const V3 segBC = S.B - E.A;
    const V3 inPlaneA = S.A - (dot(segAC, segDC) / lineDirSqrMag) * segDC;
    const V3 inPlaneB = S.B - (dot(segBC, segDC) / lineDirSqrMag) * segDC;
    const V3 inPlaneBA = inPlaneB - inPlaneA;
    double t = dot(E.A - inPlaneA, inPlaneBA) / dot(inPlaneBA, inPlaneBA);
    t = (inPlaneA != inPlaneB) ? t : 0.0;
    const V3 segABtoLineCD = edge_lerp(S, clamp01(t));
    const V3 segCDtoSegAB = edge_constrain(E, segABtoLineCD);
    const V3 segABtoSegCD = edge_constrain(S, segCDtoSegAB);
    Q_out = segCDtoSegAB;
    P_out = segABtoSegCD;
    return norm(Q_out - P_out);
}
// common/edge.h:71-74
inline double edge_project(const Edge& E, V3 V) {
    const V3 AB = E.B - E.A;
    return dot(V - E.A, AB) / dot(AB, AB);
}

// Axis-aligned box, common/bbox.h and common/triangle.h:78-88.
struct BBox {
    V3 lo, hi;
};
inline BBox tri_bbox(const Tri& T) {
    return BBox{V3{dmin(dmin(T.A.x, T.B.x), T.C.x), dmin(dmin(T.A.y, T.B.y), T.C.y), dmin(dmin(T.A.z, T.B.z), T.C.z)},
                V3{dmax(dmax(T.A.x, T.B.x), T.C.x), dmax(dmax(T.A.y, T.B.y), T.C.y), dmax(dmax(T.A.z, T.B.z), T.C.z)}};
}
inline BBox bbox_union(const BBox& a, const BBox& b) {
    return BBox{V3{dmin(a.lo.x, b.lo.x), dmin(a.lo.y, b.lo.y), dmin(a.lo.z, b.lo.z)},
                V3{dmax(a.hi.x, b.hi.x), dmax(a.hi.y, b.hi.y), dmax(a.hi.z, b.hi.z)}};
}
inline BBox bbox_expand(const BBox& a, double e) {
    return BBox{V3{a.lo.x - e, a.lo.y - e, a.lo.z - e}, V3{a.hi.x + e, a.hi.y + e, a.hi.z + e}};
}
// common/bbox.h:7-20
inline bool overlapping_range(double al, double au, double bl, double bu) {
    if (bl < al) return bu > al;
    return bl < au;
}
inline bool bbox_overlap(const BBox& a, const BBox& b) {
    const bool x = overlapping_range(a.lo.x, a.hi.x, b.lo.x, b.hi.x);
    const bool y = overlapping_range(a.lo.y, a.hi.y, b.lo.y, b.hi.y);
    const bool z = overlapping_range(a.lo.z, a.hi.z, b.lo.z, b.hi.z);
    return x && y && z;
}

}  // namespace d2o
