// FP64 geometry for the contact hot path, usable from host and device.
//
// Restates the reference's geometry (common/triangle.h, common/edge.h,
// common/basic_utils.h, common/bbox.h) and CCD primitives
// (collision_detection/continuous_comparison.h, comparison_dist.h) with a
// fixed evaluation order:
//   dot(a,b)   = (a.x*b.x + a.y*b.y) + a.z*b.z
//   cross(a,b) = (a.y*b.z - a.z*b.y, a.z*b.x - a.x*b.z, a.x*b.y - a.y*b.x)
//   M*p        = ((m_r0*x + m_r1*y) + m_r2*z) + m_r3, then divided by row 3
// Matrices are 16 doubles, row major.  Rigid transforms have the bottom row
// (0,0,0,1): their homogeneous w is exactly 1 for finite points, so the
// division is skipped (same bits).  A matrix lerped between two rigid
// transforms, (1-t)*S + t*E, has bottom row (0,0,0,(1-t)+t); its entries are
// formed on the fly and w = (1-t)+t exactly as the full product would give.
#pragma once
#include <cfloat>

#include "d2g_math.cuh"

namespace d2g {

struct V3 {
    double x, y, z;
};

D2G_HD V3 mk(double x, double y, double z) {
    V3 r;
    r.x = x;
    r.y = y;
    r.z = z;
    return r;
}
D2G_HD V3 operator+(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
D2G_HD V3 operator-(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
D2G_HD V3 operator-(V3 a) { return mk(-a.x, -a.y, -a.z); }
D2G_HD V3 operator*(V3 a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
D2G_HD V3 operator*(double s, V3 a) { return mk(s * a.x, s * a.y, s * a.z); }
D2G_HD V3 operator/(V3 a, double s) { return mk(a.x / s, a.y / s, a.z / s); }
D2G_HD bool vne(V3 a, V3 b) { return a.x != b.x || a.y != b.y || a.z != b.z; }
D2G_HD double dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
D2G_HD V3 cross(V3 a, V3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
D2G_HD double norm(V3 a) { return sqrt(dot(a, a)); }
D2G_HD V3 normalized(V3 a) {
    const double z = dot(a, a);
    if (z > 0.0) {
        const double s = sqrt(z);
        return mk(a.x / s, a.y / s, a.z / s);
    }
    return a;
}
D2G_HD double dmin(double a, double b) { return (b < a) ? b : a; }
D2G_HD double dmax(double a, double b) { return (a < b) ? b : a; }
D2G_HD double dclamp(double v, double lo, double hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }
D2G_HD double clamp01(double t) {
    if (t < 0) return 0;
    if (t > 1) return 1;
    return t;
}
D2G_HD V3 lerp(V3 A, V3 B, double t) {
    const double u = 1 - t;
    return mk(A.x * u + B.x * t, A.y * u + B.y * t, A.z * u + B.z * t);
}
D2G_HD double lerp1(double A, double B, double t) { return A * (1 - t) + B * t; }

// ------------------------------------------------------------ 4x4 helpers --
D2G_HD V3 xform_rigid(V3 p, const double* M) {
    return mk(((M[0] * p.x + M[1] * p.y) + M[2] * p.z) + M[3] * 1.0,
              ((M[4] * p.x + M[5] * p.y) + M[6] * p.z) + M[7] * 1.0,
              ((M[8] * p.x + M[9] * p.y) + M[10] * p.z) + M[11] * 1.0);
}
D2G_HD V3 xform_general(V3 p, const double* M) {
    const double v0 = ((M[0] * p.x + M[1] * p.y) + M[2] * p.z) + M[3] * 1.0;
    const double v1 = ((M[4] * p.x + M[5] * p.y) + M[6] * p.z) + M[7] * 1.0;
    const double v2 = ((M[8] * p.x + M[9] * p.y) + M[10] * p.z) + M[11] * 1.0;
    const double v3 = ((M[12] * p.x + M[13] * p.y) + M[14] * p.z) + M[15] * 1.0;
    return mk(v0 / v3, v1 / v3, v2 / v3);
}
// p through ((1-t)*S + t*E) for rigid S, E.
D2G_HD V3 xform_lerp(V3 p, const double* S, const double* E, double t) {
    const double u = 1 - t;
    double v[3];
#pragma unroll
    for (int r = 0; r < 3; r++) {
        const double m0 = u * S[4 * r + 0] + t * E[4 * r + 0];
        const double m1 = u * S[4 * r + 1] + t * E[4 * r + 1];
        const double m2 = u * S[4 * r + 2] + t * E[4 * r + 2];
        const double m3 = u * S[4 * r + 3] + t * E[4 * r + 3];
        v[r] = ((m0 * p.x + m1 * p.y) + m2 * p.z) + m3 * 1.0;
    }
    const double w = u * 1.0 + t * 1.0;
    return mk(v[0] / w, v[1] / w, v[2] / w);
}

D2G_HD void mat_mul(const double* A, const double* B, double* R) {
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
            R[4 * i + j] = ((A[4 * i + 0] * B[0 + j] + A[4 * i + 1] * B[4 + j]) + A[4 * i + 2] * B[8 + j]) +
                           A[4 * i + 3] * B[12 + j];
}

// 4x4 inverse by complementary 2x2 minors (cofactor method).
D2G_HD void mat_inverse(const double* m, double* R) {
#define A_(i, j) m[4 * (i) + (j)]
    const double s0 = A_(0, 0) * A_(1, 1) - A_(1, 0) * A_(0, 1);
    const double s1 = A_(0, 0) * A_(1, 2) - A_(1, 0) * A_(0, 2);
    const double s2 = A_(0, 0) * A_(1, 3) - A_(1, 0) * A_(0, 3);
    const double s3 = A_(0, 1) * A_(1, 2) - A_(1, 1) * A_(0, 2);
    const double s4 = A_(0, 1) * A_(1, 3) - A_(1, 1) * A_(0, 3);
    const double s5 = A_(0, 2) * A_(1, 3) - A_(1, 2) * A_(0, 3);
    const double c5 = A_(2, 2) * A_(3, 3) - A_(3, 2) * A_(2, 3);
    const double c4 = A_(2, 1) * A_(3, 3) - A_(3, 1) * A_(2, 3);
    const double c3 = A_(2, 1) * A_(3, 2) - A_(3, 1) * A_(2, 2);
    const double c2 = A_(2, 0) * A_(3, 3) - A_(3, 0) * A_(2, 3);
    const double c1 = A_(2, 0) * A_(3, 2) - A_(3, 0) * A_(2, 2);
    const double c0 = A_(2, 0) * A_(3, 1) - A_(3, 0) * A_(2, 1);
    const double det = ((((s0 * c5 - s1 * c4) + s2 * c3) + s3 * c2) - s4 * c1) + s5 * c0;
    const double id = 1.0 / det;
    R[0] = ((A_(1, 1) * c5 - A_(1, 2) * c4) + A_(1, 3) * c3) * id;
    R[1] = ((-A_(0, 1) * c5 + A_(0, 2) * c4) - A_(0, 3) * c3) * id;
    R[2] = ((A_(3, 1) * s5 - A_(3, 2) * s4) + A_(3, 3) * s3) * id;
    R[3] = ((-A_(2, 1) * s5 + A_(2, 2) * s4) - A_(2, 3) * s3) * id;
    R[4] = ((-A_(1, 0) * c5 + A_(1, 2) * c2) - A_(1, 3) * c1) * id;
    R[5] = ((A_(0, 0) * c5 - A_(0, 2) * c2) + A_(0, 3) * c1) * id;
    R[6] = ((-A_(3, 0) * s5 + A_(3, 2) * s2) - A_(3, 3) * s1) * id;
    R[7] = ((A_(2, 0) * s5 - A_(2, 2) * s2) + A_(2, 3) * s1) * id;
    R[8] = ((A_(1, 0) * c4 - A_(1, 1) * c2) + A_(1, 3) * c0) * id;
    R[9] = ((-A_(0, 0) * c4 + A_(0, 1) * c2) - A_(0, 3) * c0) * id;
    R[10] = ((A_(3, 0) * s4 - A_(3, 1) * s2) + A_(3, 3) * s0) * id;
    R[11] = ((-A_(2, 0) * s4 + A_(2, 1) * s2) - A_(2, 3) * s0) * id;
    R[12] = ((-A_(1, 0) * c3 + A_(1, 1) * c1) - A_(1, 2) * c0) * id;
    R[13] = ((A_(0, 0) * c3 - A_(0, 1) * c1) + A_(0, 2) * c0) * id;
    R[14] = ((-A_(3, 0) * s3 + A_(3, 1) * s1) - A_(3, 2) * s0) * id;
    R[15] = ((A_(2, 0) * s3 - A_(2, 1) * s1) + A_(2, 2) * s0) * id;
#undef A_
}

// -------------------------------------------------------------- quaternions
struct Quat {
    double w, x, y, z;
};
D2G_HD Quat mkq(double w, double x, double y, double z) {
    Quat q;
    q.w = w;
    q.x = x;
    q.y = y;
    q.z = z;
    return q;
}
D2G_HD Quat qmul(const Quat& a, const Quat& b) {
    return mkq(((a.w * b.w - a.x * b.x) - a.y * b.y) - a.z * b.z, ((a.w * b.x + a.x * b.w) + a.y * b.z) - a.z * b.y,
               ((a.w * b.y + a.y * b.w) + a.z * b.x) - a.x * b.z, ((a.w * b.z + a.z * b.w) + a.x * b.y) - a.y * b.x);
}
// Rotation matrix of a quaternion (Eigen's formula), R[9] row major.
D2G_HD void qmat(const Quat& q, double* R) {
    const double tx = 2.0 * q.x, ty = 2.0 * q.y, tz = 2.0 * q.z;
    const double twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
    const double txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
    const double tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
    R[0] = 1.0 - (tyy + tzz);
    R[1] = txy - twz;
    R[2] = txz + twy;
    R[3] = txy + twz;
    R[4] = 1.0 - (txx + tzz);
    R[5] = tyz - twx;
    R[6] = txz - twy;
    R[7] = tyz + twx;
    R[8] = 1.0 - (txx + tyy);
}
// common/basic_utils.h:79-95 -> 16 doubles.
D2G_HD void transformation(const Quat& q, V3 t, double* T) {
    double R[9];
    qmat(q, R);
    T[0] = R[0];
    T[1] = R[1];
    T[2] = R[2];
    T[3] = t.x;
    T[4] = R[3];
    T[5] = R[4];
    T[6] = R[5];
    T[7] = t.y;
    T[8] = R[6];
    T[9] = R[7];
    T[10] = R[8];
    T[11] = t.z;
    T[12] = 0.0;
    T[13] = 0.0;
    T[14] = 0.0;
    T[15] = 1.0;
}
D2G_HD void m3_mul(const double* A, const double* B, double* R) {
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            R[3 * i + j] = (A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j]) + A[3 * i + 2] * B[6 + j];
}
D2G_HD void m3_mul_bt(const double* A, const double* B, double* R) {  // A * B^T
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            R[3 * i + j] = (A[3 * i] * B[3 * j] + A[3 * i + 1] * B[3 * j + 1]) + A[3 * i + 2] * B[3 * j + 2];
}
D2G_HD V3 m3_vec(const double* A, V3 v) {
    return mk((A[0] * v.x + A[1] * v.y) + A[2] * v.z, (A[3] * v.x + A[4] * v.y) + A[5] * v.z,
              (A[6] * v.x + A[7] * v.y) + A[8] * v.z);
}
// (v^T A) v
D2G_HD double quad_form(V3 v, const double* A) {
    const double r0 = (v.x * A[0] + v.y * A[3]) + v.z * A[6];
    const double r1 = (v.x * A[1] + v.y * A[4]) + v.z * A[7];
    const double r2 = (v.x * A[2] + v.y * A[5]) + v.z * A[8];
    return (r0 * v.x + r1 * v.y) + r2 * v.z;
}
// common/basic_utils.cpp:36-44
D2G_HD Quat qexp(V3 d) {
    if (norm(d) == 0.0) return mkq(1.0, 0.0, 0.0, 0.0);
    const double n = norm(d);
    const double s = m_sin(n);
    return mkq(m_cos(n), (d.x / n) * s, (d.y / n) * s, (d.z / n) * s);
}
// Rotated inverse inertia R * ii * R^T, with R from q.
D2G_HD void world_inv_inertia(const Quat& q, const double* ii, double* Iinv) {
    double R[9], T[9];
    qmat(q, R);
    m3_mul(R, ii, T);
    m3_mul_bt(T, R, Iinv);
}

// State record: time, qw qx qy qz, L xyz, x xyz, v xyz.
struct State {
    double time;
    Quat q;
    V3 L, x, v;
};
D2G_HD State load_state(const double* p) {
    State s;
    s.time = p[0];
    s.q = mkq(p[1], p[2], p[3], p[4]);
    s.L = mk(p[5], p[6], p[7]);
    s.x = mk(p[8], p[9], p[10]);
    s.v = mk(p[11], p[12], p[13]);
    return s;
}
D2G_HD void store_state(double* p, const State& s) {
    p[0] = s.time;
    p[1] = s.q.w;
    p[2] = s.q.x;
    p[3] = s.q.y;
    p[4] = s.q.z;
    p[5] = s.L.x;
    p[6] = s.L.y;
    p[7] = s.L.z;
    p[8] = s.x.x;
    p[9] = s.x.y;
    p[10] = s.x.z;
    p[11] = s.v.x;
    p[12] = s.v.y;
    p[13] = s.v.z;
}
// model/state.cpp:90-102 State::extrapolate
D2G_HD State extrapolate(const State& s, double t, const double* ii) {
    State r;
    r.time = s.time + t;
    r.v = s.v;
    r.x = s.x + t * s.v;
    double Iinv[9];
    world_inv_inertia(s.q, ii, Iinv);
    const V3 omega = m3_vec(Iinv, s.L);
    r.q = qmul(s.q, qexp((0.5 * omega) * t));
    r.L = s.L;
    return r;
}

// Slerp as Eigen's QuaternionBase::slerp: shortest arc, linear weights when
// the quaternions are within one ulp of parallel (used by State::interpolate).
D2G_HD Quat qslerp(const Quat& a, double t, const Quat& b) {
    const double one = 1.0 - DBL_EPSILON;
    const double d = ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w;
    const double absD = fabs(d);
    double s0, s1;
    if (absD >= one) {
        s0 = 1.0 - t;
        s1 = t;
    } else {
        const double theta = m_acos(absD);
        const double sinTheta = m_sin(theta);
        s0 = m_sin((1.0 - t) * theta) / sinTheta;
        s1 = m_sin(t * theta) / sinTheta;
    }
    if (d < 0.0) s1 = -s1;
    return mkq(s0 * a.w + s1 * b.w, s0 * a.x + s1 * b.x, s0 * a.y + s1 * b.y, s0 * a.z + s1 * b.z);
}
// model/state.cpp:55-70 State::interpolate (this = cur); false where the reference throws.
D2G_HD bool interpolate(const State& cur, const State& last, double time, State& out) {
    if (time > cur.time || time < last.time || last.time > cur.time) return false;
    if (last.time == cur.time) {
        out = cur;
        return true;
    }
    const double t = (time - last.time) / (cur.time - last.time);
    out.time = time;
    out.x = t * cur.x + (1 - t) * last.x;
    out.v = t * cur.v + (1 - t) * last.v;
    out.L = t * cur.L + (1 - t) * last.L;
    out.q = qslerp(last.q, t, cur.q);
    return true;
}
// collision_detection/continuous_comparison.h:12-36
D2G_HD double sphere_sphere_first_intersect(V3 a_pos, V3 a_vel, double a_rad, V3 b_pos, V3 b_vel, double b_rad) {
    const V3 ab = a_pos - b_pos;
    const V3 rel = a_vel - b_vel;
    const double r = a_rad + b_rad;
    const double c = dot(ab, ab) - r * r;
    if (c < 0.0) return 0.0;
    const double a = dot(rel, rel);
    const double b = dot(rel, ab);
    if (b >= 0.0) return -1.0;
    const double d = b * b - a * c;
    if (d < 0.0) return -1.0;
    return (-b - sqrt(d)) / a;
}

// ------------------------------------------------------------- triangles --
struct Tri {
    V3 A, B, C;
};
struct Edge {
    V3 A, B;
};
D2G_HD Tri load_tri(const double* p) {
    Tri t;
    t.A = mk(p[0], p[1], p[2]);
    t.B = mk(p[3], p[4], p[5]);
    t.C = mk(p[6], p[7], p[8]);
    return t;
}
D2G_HD V3 tvert(const Tri& T, int i) { return i == 0 ? T.A : (i == 1 ? T.B : T.C); }
D2G_HD Edge tedge(const Tri& T, int i) {
    Edge e;
    e.A = i == 0 ? T.A : (i == 1 ? T.B : T.C);
    e.B = i == 0 ? T.B : (i == 1 ? T.C : T.A);
    return e;
}
D2G_HD Tri tri_xform_rigid(const Tri& T, const double* M) {
    Tri r;
    r.A = xform_rigid(T.A, M);
    r.B = xform_rigid(T.B, M);
    r.C = xform_rigid(T.C, M);
    return r;
}
D2G_HD V3 tri_normal(const Tri& T) { return normalized(cross(T.B - T.A, T.C - T.A)); }

// common/triangle.h:90-103 (float arithmetic after double dot products).
D2G_HD void tri_bary(const Tri& T, V3 P, double& u_out, double& v_out) {
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
}
D2G_HD bool bary_inside(double u, double v) { return 0.0 < u && u < 1.0 && 0.0 < v && v < 1.0 && u + v < 1.0; }

// common/triangle.h:105-131
D2G_HD V3 tri_intersect_segment(const Tri& T, V3 start, V3 end, double& t, bool& t_inf, bool& isInt) {
    const V3 AP = T.A - start;
    const V3 n = tri_normal(T);
    const V3 D = end - start;
    const double p1 = dot(AP, n);
    const double p2 = dot(D, n);
    t_inf = false;
    if (fabs(p2) <= DBL_EPSILON) {
        t = 0.0;
        t_inf = true;
        isInt = false;
        return mk(0, 0, 0);
    }
    t = p1 / p2;
    if (0.0 < t && t < 1.0) {
        double u, v;
        tri_bary(T, start + D * t, u, v);
        isInt = bary_inside(u, v);
        const double s = 1 - t;
        return mk(start.x * s + end.x * t, start.y * s + end.y * t, start.z * s + end.z * t);
    }
    isInt = false;
    return mk(0, 0, 0);
}

// common/triangle.h:133-141
D2G_HD V3 tri_project_to_plane(const Tri& T, V3 pt, bool& inTri) {
    const V3 AP = pt - T.A;
    const V3 n = tri_normal(T);
    const V3 onPlane = pt - dot(AP, n) * n;
    double u, v;
    tri_bary(T, onPlane, u, v);
    inTri = bary_inside(u, v);
    return onPlane;
}

// common/edge.h:61-69
D2G_HD V3 edge_constrain(V3 A, V3 B, V3 pos) {
    const V3 ba = B - A;
    const double t = dot(pos - A, ba) / dot(ba, ba);
    return lerp(A, B, clamp01(t));
}
// common/edge.h:40-59, this = (SA,SB), other = (EA,EB)
D2G_HD double edge_closest(V3 SA, V3 SB, V3 EA, V3 EB, V3& P_out, V3& Q_out) {
    const V3 segDC = EB - EA;
    const double lineDirSqrMag = dot(segDC, segDC);
    const V3 segAC = SA - EA;
    const V3 segBC = SB - EA;
    const V3 inPlaneA = SA - (dot(segAC, segDC) / lineDirSqrMag) * segDC;
    const V3 inPlaneB = SB - (dot(segBC, segDC) / lineDirSqrMag) * segDC;
    const V3 inPlaneBA = inPlaneB - inPlaneA;
    double t = dot(EA - inPlaneA, inPlaneBA) / dot(inPlaneBA, inPlaneBA);
    t = vne(inPlaneA, inPlaneB) ? t : 0.0;
    const V3 segABtoLineCD = lerp(SA, SB, clamp01(t));
    const V3 segCDtoSegAB = edge_constrain(EA, EB, segABtoLineCD);
    const V3 segABtoSegCD = edge_constrain(SA, SB, segCDtoSegAB);
    Q_out = segCDtoSegAB;
    P_out = segABtoSegCD;
    return norm(Q_out - P_out);
}
D2G_HD double edge_project(V3 A, V3 B, V3 V) {
    const V3 AB = B - A;
    return dot(V - A, AB) / dot(AB, AB);
}

// ------------------------------------------------------ discrete tri-tri --
// collision_detection/comparison_dist.h:12-189
D2G_HD double tri_tri_dist(const Tri& a, const Tri& b, V3& P, V3& Q) {
    V3 Pc = mk(0, 0, 0), Qc = mk(0, 0, 0), Pt, Qt;
    double dc = 1.0 / 0.0;
    bool in;
    for (int i = 0; i < 3; i++) {
        const V3 bv = tvert(b, i);
        Pt = tri_project_to_plane(a, bv, in);
        if (in) {
            const double d = norm(Pt - bv);
            if (d < dc) {
                Pc = Pt;
                Qc = bv;
                dc = d;
            }
        }
    }
    for (int i = 0; i < 3; i++) {
        const V3 av = tvert(a, i);
        Qt = tri_project_to_plane(b, av, in);
        if (in) {
            const double d = norm(av - Qt);
            if (d < dc) {
                Pc = av;
                Qc = Qt;
                dc = d;
            }
        }
    }
    for (int i = 0; i < 3; i++) {
        const Edge ea = tedge(a, i);
        for (int j = 0; j < 3; j++) {
            const Edge eb = tedge(b, j);
            const double d = edge_closest(ea.A, ea.B, eb.A, eb.B, Pt, Qt);
            if (d < dc) {
                Pc = Pt;
                Qc = Qt;
                dc = d;
            }
        }
    }
    double t;
    bool t_inf, isInt;
    for (int j = 0; j < 3; j++) {
        const Edge e = tedge(b, j);
        tri_intersect_segment(a, e.A, e.B, t, t_inf, isInt);
        if (isInt) {
            Pc = lerp(e.A, e.B, t);
            Qc = Pc;
        }
    }
    for (int j = 0; j < 3; j++) {
        const Edge e = tedge(a, j);
        tri_intersect_segment(b, e.A, e.B, t, t_inf, isInt);
        if (isInt) {
            Pc = lerp(e.A, e.B, t);
            Qc = Pc;
        }
    }
    P = Pc;
    Q = Qc;
    return norm(Pc - Qc);
}

// ------------------------------------------------------------------ CCD ----
struct Ccd {
    double dist;
    V3 P, Q;
    double toc;
};
D2G_HD void ccd_take(Ccd& best, const Ccd& c) {
    if (c.dist < best.dist || (c.dist == best.dist && c.toc < best.toc)) best = c;
}

// collision_detection/continuous_comparison.h:41-98 pointTriCCDLinear.
// Cs / Ce = inverse(tri_T_start) * pt_T_start (general 4x4), tS / tE rigid.
D2G_HD Ccd point_tri_ccd(V3 pt, const double* Cs, const double* Ce, const Tri& tri, const double* tS,
                         const double* tE) {
    Ccd r;
    r.P = mk(0, 0, 0);
    r.Q = mk(0, 0, 0);
    const V3 ps = xform_general(pt, Cs);
    const V3 pe = xform_general(pt, Ce);
    r.toc = 1.0;
    bool isInt, t_inf;
    double t;
    const V3 inter = tri_intersect_segment(tri, ps, pe, t, t_inf, isInt);
    if (0 < t && t < 1 && isInt) {
        r.P = xform_lerp(inter, tS, tE, t);
        r.Q = r.P;
        r.toc = t;
        r.dist = 0;
        return r;
    } else if (t_inf) {
        bool above;
        V3 closest = lerp(ps, pe, 0.0);
        V3 onPlane = tri_project_to_plane(tri, closest, above);
        if (above) {
            r.P = xform_rigid(closest, tS);
            r.Q = xform_rigid(onPlane, tS);
            r.toc = 0.0;
            r.dist = norm(r.P - r.Q);
            return r;
        }
        closest = lerp(ps, pe, 1.0);
        onPlane = tri_project_to_plane(tri, closest, above);
        if (above) {
            r.P = xform_rigid(closest, tE);
            r.Q = xform_rigid(onPlane, tE);
            r.toc = 1.0;
            r.dist = norm(r.P - r.Q);
            return r;
        }
    } else {
        t = clamp01(t);
        const V3 closest = lerp(ps, pe, t);
        bool above;
        const V3 onPlane = tri_project_to_plane(tri, closest, above);
        if (above) {
            r.P = xform_lerp(closest, tS, tE, t);
            r.Q = xform_lerp(onPlane, tS, tE, t);
            r.toc = t;
            r.dist = norm(r.P - r.Q);
            return r;
        }
    }
    r.dist = 1.0 / 0.0;
    return r;
}

// Newton quantities of edgeEdgeCCD (continuous_comparison.h:630-631), the
// generated expressions restated with shared sub-expressions f, g, h.
D2G_HD void ee_newton_terms(const Edge& aS, const Edge& aE, const Edge& bS, const Edge& bE, double pa, double pb,
                            double t, double& t_diff, double& t_diff2) {
    const double omt = 1 - t, ompa = 1 - pa, ompb = 1 - pb, pbm1 = pb - 1;
    double gf2[3], gh[3], ff[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const double aSA = k == 0 ? aS.A.x : (k == 1 ? aS.A.y : aS.A.z);
        const double aSB = k == 0 ? aS.B.x : (k == 1 ? aS.B.y : aS.B.z);
        const double aEA = k == 0 ? aE.A.x : (k == 1 ? aE.A.y : aE.A.z);
        const double aEB = k == 0 ? aE.B.x : (k == 1 ? aE.B.y : aE.B.z);
        const double bSA = k == 0 ? bS.A.x : (k == 1 ? bS.A.y : bS.A.z);
        const double bSB = k == 0 ? bS.B.x : (k == 1 ? bS.B.y : bS.B.z);
        const double bEA = k == 0 ? bE.A.x : (k == 1 ? bE.A.y : bE.A.z);
        const double bEB = k == 0 ? bE.B.x : (k == 1 ? bE.B.y : bE.B.z);
        const double f = ((pa * (aEB + aSB * omt) - pb * (bEB + bSB * omt)) + ompa * (aEA * t + aSA * omt)) -
                         ompb * (bEA * t + bSA * omt);
        const double g = ((-2 * aSB * pa + 2 * bSB * pb) + 2 * ompa * (aEA - aSA)) + 2 * (bEA - bSA) * pbm1;
        const double h = ((-aSB * pa / 2 + bSB * pb / 2) + ompa * (aEA - aSA) / 2) + (bEA - bSA) * pbm1 / 2;
        gf2[k] = g * f / 2;
        gh[k] = g * h;
        ff[k] = f * f;
    }
    const double gf = (gf2[0] + gf2[1]) + gf2[2];
    const double S = (ff[0] + ff[1]) + ff[2];
    const double sS = sqrt(S);
    const double GH = (gh[0] + gh[1]) + gh[2];
    t_diff = gf / sS;
    t_diff2 = GH / sS + ((-gf) * gf) / m_pow15(S);
}

// The pieces of collision_detection/continuous_comparison.h:565-673
// edgeEdgeCCD, shared by edge_edge_ccd below and the phased kernels.
// Coplanarity triple product of two edges (:570-573).
D2G_HD double ee_coplanarity(const Edge& a, const Edge& b) {
    const V3 n = cross(a.B - a.A, b.A - a.A);
    return dot(b.B - a.A, n);
}

// The bisection on a sign change of the triple product (:574-607): 20 halvings,
// then the closest points at the middle time.  Returns the distance.
D2G_HD double ee_bisect(const Edge& aS, const Edge& aE, const Edge& bS, const Edge& bE, double dot_start, Ccd& r) {
    double t_lower = 0.0, t_upper = 1.0;
    for (int iter = 0; iter < 20; iter++) {
        const double t_mid = (t_lower + t_upper) / 2.0;
        const V3 atA = lerp(aS.A, aE.A, t_mid), atB = lerp(aS.B, aE.B, t_mid);
        const V3 btA = lerp(bS.A, bE.A, t_mid), btB = lerp(bS.B, bE.B, t_mid);
        const V3 n_mid = cross(atB - atA, btA - atA);
        const double dot_mid = dot(btB - atA, n_mid);
        if (fabs(dot_mid) < 1e-8) {
            t_lower = t_mid;
            t_upper = t_mid;
            break;
        } else if (dot_start * dot_mid < 0.0) {
            t_upper = t_mid;
        } else {
            t_lower = t_mid;
        }
    }
    const double t_mid = (t_lower + t_upper) / 2.0;
    const V3 atA = lerp(aS.A, aE.A, t_mid), atB = lerp(aS.B, aE.B, t_mid);
    const V3 btA = lerp(bS.A, bE.A, t_mid), btB = lerp(bS.B, bE.B, t_mid);
    const double d = edge_closest(atA, atB, btA, btB, r.P, r.Q);
    r.toc = t_mid;
    return d;
}

// One Newton iteration from time t (:609-637): the closest points at t update
// the best (min_dist, r), then t moves by -f'/f'' and is clamped to [0, 1].
// Returns true when the iteration loop ends here: each iteration is a
// function of t alone, so once t repeats (or is NaN) the remaining iterations
// recompute the same distance, which cannot lower min_dist, and stopping
// gives the same result.
D2G_HD bool ee_newton_iter(const Edge& aS, const Edge& aE, const Edge& bS, const Edge& bE, double& t,
                           double& min_dist, Ccd& r, double* dist_out = nullptr) {
    const V3 atA = lerp(aS.A, aE.A, t), atB = lerp(aS.B, aE.B, t);
    const V3 btA = lerp(bS.A, bE.A, t), btB = lerp(bS.B, bE.B, t);
    V3 P, Q;
    const double dist = edge_closest(atA, atB, btA, btB, P, Q);
    if (dist_out) *dist_out = dist;
    if (dist < min_dist) {
        min_dist = dist;
        r.P = P;
        r.Q = Q;
        r.toc = t;
    }
    const double pa = edge_project(atA, atB, P);
    const double pb = edge_project(btA, btB, Q);
    double td, td2;
    ee_newton_terms(aS, aE, bS, bE, pa, pb, t, td, td2);
    const double t_prev = t;
    t = t - td / td2;
    t = clamp01(t);
    return t == t_prev || t != t;
}

constexpr int kEeNewtonIters = 10;

// collision_detection/continuous_comparison.h:565-673 edgeEdgeCCD.
D2G_HD Ccd edge_edge_ccd(const Edge& aS, const Edge& aE, const Edge& bS, const Edge& bE) {
    Ccd r;
    r.P = mk(0, 0, 0);
    r.Q = mk(0, 0, 0);
    r.toc = 0.0;
    double min_dist = DBL_MAX;
    const double dot_start = ee_coplanarity(aS, bS);
    const double dot_end = ee_coplanarity(aE, bE);
    if (dot_start * dot_end < 0.0) min_dist = ee_bisect(aS, aE, bS, bE, dot_start, r);
    if (min_dist > 1e-8) {
        double t = 0.0;
        for (int iter = 0; iter < kEeNewtonIters; iter++)
            if (ee_newton_iter(aS, aE, bS, bE, t, min_dist, r)) break;
    }
    r.dist = min_dist;
    return r;
}

// Pose matrices of one body pair for CCD: rigid start/end transforms of a
// and b, and the products inverse(T_b) * T_a (a's points into b's frame) and
// inverse(T_a) * T_b, at start and end.  Layout: 8 matrices x 16 doubles.
enum { PM_AS = 0, PM_AE = 16, PM_BS = 32, PM_BE = 48, PM_ABS = 64, PM_ABE = 80, PM_BAS = 96, PM_BAE = 112,
       PM_SIZE = 128 };

D2G_HD void pair_mats(const State& aS, const State& aE, const State& bS, const State& bE, double* M) {
    transformation(aS.q, aS.x, M + PM_AS);
    transformation(aE.q, aE.x, M + PM_AE);
    transformation(bS.q, bS.x, M + PM_BS);
    transformation(bE.q, bE.x, M + PM_BE);
    double inv[16];
    mat_inverse(M + PM_BS, inv);
    mat_mul(inv, M + PM_AS, M + PM_ABS);
    mat_inverse(M + PM_BE, inv);
    mat_mul(inv, M + PM_AE, M + PM_ABE);
    mat_inverse(M + PM_AS, inv);
    mat_mul(inv, M + PM_BS, M + PM_BAS);
    mat_inverse(M + PM_AE, inv);
    mat_mul(inv, M + PM_BE, M + PM_BAE);
}

// One of the 15 sub-tests of triTriCCDLinear (continuous_comparison.h:692-777),
// in the reference's order s = 5*i + r: r=0 point a_i vs tri b, r=1 point b_i
// vs tri a, r=2..4 edge a_i vs edge b_(r-2).  a_s/a_e/b_s/b_e are the
// triangles transformed to start / end.
D2G_HD Ccd tri_tri_subtest(int s, const Tri& a, const Tri& b, const Tri& a_s, const Tri& a_e, const Tri& b_s,
                           const Tri& b_e, const double* M) {
    const int i = s / 5, r = s % 5;
    if (r == 0) return point_tri_ccd(tvert(a, i), M + PM_ABS, M + PM_ABE, b, M + PM_BS, M + PM_BE);
    if (r == 1) return point_tri_ccd(tvert(b, i), M + PM_BAS, M + PM_BAE, a, M + PM_AS, M + PM_AE);
    const int j = r - 2;
    return edge_edge_ccd(tedge(a_s, i), tedge(a_e, i), tedge(b_s, j), tedge(b_e, j));
}

D2G_HD Ccd tri_tri_ccd(const Tri& a, const Tri& b, const double* M) {
    Ccd best;
    best.dist = 1.0 / 0.0;
    best.toc = 1.0;
    best.P = mk(0, 0, 0);
    best.Q = mk(0, 0, 0);
    const Tri a_s = tri_xform_rigid(a, M + PM_AS), a_e = tri_xform_rigid(a, M + PM_AE);
    const Tri b_s = tri_xform_rigid(b, M + PM_BS), b_e = tri_xform_rigid(b, M + PM_BE);
    for (int s = 0; s < 15; s++) ccd_take(best, tri_tri_subtest(s, a, b, a_s, a_e, b_s, b_e, M));
    return best;
}

// Swept box of a triangle between two rigid poses, expanded by eps
// (continuous_comparison.h:805,810; common/bbox.h).
struct Box {
    double lo[3], hi[3];
};
D2G_HD Box swept_box(const Tri& t, const double* S, const double* E, double eps) {
    const Tri s = tri_xform_rigid(t, S), e = tri_xform_rigid(t, E);
    Box b;
    const double sx[3] = {s.A.x, s.B.x, s.C.x}, sy[3] = {s.A.y, s.B.y, s.C.y}, sz[3] = {s.A.z, s.B.z, s.C.z};
    const double ex[3] = {e.A.x, e.B.x, e.C.x}, ey[3] = {e.A.y, e.B.y, e.C.y}, ez[3] = {e.A.z, e.B.z, e.C.z};
    const double slo[3] = {dmin(dmin(sx[0], sx[1]), sx[2]), dmin(dmin(sy[0], sy[1]), sy[2]),
                           dmin(dmin(sz[0], sz[1]), sz[2])};
    const double shi[3] = {dmax(dmax(sx[0], sx[1]), sx[2]), dmax(dmax(sy[0], sy[1]), sy[2]),
                           dmax(dmax(sz[0], sz[1]), sz[2])};
    const double elo[3] = {dmin(dmin(ex[0], ex[1]), ex[2]), dmin(dmin(ey[0], ey[1]), ey[2]),
                           dmin(dmin(ez[0], ez[1]), ez[2])};
    const double ehi[3] = {dmax(dmax(ex[0], ex[1]), ex[2]), dmax(dmax(ey[0], ey[1]), ey[2]),
                           dmax(dmax(ez[0], ez[1]), ez[2])};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        b.lo[k] = dmin(slo[k], elo[k]) - eps;
        b.hi[k] = dmax(shi[k], ehi[k]) + eps;
    }
    return b;
}
D2G_HD bool range_overlap(double al, double au, double bl, double bu) {
    if (bl < al) return bu > al;
    return bl < au;
}
D2G_HD bool box_overlap(const Box& a, const Box& b) {
    const bool x = range_overlap(a.lo[0], a.hi[0], b.lo[0], b.hi[0]);
    const bool y = range_overlap(a.lo[1], a.hi[1], b.lo[1], b.hi[1]);
    const bool z = range_overlap(a.lo[2], a.hi[2], b.lo[2], b.hi[2]);
    return x && y && z;
}

}  // namespace d2g
