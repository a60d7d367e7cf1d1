// Oracle (test infrastructure only): body state, surrogate-tree storage,
// discrete narrow phase and continuous collision detection, restated from
// the reference (file:line cited per function).  Plain C++, FP64.
#pragma once
#include <algorithm>
#include <cstdint>
#include <vector>

#include "d2o_geom.hpp"

namespace d2o {

// ------------------------------------------------------------ state --------
// model/state.h:6-36 — time, rotation, angular momentum, translation, velocity.
struct State {
    double time;
    Quat q;
    V3 L, x, v;
};

inline State state_identity() { return State{0.0, Quat{1, 0, 0, 0}, V3{0, 0, 0}, V3{0, 0, 0}, V3{0, 0, 0}}; }
inline M4 state_transform(const State& s) { return transformation(s.q, s.x); }

// model/state.cpp:90-102 State::extrapolate
inline State state_extrapolate(const State& s, double t, const M3& ii) {
    State r;
    r.time = s.time + t;
    r.v = s.v;
    r.x = s.x + t * s.v;
    const M3 R = qmat(s.q);
    const M3 Iinv = m3_mul(m3_mul(R, ii), m3_transpose(R));
    const V3 omega = m3_vec(Iinv, s.L);
    const Quat d = qexp((0.5 * omega) * t);
    r.q = qmul(s.q, d);
    r.L = s.L;
    return r;
}

// model/state.cpp:55-70 State::interpolate (this = cur, argument = last)
inline bool state_interpolate(const State& cur, const State& last, double time, State& out) {
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

// model/state.cpp:81-84 State::pointVelocity(pt, inv_inertia) — body-frame
// inverse inertia applied without rotation (as the reference does).
inline V3 state_point_velocity(const State& s, V3 pt, const M3& ii) {
    const V3 w = m3_vec(ii, s.L);
    return s.v + cross(w, pt - s.x);
}

// model/particle.cpp:72-78 Particle::futurePointVelocity (world-frame inertia).
inline V3 future_point_velocity(const State& f, const M3& ii, V3 pt) {
    const M3 R = qmat(f.q);
    const M3 Iinv = m3_mul(m3_mul(R, ii), m3_transpose(R));
    const V3 omega = m3_vec(Iinv, f.L);
    return f.v + cross(omega, pt - f.x);
}

// model/state.cpp:120-122
inline bool state_stationary(const State& s) { return norm(s.v) < 1e-4 && norm(s.L) < 1e-4; }

// --------------------------------------------------------- trees -----------
// model/surrogate_components.h:11-20 Node (node id == bucket id: nodes and
// buckets are appended together in surrogate_tree.cpp:57-69,86-100) and
// :66-88 BucketSoup (<= 8 triangles with eps / inner_eps).
struct Node {
    int child_first, num_children, is_inner, depth;
};

struct TreeSet {
    int n_meshes = 0;
    const int32_t* mesh_node_off = nullptr;  // [n_meshes+1]
    const int32_t* nodes = nullptr;          // [N][4] child_first, num_children, is_inner, depth
    const int32_t* ntris = nullptr;          // [N]
    const double* tris = nullptr;            // [N][8][9]  A.xyz B.xyz C.xyz
    const double* eps = nullptr;             // [N][8]
    const double* inner_eps = nullptr;       // [N][8]

    int root(int mesh) const { return mesh_node_off[mesh]; }
    Node node(int g) const {
        const int32_t* n = nodes + 4 * (size_t)g;
        return Node{n[0], n[1], n[2], n[3]};
    }
    int nt(int g) const { return ntris[g]; }
    Tri tri(int g, int i) const {
        const double* p = tris + (size_t)g * 72 + i * 9;
        return Tri{V3{p[0], p[1], p[2]}, V3{p[3], p[4], p[5]}, V3{p[6], p[7], p[8]}};
    }
    double e(int g, int i) const { return eps[(size_t)g * 8 + i]; }
    double ie(int g, int i) const { return inner_eps[(size_t)g * 8 + i]; }
};
// Node child indices are stored GLOBAL (already offset by the mesh's first node).

// ---------------------------------------------------------- bodies ---------
// model/particle.h:9-64 (only the fields the hot path reads).
struct Body {
    int mesh = 0;
    bool is_static = false;
    double geo_eps = 0, mu = 0, mass = 1;
    M3 ii{};  // inverse body inertia
    State last = state_identity(), cur = state_identity(), fut = state_identity();
    double last_dt = 1.0;
    int sleep_not_moved_steps = 0;
    bool sleeping = false;
    double bounding_radius = 0;
};

// --------------------------------------------------------- contacts --------
// collision_detection/contact.h:9-28 Contact and :73-83 ContinuousContact.
struct Contact {
    V3 A, B;
    double eps_a, eps_b, eps_inner_a, eps_inner_b;
    double toc;  // continuous contacts only
    int pa, pb;
};

// collision_detection/contact.h:32-40 compareContacts
inline bool compare_contacts(const Contact& a, const Contact& b) {
    const double a_eps = a.eps_a + a.eps_b;
    const double b_eps = b.eps_a + b.eps_b;
    if (a_eps == b_eps) return norm(a.A - a.B) < norm(b.A - b.B);
    return a_eps < b_eps;
}

// collision_detection/contact.h:44-69 filterContacts.  The reference uses the
// unstable std::sort; the declared order here is std::stable_sort (ties keep
// input order), matched by the GPU.  `unstable` selects std::sort instead.
inline std::vector<Contact> filter_contacts(std::vector<Contact> unf, double margin, bool unstable = false) {
    if (unstable)
        std::sort(unf.begin(), unf.end(), compare_contacts);
    else
        std::stable_sort(unf.begin(), unf.end(), compare_contacts);
    std::vector<Contact> out;
    for (const Contact& ct : unf) {
        bool new_point = true;
        for (const Contact& h : out) {
            const V3 ht_mid = (ct.A + ct.B) / 2;
            const V3 h_mid = (h.A + h.B) / 2;
            const double dist = norm(ht_mid - h_mid);
            const double search = (ct.eps_a + ct.eps_b) + margin;
            if (dist < search) {
                new_point = false;
                break;
            }
        }
        if (new_point) out.push_back(ct);
    }
    return out;
}

// collision_detection/contact.h:86-123 filterContinuousContacts (sort key eps only).
inline std::vector<Contact> filter_continuous_contacts(std::vector<Contact> unf, double margin) {
    std::stable_sort(unf.begin(), unf.end(), [](const Contact& a, const Contact& b) {
        return (a.eps_a + a.eps_b) < (b.eps_a + b.eps_b);
    });
    std::vector<Contact> out;
    for (const Contact& ct : unf) {
        bool new_point = true;
        for (const Contact& h : out) {
            const double dist = norm((ct.A + ct.B) / 2 - (h.A + h.B) / 2);
            if (dist < (ct.eps_a + ct.eps_b) + margin) {
                new_point = false;
                break;
            }
        }
        if (new_point) out.push_back(ct);
    }
    return out;
}

// ------------------------------------------------ discrete tri-tri ---------
// collision_detection/comparison_dist.h:12-189 _comparisonDist
struct DistResult {
    double dist;
    V3 P, Q;
};
inline DistResult tri_tri_dist(const Tri& a, const Tri& b) {
    V3 Pc{0, 0, 0}, Qc{0, 0, 0}, Pt, Qt;
    double dc = std::numeric_limits<double>::infinity();
    bool in;
    for (int i = 0; i < 3; i++) {  // b's vertices onto a's plane
        const V3 bv = tri_vertex(b, i);
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
    for (int i = 0; i < 3; i++) {  // a's vertices onto b's plane
        const V3 av = tri_vertex(a, i);
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
    for (int i = 0; i < 3; i++) {  // 9 edge pairs, a-edge outer
        for (int j = 0; j < 3; j++) {
            const double d = edge_closest(tri_edge(a, i), tri_edge(b, j), Pt, Qt);
            if (d < dc) {
                Pc = Pt;
                Qc = Qt;
                dc = d;
            }
        }
    }
    double t;
    bool t_inf, isInt;
    for (int j = 0; j < 3; j++) {  // b's edges through a
        const Edge e = tri_edge(b, j);
        tri_intersect_segment(a, e, t, t_inf, isInt);
        if (isInt) {
            Pc = edge_lerp(e, t);
            Qc = edge_lerp(e, t);
            dc = 0.0;
        }
    }
    for (int j = 0; j < 3; j++) {  // a's edges through b
        const Edge e = tri_edge(a, j);
        tri_intersect_segment(b, e, t, t_inf, isInt);
        if (isInt) {
            Pc = edge_lerp(e, t);
            Qc = edge_lerp(e, t);
            dc = 0.0;
        }
    }
    (void)dc;
    return DistResult{norm(Pc - Qc), Pc, Qc};
}

// ------------------------------------------------------------ CCD ----------
// collision_detection/continuous_comparison.h:12-36
inline double sphere_sphere_first_intersect(V3 a_pos, V3 a_vel, double a_rad, V3 b_pos, V3 b_vel, double b_rad) {
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
    return (-b - std::sqrt(d)) / a;
}

struct CcdResult {
    double dist;
    V3 P, Q;
    double toc;
};

// collision_detection/continuous_comparison.h:41-98 pointTriCCDLinear.
// `C_start` = inverse(tri_T_start) * pt_T_start and `C_end` likewise: the
// reference computes (inverse * T) * p; the product is formed first here too.
inline CcdResult point_tri_ccd_c(V3 pt, const M4& C_start, const M4& C_end, const Tri& tri, const M4& tri_T_start,
                                 const M4& tri_T_end) {
    CcdResult r;
    r.P = V3{0, 0, 0};
    r.Q = V3{0, 0, 0};
    const V3 pt_start = xform(pt, C_start);
    const V3 pt_end = xform(pt, C_end);
    const Edge e{pt_start, pt_end};
    r.toc = 1.0;
    bool isInt, t_inf;
    double t;
    const V3 inter = tri_intersect_segment(tri, e, t, t_inf, isInt);
    if (0 < t && t < 1 && isInt) {
        const M4 tT = mat_lerp(tri_T_start, tri_T_end, t);
        r.P = xform(inter, tT);
        r.Q = xform(inter, tT);
        r.toc = t;
        r.dist = 0;
        return r;
    } else if (t_inf) {
        t = 0;
        V3 closest = edge_lerp(e, t);
        bool above;
        V3 onPlane = tri_project_to_plane(tri, closest, above);
        if (above) {
            r.P = xform(closest, tri_T_start);
            r.Q = xform(onPlane, tri_T_start);
            r.toc = t;
            r.dist = norm(r.P - r.Q);
            return r;
        }
        t = 1;
        closest = edge_lerp(e, t);
        onPlane = tri_project_to_plane(tri, closest, above);
        if (above) {
            r.P = xform(closest, tri_T_end);
            r.Q = xform(onPlane, tri_T_end);
            r.toc = t;
            r.dist = norm(r.P - r.Q);
            return r;
        }
    } else {
        t = clamp01(t);
        const M4 tT = mat_lerp(tri_T_start, tri_T_end, t);
        const V3 closest = edge_lerp(e, t);
        bool above;
        const V3 onPlane = tri_project_to_plane(tri, closest, above);
        if (above) {
            r.P = xform(closest, tT);
            r.Q = xform(onPlane, tT);
            r.toc = t;
            r.dist = norm(r.P - r.Q);
            return r;
        }
    }
    r.dist = std::numeric_limits<double>::infinity();
    return r;
}

inline CcdResult point_tri_ccd(V3 pt, const M4& pt_T_start, const M4& pt_T_end, const Tri& tri, const M4& tri_T_start,
                               const M4& tri_T_end) {
    const M4 Cs = mat_mul(mat_inverse(tri_T_start), pt_T_start);
    const M4 Ce = mat_mul(mat_inverse(tri_T_end), pt_T_end);
    return point_tri_ccd_c(pt, Cs, Ce, tri, tri_T_start, tri_T_end);
}

// One Newton step quantity of edgeEdgeCCD (continuous_comparison.h:630-631),
// the sympy-generated expressions restated with shared sub-expressions:
//   f_k = pa*(aEB + aSB*(1-t)) - pb*(bEB + bSB*(1-t))
//         + (1-pa)*(aEA*t + aSA*(1-t)) - (1-pb)*(bEA*t + bSA*(1-t))
//   g_k = -2*aSB*pa + 2*bSB*pb + 2*(1-pa)*(aEA-aSA) + 2*(bEA-bSA)*(pb-1)
//   h_k = g_k / 4 written term-wise as in the reference
//   t_diff  = (sum g_k*f_k/2) / sqrt(S),      S = sum f_k^2
//   t_diff2 = (sum g_k*h_k) / sqrt(S) - (sum g_k*f_k/2)^2 / S^(3/2)
inline void ee_newton_terms(const Edge& aS, const Edge& aE, const Edge& bS, const Edge& bE, double pa, double pb,
                            double t, double& t_diff, double& t_diff2) {
    const double aSA[3] = {aS.A.x, aS.A.y, aS.A.z}, aSB[3] = {aS.B.x, aS.B.y, aS.B.z};
    const double aEA[3] = {aE.A.x, aE.A.y, aE.A.z}, aEB[3] = {aE.B.x, aE.B.y, aE.B.z};
    const double bSA[3] = {bS.A.x, bS.A.y, bS.A.z}, bSB[3] = {bS.B.x, bS.B.y, bS.B.z};
    const double bEA[3] = {bE.A.x, bE.A.y, bE.A.z}, bEB[3] = {bE.B.x, bE.B.y, bE.B.z};
    double gf2[3], gh[3], ff[3];
    const double omt = 1 - t, ompa = 1 - pa, ompb = 1 - pb, pbm1 = pb - 1;
    for (int k = 0; k < 3; k++) {
        const double f = ((pa * (aEB[k] + aSB[k] * omt) - pb * (bEB[k] + bSB[k] * omt)) +
                          ompa * (aEA[k] * t + aSA[k] * omt)) -
                         ompb * (bEA[k] * t + bSA[k] * omt);
        const double g = ((-2 * aSB[k] * pa + 2 * bSB[k] * pb) + 2 * ompa * (aEA[k] - aSA[k])) +
                         2 * (bEA[k] - bSA[k]) * pbm1;
        const double h = ((-aSB[k] * pa / 2 + bSB[k] * pb / 2) + ompa * (aEA[k] - aSA[k]) / 2) +
                         (bEA[k] - bSA[k]) * pbm1 / 2;
        gf2[k] = g * f / 2;
        gh[k] = g * h;
        ff[k] = f * f;
    }
    const double gf = (gf2[0] + gf2[1]) + gf2[2];
    const double S = (ff[0] + ff[1]) + ff[2];
    const double sS = std::sqrt(S);
    const double GH = (gh[0] + gh[1]) + gh[2];
    t_diff = gf / sS;
    t_diff2 = GH / sS + ((-gf) * gf) / pow15(S);
}

// collision_detection/continuous_comparison.h:565-673 edgeEdgeCCD.
// When every candidate distance is NaN the reference leaves P/Q/toc unset;
// here they stay (0,0,0)/(0,0,0)/0.
inline CcdResult edge_edge_ccd(const Edge& aS, const Edge& aE, const Edge& bS, const Edge& bE) {
    CcdResult r;
    r.P = V3{0, 0, 0};
    r.Q = V3{0, 0, 0};
    r.toc = 0.0;
    double min_dist = std::numeric_limits<double>::max();
    const V3 n_start = cross(aS.B - aS.A, bS.A - aS.A);
    const double dot_start = dot(bS.B - aS.A, n_start);
    const V3 n_end = cross(aE.B - aE.A, bE.A - aE.A);
    const double dot_end = dot(bE.B - aE.A, n_end);
    if (dot_start * dot_end < 0.0) {
        double t_lower = 0.0, t_upper = 1.0;
        for (int iter = 0; iter < 20; iter++) {
            const double t_mid = (t_lower + t_upper) / 2.0;
            const Edge at{lerp(aS.A, aE.A, t_mid), lerp(aS.B, aE.B, t_mid)};
            const Edge bt{lerp(bS.A, bE.A, t_mid), lerp(bS.B, bE.B, t_mid)};
            const V3 n_mid = cross(at.B - at.A, bt.A - at.A);
            const double dot_mid = dot(bt.B - at.A, n_mid);
            if (std::fabs(dot_mid) < 1e-8) {
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
        const Edge at{lerp(aS.A, aE.A, t_mid), lerp(aS.B, aE.B, t_mid)};
        const Edge bt{lerp(bS.A, bE.A, t_mid), lerp(bS.B, bE.B, t_mid)};
        min_dist = edge_closest(at, bt, r.P, r.Q);
        r.toc = t_mid;
    }
    if (min_dist > 1e-8) {
        double t = 0.0;
        for (int iter = 0; iter < 10; iter++) {
            const Edge at{lerp(aS.A, aE.A, t), lerp(aS.B, aE.B, t)};
            const Edge bt{lerp(bS.A, bE.A, t), lerp(bS.B, bE.B, t)};
            V3 P, Q;
            const double dist = edge_closest(at, bt, P, Q);
            if (dist < min_dist) {
                min_dist = dist;
                r.P = P;
                r.Q = Q;
                r.toc = t;
            }
            const double pa = edge_project(at, P);
            const double pb = edge_project(bt, Q);
            double td, td2;
            ee_newton_terms(aS, aE, bS, bE, pa, pb, t, td, td2);
            t = t - td / td2;
            t = clamp01(t);
        }
    }
    r.dist = min_dist;
    return r;
}

// Sequential (dist, toc) reduction of triTriCCDLinear
// (continuous_comparison.h:709, 720, 770).
inline void ccd_take(CcdResult& best, const CcdResult& c) {
    if (c.dist < best.dist || (c.dist == best.dist && c.toc < best.toc)) best = c;
}

// collision_detection/continuous_comparison.h:680-779 triTriCCDLinear, with the
// per-body-pair products inverse(T_tri) * T_pt supplied by the caller.
struct PairMats {
    M4 aS, aE, bS, bE;  // rigid transforms of a and b at start / end
    M4 ab_S, ab_E;      // inverse(bS) * aS, inverse(bE) * aE : a's points into b's frame
    M4 ba_S, ba_E;      // inverse(aS) * bS, inverse(aE) * bE
};
inline PairMats pair_mats(const M4& aS, const M4& aE, const M4& bS, const M4& bE) {
    PairMats m;
    m.aS = aS;
    m.aE = aE;
    m.bS = bS;
    m.bE = bE;
    m.ab_S = mat_mul(mat_inverse(bS), aS);
    m.ab_E = mat_mul(mat_inverse(bE), aE);
    m.ba_S = mat_mul(mat_inverse(aS), bS);
    m.ba_E = mat_mul(mat_inverse(aE), bE);
    return m;
}

inline CcdResult tri_tri_ccd(const Tri& a, const Tri& b, const PairMats& M) {
    CcdResult best;
    best.dist = std::numeric_limits<double>::infinity();
    best.toc = 1.0;
    best.P = V3{0, 0, 0};
    best.Q = V3{0, 0, 0};
    const Tri a_s = tri_xform(a, M.aS), a_e = tri_xform(a, M.aE);
    const Tri b_s = tri_xform(b, M.bS), b_e = tri_xform(b, M.bE);
    for (int i = 0; i < 3; i++) {
        ccd_take(best, point_tri_ccd_c(tri_vertex(a, i), M.ab_S, M.ab_E, b, M.bS, M.bE));
        ccd_take(best, point_tri_ccd_c(tri_vertex(b, i), M.ba_S, M.ba_E, a, M.aS, M.aE));
        const Edge ae_s = tri_edge(a_s, i), ae_e = tri_edge(a_e, i);
        for (int j = 0; j < 3; j++) {
            const Edge be_s = tri_edge(b_s, j), be_e = tri_edge(b_e, j);
            ccd_take(best, edge_edge_ccd(ae_s, ae_e, be_s, be_e));
        }
    }
    return best;
}

// --------------------------------------------------- tree traversals -------
struct NodePair {
    int a, b;  // global node ids
};

struct Counters {
    long long node_pairs = 0;   // node pairs visited (both stages)
    long long tri_pairs = 0;    // primitive tests that ran the full CCD / distance
    long long leaf_pairs = 0;   // connected-stage node pairs
};

// collision_detection/comparison_dist.h:205-240 findContactsBucketComparison
// (poses: future states of both bodies).
inline void bucket_comparison(const TreeSet& T, const std::vector<NodePair>& dc, const Body& a, const Body& b, int ia,
                              int ib, std::vector<Contact>& hits, std::vector<int>& pair_used, Counters* cnt) {
    const float search_dist = (float)(a.geo_eps + b.geo_eps);
    pair_used.clear();
    const M4 Ta = state_transform(a.fut), Tb = state_transform(b.fut);
    for (const NodePair& np : dc) {
        const int na = T.nt(np.a), nb = T.nt(np.b);
        if (cnt) cnt->node_pairs++;
        for (int i = 0; i < na; i++) {
            const Tri A = tri_xform(T.tri(np.a, i), Ta);
            for (int j = 0; j < nb; j++) {
                const Tri B = tri_xform(T.tri(np.b, j), Tb);
                const DistResult d = tri_tri_dist(A, B);
                if (cnt) cnt->tri_pairs++;
                if (d.dist < ((double)search_dist + T.e(np.a, i)) + T.e(np.b, j)) {
                    Contact c;
                    c.A = d.P;
                    c.B = d.Q;
                    c.eps_a = a.geo_eps + T.e(np.a, i);
                    c.eps_b = b.geo_eps + T.e(np.b, j);
                    c.eps_inner_a = T.ie(np.a, i);
                    c.eps_inner_b = T.ie(np.b, j);
                    c.toc = 0.0;
                    c.pa = ia;
                    c.pb = ib;
                    hits.push_back(c);
                }
            }
        }
        pair_used.push_back((int)hits.size());
    }
}

// Expansion rule shared by both traversals (full_tree_comparison.h:28-59).
// Returns 0 = leaf-leaf, 1 = advance a, 2 = advance b.
inline int expand_rule(const Node& a, const Node& b) {
    if (!a.is_inner && !b.is_inner) return 0;
    if (!a.is_inner) return 2;
    if (!b.is_inner) return 1;
    return (a.depth < b.depth) ? 1 : 2;
}

// collision_detection/full_tree_comparison.h:13-67 compareTreesFull.
inline std::vector<Contact> compare_trees_full(const TreeSet& T, const Body& a, const Body& b, int ia, int ib,
                                               Counters* cnt = nullptr) {
    std::vector<Contact> result;
    std::vector<NodePair> dc{NodePair{T.root(a.mesh), T.root(b.mesh)}}, next;
    std::vector<int> num_hits;
    std::vector<Contact> hits;
    while (!dc.empty()) {
        hits.clear();
        bucket_comparison(T, dc, a, b, ia, ib, hits, num_hits, cnt);
        int last = 0;
        for (size_t i = 0; i < dc.size(); i++) {
            if (num_hits[i] > last) {
                const Node na = T.node(dc[i].a), nb = T.node(dc[i].b);
                const int rule = expand_rule(na, nb);
                if (rule == 0) {
                    result.insert(result.end(), hits.begin() + last, hits.begin() + num_hits[i]);
                } else if (rule == 1) {
                    for (int c = 0; c < na.num_children; c++) next.push_back(NodePair{na.child_first + c, dc[i].b});
                } else {
                    for (int c = 0; c < nb.num_children; c++) next.push_back(NodePair{dc[i].a, nb.child_first + c});
                }
            }
            last = num_hits[i];
        }
        dc.swap(next);
        next.clear();
    }
    return result;
}

// collision_detection/continuous_comparison.h:783-828 (soup stage; bucket eps ignored).
inline void bucket_continuous_soup(const TreeSet& T, const std::vector<NodePair>& dc, const Body& a, const Body& b,
                                   int ia, int ib, const PairMats& M, std::vector<Contact>& hits,
                                   std::vector<int>& pair_used, Counters* cnt) {
    const float search_dist = (float)(a.geo_eps + b.geo_eps);
    pair_used.clear();
    for (const NodePair& np : dc) {
        const int na = T.nt(np.a), nb = T.nt(np.b);
        if (cnt) cnt->node_pairs++;
        for (int i = 0; i < na; i++) {
            const Tri at = T.tri(np.a, i);
            const BBox abox =
                bbox_expand(bbox_union(tri_bbox(tri_xform(at, M.aS)), tri_bbox(tri_xform(at, M.aE))), a.geo_eps);
            for (int j = 0; j < nb; j++) {
                const Tri bt = T.tri(np.b, j);
                const BBox bbox =
                    bbox_expand(bbox_union(tri_bbox(tri_xform(bt, M.bS)), tri_bbox(tri_xform(bt, M.bE))), b.geo_eps);
                if (bbox_overlap(abox, bbox)) {
                    if (cnt) cnt->tri_pairs++;
                    const CcdResult r = tri_tri_ccd(at, bt, M);
                    if (r.dist < (double)search_dist) {
                        Contact c;
                        c.A = r.P;
                        c.B = r.Q;
                        c.eps_a = a.geo_eps;
                        c.eps_b = b.geo_eps;
                        c.eps_inner_a = 0.0;
                        c.eps_inner_b = 0.0;
                        c.toc = r.toc;
                        c.pa = ia;
                        c.pb = ib;
                        hits.push_back(c);
                    }
                }
            }
        }
        pair_used.push_back((int)hits.size());
    }
}

// collision_detection/continuous_comparison.h:831-910 (connected stage, run on
// soup buckets: vertices and edges duplicated per triangle,
// model/surrogate_components.cpp:127-147).
inline void bucket_continuous_connected(const TreeSet& T, const std::vector<NodePair>& dc, const Body& a,
                                        const Body& b, int ia, int ib, const PairMats& M, std::vector<Contact>& hits,
                                        std::vector<int>& pair_used, Counters* cnt) {
    const float search_dist = (float)(a.geo_eps + b.geo_eps);
    pair_used.clear();
    auto emit = [&](V3 A, V3 B, double toc) {
        Contact c;
        c.A = A;
        c.B = B;
        c.eps_a = a.geo_eps;
        c.eps_b = b.geo_eps;
        c.eps_inner_a = 0.0;
        c.eps_inner_b = 0.0;
        c.toc = toc;
        c.pa = ia;
        c.pb = ib;
        hits.push_back(c);
    };
    for (const NodePair& np : dc) {
        const int na = T.nt(np.a), nb = T.nt(np.b);
        if (cnt) {
            cnt->node_pairs++;
            cnt->leaf_pairs++;
        }
        for (int vi = 0; vi < 3 * na; vi++) {  // a vertices vs b triangles
            const V3 av = tri_vertex(T.tri(np.a, vi / 3), vi % 3);
            for (int j = 0; j < nb; j++) {
                const CcdResult r = point_tri_ccd_c(av, M.ab_S, M.ab_E, T.tri(np.b, j), M.bS, M.bE);
                if (cnt) cnt->tri_pairs++;
                if (r.dist < (double)search_dist) emit(r.P, r.Q, r.toc);
            }
        }
        for (int vi = 0; vi < 3 * nb; vi++) {  // b vertices vs a triangles (P/Q swapped)
            const V3 bv = tri_vertex(T.tri(np.b, vi / 3), vi % 3);
            for (int j = 0; j < na; j++) {
                const CcdResult r = point_tri_ccd_c(bv, M.ba_S, M.ba_E, T.tri(np.a, j), M.aS, M.aE);
                if (cnt) cnt->tri_pairs++;
                if (r.dist < (double)search_dist) emit(r.Q, r.P, r.toc);
            }
        }
        for (int ei = 0; ei < 3 * na; ei++) {  // edges vs edges (P/Q swapped as in the reference)
            const Edge ae = tri_edge(T.tri(np.a, ei / 3), ei % 3);
            const Edge aes{xform(ae.A, M.aS), xform(ae.B, M.aS)};
            const Edge aee{xform(ae.A, M.aE), xform(ae.B, M.aE)};
            for (int ej = 0; ej < 3 * nb; ej++) {
                const Edge be = tri_edge(T.tri(np.b, ej / 3), ej % 3);
                const Edge bes{xform(be.A, M.bS), xform(be.B, M.bS)};
                const Edge bee{xform(be.A, M.bE), xform(be.B, M.bE)};
                const CcdResult r = edge_edge_ccd(aes, aee, bes, bee);
                if (cnt) cnt->tri_pairs++;
                if (r.dist < (double)search_dist) emit(r.Q, r.P, r.toc);
            }
        }
        pair_used.push_back((int)hits.size());
    }
}

// One expansion pass of compareTreesFullContinuous over a stage's frontier
// (full_tree_comparison.h:99-150 and 160-211).
inline void ccd_expand(const TreeSet& T, const std::vector<NodePair>& dc, const std::vector<Contact>& hits,
                       const std::vector<int>& num_hits, double max_time, std::vector<Contact>& result,
                       double& min_time_out, std::vector<NodePair>& soup_next, std::vector<NodePair>& conn_next) {
    int last = 0;
    for (size_t i = 0; i < dc.size(); i++) {
        if (num_hits[i] > last) {
            const Node na = T.node(dc[i].a), nb = T.node(dc[i].b);
            const int rule = expand_rule(na, nb);
            if (rule == 0) {
                result.insert(result.end(), hits.begin() + last, hits.begin() + num_hits[i]);
                for (const Contact& c : hits) min_time_out = dmin(min_time_out, c.toc * max_time);
            } else {
                const int nch = rule == 1 ? na.num_children : nb.num_children;
                for (int c = 0; c < nch; c++) {
                    const int ga = rule == 1 ? na.child_first + c : dc[i].a;
                    const int gb = rule == 1 ? dc[i].b : nb.child_first + c;
                    const Node ca = T.node(ga), cb = T.node(gb);
                    if (ca.is_inner || cb.is_inner)
                        soup_next.push_back(NodePair{ga, gb});
                    else
                        conn_next.push_back(NodePair{ga, gb});
                }
            }
        }
        last = num_hits[i];
    }
}

// collision_detection/full_tree_comparison.h:69-219 compareTreesFullContinuous.
// Projects both future states over max_time first (the reference mutates the
// bodies the same way, :78-79).
inline std::vector<Contact> compare_trees_full_continuous(const TreeSet& T, Body& a, Body& b, int ia, int ib,
                                                          double max_time, double& min_time_out,
                                                          Counters* cnt = nullptr) {
    std::vector<Contact> result;
    min_time_out = max_time;
    a.fut = state_extrapolate(a.cur, max_time, a.ii);
    b.fut = state_extrapolate(b.cur, max_time, b.ii);
    const PairMats M =
        pair_mats(state_transform(a.cur), state_transform(a.fut), state_transform(b.cur), state_transform(b.fut));
    std::vector<NodePair> soup{NodePair{T.root(a.mesh), T.root(b.mesh)}}, conn, soup_next, conn_next;
    std::vector<int> num_hits;
    std::vector<Contact> hits;
    while (!soup.empty() || !conn.empty()) {
        hits.clear();
        bucket_continuous_soup(T, soup, a, b, ia, ib, M, hits, num_hits, cnt);
        ccd_expand(T, soup, hits, num_hits, max_time, result, min_time_out, soup_next, conn_next);
        hits.clear();
        bucket_continuous_connected(T, conn, a, b, ia, ib, M, hits, num_hits, cnt);
        ccd_expand(T, conn, hits, num_hits, max_time, result, min_time_out, soup_next, conn_next);
        soup.swap(soup_next);
        soup_next.clear();
        conn.swap(conn_next);
        conn_next.clear();
    }
    return result;
}

}  // namespace d2o
