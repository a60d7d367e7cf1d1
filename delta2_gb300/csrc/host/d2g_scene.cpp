// Host-side scene set-up (see d2g_scene.hpp).  Compiled with
// -ffp-contract=off so scenes are bit-identical on x86-64 and Arm.
#include "d2g_scene.hpp"

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <deque>
#include <limits>
#include <map>
#include <set>
#include <thread>
#include <tuple>
#include <utility>

#include "../d2g_math.cuh"

namespace d2g {

// --------------------------------------------------------------- PCG32 -----
void Pcg32::seed(uint64_t initstate, uint64_t initseq) {
    state = 0U;
    inc = (initseq << 1u) | 1u;
    next();
    state += initstate;
    next();
}
uint32_t Pcg32::next() {
    const uint64_t old = state;
    state = old * 6364136223846793005ULL + inc;
    const uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    const uint32_t rot = (uint32_t)(old >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((-rot) & 31));
}
uint32_t Pcg32::bounded(uint32_t bound) {
    const uint32_t threshold = (0u - bound) % bound;
    for (;;) {
        const uint32_t r = next();
        if (r >= threshold) return r % bound;
    }
}
double Pcg32::uniform() {
    const uint64_t hi = next() >> 6;  // 26 bits
    const uint64_t lo = next() >> 5;  // 27 bits
    return (double)((hi << 27) | lo) * (1.0 / 9007199254740992.0);
}

namespace {

struct P3 {
    double x, y, z;
};
P3 p3(const double* v) { return P3{v[0], v[1], v[2]}; }
P3 sub(P3 a, P3 b) { return P3{a.x - b.x, a.y - b.y, a.z - b.z}; }
P3 add(P3 a, P3 b) { return P3{a.x + b.x, a.y + b.y, a.z + b.z}; }
P3 mul(P3 a, double s) { return P3{a.x * s, a.y * s, a.z * s}; }
double pdot(P3 a, P3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
P3 pcross(P3 a, P3 b) { return P3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
double pnorm(P3 a) { return std::sqrt(pdot(a, a)); }
double smin(double a, double b) { return (b < a) ? b : a; }
double smax(double a, double b) { return (a < b) ? b : a; }

// common/triangle.h:21-23
double tri_area(const double* t) {
    const P3 A = p3(t), B = p3(t + 3), C = p3(t + 6);
    return 0.5 * pnorm(pcross(sub(A, C), sub(B, C)));
}

// common/triangle.h:280-471 Triangle::distToPoint (closest point by the
// seven regions of the triangle's parameter plane).
double dist_to_point(const double* T, P3 X) {
    const P3 A = p3(T), B = p3(T + 3), C = p3(T + 6);
    const P3 AX = sub(X, A), AB = sub(B, A), AC = sub(C, A);
    const double a00 = pdot(AB, AB), a01 = pdot(AB, AC), a11 = pdot(AC, AC);
    const double b0 = -pdot(AX, AB), b1 = -pdot(AX, AC);
    const double det = a00 * a11 - a01 * a01;
    double t0 = a01 * b1 - a11 * b0;
    double t1 = a01 * b0 - a00 * b1;
    if (t0 + t1 <= det) {
        if (t0 < 0.0) {
            if (t1 < 0.0) {
                if (b0 < 0.0) {
                    t1 = 0.0;
                    t0 = (-b0 >= a00) ? 1.0 : -b0 / a00;
                } else {
                    t0 = 0.0;
                    if (b1 >= 0.0)
                        t1 = 0.0;
                    else if (-b1 >= a11)
                        t1 = 1.0;
                    else
                        t1 = -b1 / a11;
                }
            } else {
                t0 = 0.0;
                if (b1 >= 0.0)
                    t1 = 0.0;
                else if (-b1 >= a11)
                    t1 = 1.0;
                else
                    t1 = -b1 / a11;
            }
        } else if (t1 < 0.0) {
            t1 = 0.0;
            if (b0 >= 0.0)
                t0 = 0.0;
            else if (-b0 >= a00)
                t0 = 1.0;
            else
                t0 = -b0 / a00;
        } else {
            const double invDet = 1.0 / det;
            t0 *= invDet;
            t1 *= invDet;
        }
    } else {
        if (t0 < 0.0) {
            const double tmp0 = a01 + b0, tmp1 = a11 + b1;
            if (tmp1 > tmp0) {
                const double numer = tmp1 - tmp0;
                const double denom = (a00 - 2.0 * a01) + a11;
                if (numer >= denom) {
                    t0 = 1.0;
                    t1 = 0.0;
                } else {
                    t0 = numer / denom;
                    t1 = 1.0 - t0;
                }
            } else {
                t0 = 0.0;
                if (tmp1 <= 0.0)
                    t1 = 1.0;
                else if (b1 >= 0.0)
                    t1 = 0.0;
                else
                    t1 = -b1 / a11;
            }
        } else if (t1 < 0.0) {
            const double tmp0 = a01 + b1, tmp1 = a00 + b0;
            if (tmp1 > tmp0) {
                const double numer = tmp1 - tmp0;
                const double denom = (a00 - 2.0 * a01) + a11;
                if (numer >= denom) {
                    t1 = 1.0;
                    t0 = 0.0;
                } else {
                    t1 = numer / denom;
                    t0 = 1.0 - t1;
                }
            } else {
                t1 = 0.0;
                if (tmp1 <= 0.0)
                    t0 = 1.0;
                else if (b0 >= 0.0)
                    t0 = 0.0;
                else
                    t0 = -b0 / a00;
            }
        } else {
            const double numer = ((a11 + b1) - a01) - b0;
            if (numer <= 0.0) {
                t0 = 0.0;
                t1 = 1.0;
            } else {
                const double denom = (a00 - 2.0 * a01) + a11;
                if (numer >= denom) {
                    t0 = 1.0;
                    t1 = 0.0;
                } else {
                    t0 = numer / denom;
                    t1 = 1.0 - t0;
                }
            }
        }
    }
    const P3 diff = sub(X, add(add(A, mul(AB, t0)), mul(AC, t1)));
    return pnorm(diff);
}

struct TriRec {
    double v[9];
};

// model/fit_surrogate_triangle.h:247-299 selectSurrogateTriangle: the largest
// of log2(n)*10 random vertex triples.  When every draw is degenerate the
// reference keeps an uninitialised triangle; here the first non-degenerate
// triple in index order is taken (the enumeration its code intends).
bool select_surrogate(const std::vector<P3>& pts, Pcg32& rng, TriRec& out) {
    const int n = (int)pts.size();
    double best = -1;
    TriRec res;
    for (int k = 0; k < 9; k++) res.v[k] = 0.0;
    auto mk = [&](int a, int b, int c) {
        TriRec t;
        const P3 q[3] = {pts[a], pts[b], pts[c]};
        for (int i = 0; i < 3; i++) {
            t.v[3 * i] = q[i].x;
            t.v[3 * i + 1] = q[i].y;
            t.v[3 * i + 2] = q[i].z;
        }
        return t;
    };
    if (n > 3) {
        const int attempts = (int)(std::log2((double)n) * 10);
        for (int i = 0; i < attempts; i++) {
            const int a = (int)rng.bounded((uint32_t)n);
            const int b = (int)rng.bounded((uint32_t)n);
            const int c = (int)rng.bounded((uint32_t)n);
            const TriRec t = mk(a, b, c);
            const double area = tri_area(t.v);
            if (area > best && area > 0.0) {
                res = t;
                best = area;
            }
        }
        if (!(tri_area(res.v) > 0.0)) {
            for (int a = 0; a < n && !(tri_area(res.v) > 0.0); a++)
                for (int b = a + 1; b < n && !(tri_area(res.v) > 0.0); b++)
                    for (int c = b + 1; c < n; c++) {
                        res = mk(a, b, c);
                        if (tri_area(res.v) > 0.0) break;
                    }
        }
    } else {
        res = mk(0, 1, 2);
    }
    out = res;
    return tri_area(res.v) > 0.0;
}

std::vector<P3> group_points(const std::vector<TriRec>& tris, const std::vector<int>& ids) {
    std::vector<P3> pts;
    for (int id : ids) {
        pts.push_back(p3(tris[id].v));
        pts.push_back(p3(tris[id].v + 3));
        pts.push_back(p3(tris[id].v + 6));
    }
    return pts;
}

// model/construct_surrogate_tree.h:8-168 divideAndFit (k-means-like grouping).
bool divide_and_fit(const std::vector<TriRec>& tris, const std::vector<int>& tri_ids, int branching, bool force,
                    Pcg32& rng, std::vector<TriRec>& tris_out, std::vector<std::vector<int>>& ids_out,
                    std::string* err) {
    if (branching > (int)tri_ids.size()) {
        if (err) *err = "There must be more triangles than branches";
        return false;
    }
    tris_out.assign(branching, TriRec{});
    ids_out.assign(branching, {});
    // Initial group triangles: the mesh's first `branching` triangles (as the reference does).
    for (int i = 0; i < branching; i++) tris_out[i] = tris[i];
    for (int iteration = 0; iteration < 20; iteration++) {
        for (auto& g : ids_out) g.clear();
        for (int tri_i : tri_ids) {
            double best_dist = std::numeric_limits<double>::infinity();
            int best_group = 0;
            for (int g = 0; g < branching; g++) {
                const double da = dist_to_point(tris_out[g].v, p3(tris[tri_i].v));
                const double db = dist_to_point(tris_out[g].v, p3(tris[tri_i].v + 3));
                const double dc = dist_to_point(tris_out[g].v, p3(tris[tri_i].v + 6));
                const double mx = smax(smax(da, db), dc);
                if (mx < best_dist) {
                    best_group = g;
                    best_dist = mx;
                }
            }
            ids_out[best_group].push_back(tri_i);
        }
        for (int g = 0; g < branching; g++) {
            if (!ids_out[g].empty()) {
                TriRec sel;
                if (!select_surrogate(group_points(tris, ids_out[g]), rng, sel)) {
                    if (err) *err = "No valid surrogate triangle was found";
                    return false;
                }
                tris_out[g] = sel;
            }
        }
        if (force) {
            bool improving = true, branching_met = false;
            while (improving && !branching_met) {
                int largest = 0;
                size_t largest_size = 0;
                std::vector<int> zero;
                for (int g = 0; g < branching; g++) {
                    if (ids_out[g].size() > largest_size) {
                        largest_size = ids_out[g].size();
                        largest = g;
                    }
                    if (ids_out[g].empty()) zero.push_back(g);
                }
                if (!zero.empty()) {
                    std::vector<TriRec> sub;
                    std::vector<std::vector<int>> sub_ids;
                    const int num = (int)std::min(ids_out[largest].size(), zero.size() + 1);
                    const std::vector<int> src = ids_out[largest];
                    if (!divide_and_fit(tris, src, num, false, rng, sub, sub_ids, err)) return false;
                    int sub_nonzero = 0;
                    for (int s = 0; s < (int)sub.size(); s++) {
                        const int gi = s == 0 ? largest : zero[s - 1];
                        if (!sub_ids[s].empty()) {
                            sub_nonzero++;
                            ids_out[gi] = sub_ids[s];
                            tris_out[gi] = sub[s];
                        }
                    }
                    improving = sub_nonzero > 1;
                } else {
                    branching_met = true;
                }
            }
            if (!branching_met) {
                std::vector<int> zero;
                do {
                    int largest = 0;
                    size_t largest_size = 0;
                    zero.clear();
                    for (int g = 0; g < branching; g++) {
                        if (ids_out[g].size() > largest_size) {
                            largest_size = ids_out[g].size();
                            largest = g;
                        }
                        if (ids_out[g].empty()) zero.push_back(g);
                    }
                    // the reference's loop bound is re-evaluated as the largest group shrinks
                    for (size_t z = 0; z < std::min(zero.size(), ids_out[largest].size() - 1); z++) {
                        const int zi = zero[z];
                        const int tri_i = ids_out[largest].back();
                        ids_out[zi].push_back(tri_i);
                        ids_out[largest].pop_back();
                        tris_out[zi] = tris[tri_i];
                    }
                    TriRec sel;
                    if (!select_surrogate(group_points(tris, ids_out[largest]), rng, sel)) {
                        if (err) *err = "No valid surrogate triangle was found";
                        return false;
                    }
                    tris_out[largest] = sel;
                } while (!zero.empty());
            }
        }
    }
    return true;
}

// model/construct_surrogate_tree.h:172-185 calcEpss
void calc_epss(const TriRec& sur, const std::vector<TriRec>& tris, const std::vector<int>& ids, double& inner,
               double& eps) {
    inner = std::numeric_limits<double>::infinity();
    eps = 0.0;
    for (int id : ids) {
        const double a = dist_to_point(sur.v, p3(tris[id].v));
        const double b = dist_to_point(sur.v, p3(tris[id].v + 3));
        const double c = dist_to_point(sur.v, p3(tris[id].v + 6));
        inner = smin(inner, smin(a, smin(b, c)));
        eps = smax(eps, smax(a, smax(b, c)));
    }
}

void inv3(const double* m, double* r) {
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

// model/inertia.cpp:20-73 tetrahedronInertiaTensor (Tonon 2005), with the
// reference's placement of the product terms.  `sign` carries the tet's
// orientation (the reference passes density -1 for tetgen's orientation).
void tet_inertia(P3 a, P3 b, P3 c, P3 d, double sign, double* I) {
    const double A[3] = {a.x, a.y, a.z}, B[3] = {b.x, b.y, b.z}, C[3] = {c.x, c.y, c.z}, D[3] = {d.x, d.y, d.z};
    const double detJ = pdot(sub(a, d), pcross(sub(b, d), sub(c, d)));
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

}  // namespace

// ------------------------------------------------------------------ meshes -
Mesh make_cube(double h) {
    Mesh m;
    const double V[8][3] = {{1, 1, 1}, {1, 1, -1}, {1, -1, 1}, {1, -1, -1},
                            {-1, 1, 1}, {-1, 1, -1}, {-1, -1, 1}, {-1, -1, -1}};
    const int F[12][3] = {{0, 2, 1}, {1, 2, 3}, {2, 6, 3}, {3, 6, 7}, {4, 5, 6}, {5, 7, 6},
                          {4, 0, 1}, {4, 1, 5}, {0, 4, 6}, {0, 6, 2}, {3, 7, 1}, {7, 5, 1}};
    for (auto& v : V)
        for (double c : v) m.V.push_back(c * h);
    for (auto& f : F)
        for (int c : f) m.F.push_back(c);
    return m;
}

Mesh make_plane(double width) {
    Mesh m;
    const double h = width / 2.0;
    m.V = {h, h, 0.0, h, -h, 0.0, -h, h, 0.0, -h, -h, 0.0};
    m.F = {0, 2, 1, 1, 2, 3};
    return m;
}

// A box open at the top: floor [-w/2, w/2]^2 at z = 0 and four walls of
// height h, ten triangles wound so that their normals face the inside.
Mesh make_open_box(double w, double h) {
    Mesh m;
    const double a = w / 2.0;
    m.V = {-a, -a, 0.0, a, -a, 0.0, a, a, 0.0, -a, a, 0.0, -a, -a, h, a, -a, h, a, a, h, -a, a, h};
    m.F = {0, 1, 2, 0, 2, 3,   // floor (+z)
           0, 5, 1, 0, 4, 5,   // y = -a (+y)
           1, 6, 2, 1, 5, 6,   // x = +a (-x)
           2, 7, 3, 2, 6, 7,   // y = +a (-y)
           3, 4, 0, 3, 7, 4};  // x = -a (+x)
    return m;
}

Mesh make_icosphere(int subdiv, double radius, double noise, Pcg32* rng) {
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    std::vector<P3> V = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                         {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    std::vector<std::array<int, 3>> F = {{0, 11, 5}, {0, 5, 1},  {0, 1, 7},   {0, 7, 10}, {0, 10, 11},
                                         {1, 5, 9},  {5, 11, 4}, {11, 10, 2}, {10, 7, 6}, {7, 1, 8},
                                         {3, 9, 4},  {3, 4, 2},  {3, 2, 6},   {3, 6, 8},  {3, 8, 9},
                                         {4, 9, 5},  {2, 4, 11}, {6, 2, 10},  {8, 6, 7},  {9, 8, 1}};
    for (auto& v : V) v = mul(v, 1.0 / pnorm(v));
    for (int s = 0; s < subdiv; s++) {
        std::map<std::pair<int, int>, int> mid;
        auto midpoint = [&](int a, int b) {
            const auto key = std::make_pair(std::min(a, b), std::max(a, b));
            auto f = mid.find(key);
            if (f != mid.end()) return f->second;
            P3 m = mul(add(V[a], V[b]), 0.5);
            m = mul(m, 1.0 / pnorm(m));
            V.push_back(m);
            mid[key] = (int)V.size() - 1;
            return (int)V.size() - 1;
        };
        std::vector<std::array<int, 3>> G;
        for (auto& f : F) {
            const int ab = midpoint(f[0], f[1]), bc = midpoint(f[1], f[2]), ca = midpoint(f[2], f[0]);
            G.push_back({f[0], ab, ca});
            G.push_back({f[1], bc, ab});
            G.push_back({f[2], ca, bc});
            G.push_back({ab, bc, ca});
        }
        F.swap(G);
    }
    Mesh m;
    for (auto& v : V) {
        double r = radius;
        if (noise != 0.0 && rng) r = radius * (1.0 + noise * (2.0 * rng->uniform() - 1.0));
        m.V.push_back(v.x * r);
        m.V.push_back(v.y * r);
        m.V.push_back(v.z * r);
    }
    for (auto& f : F) {  // orient outward (normal away from the centre)
        const P3 a = p3(&m.V[3 * f[0]]), b = p3(&m.V[3 * f[1]]), c = p3(&m.V[3 * f[2]]);
        const P3 n = pcross(sub(b, a), sub(c, a));
        if (pdot(n, add(add(a, b), c)) < 0.0) std::swap(f[1], f[2]);
        m.F.push_back(f[0]);
        m.F.push_back(f[1]);
        m.F.push_back(f[2]);
    }
    return m;
}

// Incremental convex hull (Barber, Dobkin & Huhdanpaa style visible-face
// removal and horizon re-triangulation) of points drawn uniformly in a ball.
Mesh make_hull(int npts, double radius, Pcg32& rng) {
    std::vector<P3> P;
    while ((int)P.size() < npts) {
        const P3 q{2.0 * rng.uniform() - 1.0, 2.0 * rng.uniform() - 1.0, 2.0 * rng.uniform() - 1.0};
        if (pdot(q, q) <= 1.0) P.push_back(mul(q, radius));
    }
    const int n = (int)P.size();
    int i0 = 0, i1 = 0, i2 = 0, i3 = 0;
    double best = -1;
    for (int i = 1; i < n; i++) {
        const double d = pdot(sub(P[i], P[i0]), sub(P[i], P[i0]));
        if (d > best) {
            best = d;
            i1 = i;
        }
    }
    best = -1;
    const P3 dir = sub(P[i1], P[i0]);
    for (int i = 0; i < n; i++) {
        const P3 c = pcross(dir, sub(P[i], P[i0]));
        const double d = pdot(c, c);
        if (d > best) {
            best = d;
            i2 = i;
        }
    }
    best = -1;
    const P3 nrm = pcross(sub(P[i1], P[i0]), sub(P[i2], P[i0]));
    for (int i = 0; i < n; i++) {
        const double d = std::fabs(pdot(nrm, sub(P[i], P[i0])));
        if (d > best) {
            best = d;
            i3 = i;
        }
    }
    std::vector<std::array<int, 3>> faces;
    const int tet[4] = {i0, i1, i2, i3};
    const int tf[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};
    for (int f = 0; f < 4; f++) {
        std::array<int, 3> F = {tet[tf[f][0]], tet[tf[f][1]], tet[tf[f][2]]};
        const int other = tet[6 - tf[f][0] - tf[f][1] - tf[f][2]];
        const P3 nn = pcross(sub(P[F[1]], P[F[0]]), sub(P[F[2]], P[F[0]]));
        if (pdot(nn, sub(P[other], P[F[0]])) > 0.0) std::swap(F[1], F[2]);
        faces.push_back(F);
    }
    const double tol = 1e-12 * radius * radius * radius;
    for (int p = 0; p < n; p++) {
        if (p == i0 || p == i1 || p == i2 || p == i3) continue;
        std::vector<char> vis(faces.size(), 0);
        bool any = false;
        for (size_t f = 0; f < faces.size(); f++) {
            const auto& F = faces[f];
            const P3 nn = pcross(sub(P[F[1]], P[F[0]]), sub(P[F[2]], P[F[0]]));
            if (pdot(nn, sub(P[p], P[F[0]])) > tol) {
                vis[f] = 1;
                any = true;
            }
        }
        if (!any) continue;
        std::set<std::pair<int, int>> vis_edges;
        for (size_t f = 0; f < faces.size(); f++)
            if (vis[f])
                for (int k = 0; k < 3; k++) vis_edges.insert(std::make_pair(faces[f][k], faces[f][(k + 1) % 3]));
        std::vector<std::pair<int, int>> horizon;
        for (size_t f = 0; f < faces.size(); f++)
            if (vis[f])
                for (int k = 0; k < 3; k++) {
                    const int u = faces[f][k], v = faces[f][(k + 1) % 3];
                    if (!vis_edges.count(std::make_pair(v, u))) horizon.push_back(std::make_pair(u, v));
                }
        std::vector<std::array<int, 3>> kept;
        for (size_t f = 0; f < faces.size(); f++)
            if (!vis[f]) kept.push_back(faces[f]);
        for (const auto& e : horizon) kept.push_back({e.first, e.second, p});
        faces.swap(kept);
    }
    std::vector<int> remap(n, -1);
    Mesh m;
    for (int i = 0; i < n; i++) {
        bool used = false;
        for (const auto& f : faces) used = used || f[0] == i || f[1] == i || f[2] == i;
        if (used) {
            remap[i] = m.nv();
            m.V.push_back(P[i].x);
            m.V.push_back(P[i].y);
            m.V.push_back(P[i].z);
        }
    }
    for (const auto& f : faces)
        for (int k = 0; k < 3; k++) m.F.push_back(remap[f[k]]);
    return m;
}

// ------------------------------------------------------- mass properties ---
MassProps mass_volume(const Mesh& m) {
    MassProps mp;
    double vol = 0;
    P3 com{0, 0, 0};
    for (int f = 0; f < m.nf(); f++) {
        const P3 a = p3(&m.V[3 * m.F[3 * f]]), b = p3(&m.V[3 * m.F[3 * f + 1]]), c = p3(&m.V[3 * m.F[3 * f + 2]]);
        const double v = pdot(a, pcross(b, c)) / 6.0;
        vol += v;
        com = add(com, mul(add(add(a, b), c), v / 4.0));
    }
    com = mul(com, 1.0 / vol);
    mp.volume = vol;
    mp.com[0] = com.x;
    mp.com[1] = com.y;
    mp.com[2] = com.z;
    for (int k = 0; k < 9; k++) mp.unit_inertia[k] = 0.0;
    for (int f = 0; f < m.nf(); f++) {
        const P3 a = sub(p3(&m.V[3 * m.F[3 * f]]), com), b = sub(p3(&m.V[3 * m.F[3 * f + 1]]), com),
                 c = sub(p3(&m.V[3 * m.F[3 * f + 2]]), com);
        tet_inertia(a, b, c, P3{0, 0, 0}, 1.0, mp.unit_inertia);
    }
    inv3(mp.unit_inertia, mp.unit_inertia_inv);
    return mp;
}

MassProps mass_surface(const Mesh& m, double thickness) {
    MassProps mp;
    double vol = 0;
    P3 com{0, 0, 0};
    for (int f = 0; f < m.nf(); f++) {
        double t[9];
        for (int k = 0; k < 3; k++)
            for (int j = 0; j < 3; j++) t[3 * k + j] = m.V[3 * m.F[3 * f + k] + j];
        const double tv = tri_area(t) * thickness;
        vol += tv;
        com = add(com, mul(mul(add(add(p3(t), p3(t + 3)), p3(t + 6)), 1.0 / 3.0), tv));
    }
    com = mul(com, 1.0 / vol);
    mp.volume = vol;
    mp.com[0] = com.x;
    mp.com[1] = com.y;
    mp.com[2] = com.z;
    for (int k = 0; k < 9; k++) mp.unit_inertia[k] = 0.0;
    for (int f = 0; f < m.nf(); f++) {
        double t[9];
        for (int k = 0; k < 3; k++)
            for (int j = 0; j < 3; j++) t[3 * k + j] = m.V[3 * m.F[3 * f + k] + j] - mp.com[j];
        const double tv = tri_area(t) * thickness;
        for (int k = 0; k < 3; k++) {  // model/inertia.cpp:75-84 pointInertiaTensor
            const double x = t[3 * k], y = t[3 * k + 1], z = t[3 * k + 2];
            const double pi[9] = {y * y + z * z, -x * y, -x * z, -x * y, x * x + z * z, -y * z, -x * z, -y * z, x * x + y * y};
            for (int j = 0; j < 9; j++) mp.unit_inertia[j] += tv * pi[j] / 3.0;
        }
    }
    inv3(mp.unit_inertia, mp.unit_inertia_inv);
    return mp;
}

void shift_vertices(Mesh& m, const double* c) {
    for (int i = 0; i < m.nv(); i++)
        for (int k = 0; k < 3; k++) m.V[3 * i + k] = m.V[3 * i + k] - c[k];
}

// ------------------------------------------------------------ tree build ---
bool build_tree(const Mesh& m, Pcg32& rng, Tree& out, std::string* err) {
    std::vector<TriRec> tris(m.nf());
    for (int f = 0; f < m.nf(); f++)
        for (int k = 0; k < 3; k++)
            for (int j = 0; j < 3; j++) tris[f].v[3 * k + j] = m.V[3 * m.F[3 * f + k] + j];
    out = Tree();
    std::vector<int> ids(m.nf());
    for (int i = 0; i < m.nf(); i++) ids[i] = i;
    std::deque<std::tuple<std::vector<int>, int, int>> q;
    q.push_back(std::make_tuple(ids, 0, -1));
    while (!q.empty()) {
        std::vector<int> g;
        int depth, parent;
        std::tie(g, depth, parent) = q.front();
        q.pop_front();
        const int node_id = out.n();
        int32_t node[4] = {-1, 0, 0, depth};
        std::vector<TriRec> bt;
        std::vector<double> e(8, 0.0), ie(8, 0.0);
        if (g.size() < 8) {
            for (int id : g) bt.push_back(tris[id]);
        } else {
            std::vector<TriRec> sur;
            std::vector<std::vector<int>> grp;
            if (!divide_and_fit(tris, g, 8, true, rng, sur, grp, err)) return false;
            for (size_t i = 0; i < grp.size(); i++) calc_epss(sur[i], tris, grp[i], ie[i], e[i]);
            bt = sur;
            node[1] = (int32_t)sur.size();
            node[2] = 1;
            for (size_t i = 0; i < sur.size(); i++) q.push_back(std::make_tuple(grp[i], depth + 1, node_id));
        }
        if (bt.size() > 8) {
            if (err) *err = "A bucket can only hold so many triangles.";
            return false;
        }
        for (int k = 0; k < 4; k++) out.nodes.push_back(node[k]);
        out.ntris.push_back((int32_t)bt.size());
        for (int i = 0; i < 8; i++)
            for (int k = 0; k < 9; k++) out.tris.push_back(i < (int)bt.size() ? bt[i].v[k] : 0.0);
        for (int i = 0; i < 8; i++) {
            out.eps.push_back(i < (int)bt.size() ? e[i] : 0.0);
            out.inner_eps.push_back(i < (int)bt.size() ? ie[i] : 0.0);
        }
        if (parent != -1 && out.nodes[4 * parent] == -1) out.nodes[4 * parent] = node_id;
    }
    return true;
}

// ------------------------------------------------------------ scenes -------
int scene_add_mesh(Scene& s, const Mesh& m, Pcg32& tree_rng, std::string* err) {
    Tree t;
    if (!build_tree(m, tree_rng, t, err)) return -1;
    return scene_add_tree(s, t, m.nf());
}

int scene_add_tree(Scene& s, const Tree& t, int n_faces) {
    if (s.mesh_node_off.empty()) s.mesh_node_off.push_back(0);
    const int base = s.mesh_node_off.back();
    for (int i = 0; i < t.n(); i++) {
        const int cf = t.nodes[4 * i];
        s.nodes.push_back(cf < 0 ? -1 : cf + base);
        s.nodes.push_back(t.nodes[4 * i + 1]);
        s.nodes.push_back(t.nodes[4 * i + 2]);
        s.nodes.push_back(t.nodes[4 * i + 3]);
    }
    s.ntris.insert(s.ntris.end(), t.ntris.begin(), t.ntris.end());
    s.tris.insert(s.tris.end(), t.tris.begin(), t.tris.end());
    s.eps.insert(s.eps.end(), t.eps.begin(), t.eps.end());
    s.inner_eps.insert(s.inner_eps.end(), t.inner_eps.begin(), t.inner_eps.end());
    s.mesh_node_off.push_back(base + t.n());
    s.mesh_ntris.push_back(n_faces);
    return (int)s.mesh_node_off.size() - 2;
}

// Trees of many meshes on all host cores; mesh k's tree draws from its own
// PCG32 stream (42, stream0 + k), so the trees do not depend on the order in
// which the threads build them.
bool build_trees_parallel(const std::vector<Mesh>& meshes, uint64_t stream0, std::vector<Tree>& out,
                          std::string* err) {
    const int n = (int)meshes.size();
    out.assign(n, Tree());
    std::vector<std::string> errs(n);
    std::atomic<int> next{0};
    std::atomic<bool> failed{false};
    auto work = [&]() {
        for (;;) {
            const int k = next.fetch_add(1);
            if (k >= n || failed.load()) break;
            Pcg32 r;
            r.seed(42u, stream0 + (uint64_t)k);
            if (!build_tree(meshes[k], r, out[k], &errs[k])) failed.store(true);
        }
    };
    const unsigned hw = std::thread::hardware_concurrency();
    const int nt = (int)std::max(1u, std::min(64u, std::min(hw ? hw : 1u, (unsigned)std::max(n, 1))));
    std::vector<std::thread> pool;
    for (int i = 1; i < nt; i++) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
    for (int k = 0; k < n; k++)
        if (!errs[k].empty()) {
            if (err) *err = errs[k];
            return false;
        }
    return !failed.load();
}

namespace {

void push_state(std::vector<double>& v, const double* x, const double* q, const double* vel) {
    const double rec[14] = {0.0, q[0], q[1], q[2], q[3], 0.0, 0.0, 0.0, x[0], x[1], x[2], vel[0], vel[1], vel[2]};
    v.insert(v.end(), rec, rec + 14);
}

void add_body(Scene& s, int mesh, const Mesh& m, const MassProps& mp, bool is_static, double density, double geo_eps,
              double mu, const double* x, const double* q, const double* v, float dt) {
    s.mesh.push_back(mesh);
    s.is_static.push_back(is_static ? 1 : 0);
    s.geo_eps.push_back(geo_eps);
    s.mu.push_back(mu);
    s.mass.push_back(density * mp.volume);
    for (int k = 0; k < 9; k++) s.inv_inertia.push_back((mp.unit_inertia_inv[k] * 1.0) / density);
    const double zero[3] = {0, 0, 0}, ident[4] = {1, 0, 0, 0};
    push_state(s.last, zero, ident, zero);  // Particle's last_state starts default-constructed
    push_state(s.cur, x, q, v);
    push_state(s.fut, zero, ident, zero);
    s.last_dt.push_back((double)dt);  // TimeStepSelectionStrategy::init
    s.sleep_steps.push_back(0);
    s.sleeping.push_back(0);
    double br = 0;
    float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
    for (int i = 0; i < m.nv(); i++) {
        const double* p = &m.V[3 * i];
        br = std::max(br, std::sqrt((p[0] * p[0] + p[1] * p[1]) + p[2] * p[2]));
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(lo[k], (float)p[k]);
            hi[k] = std::max(hi[k], (float)p[k]);
        }
    }
    s.bounding_radius.push_back(br);
    for (int k = 0; k < 3; k++) s.local_aabb.push_back(lo[k]);
    for (int k = 0; k < 3; k++) s.local_aabb.push_back(hi[k]);
}

// Uniform rotation (Shoemake, "Uniform random rotations", Graphics Gems III).
void random_quat(Pcg32& rng, double* q) {
    const double u1 = rng.uniform(), u2 = rng.uniform(), u3 = rng.uniform();
    const double a = std::sqrt(1.0 - u1), b = std::sqrt(u1);
    const double t2 = 6.283185307179586 * u2, t3 = 6.283185307179586 * u3;
    q[0] = b * m_cos(t3);  // w
    q[1] = a * m_sin(t2);
    q[2] = a * m_cos(t2);
    q[3] = b * m_sin(t3);
}

// Largest |coordinate| of the mesh's vertices rotated by q (w, x, y, z).
double max_axis_extent(const Mesh& m, const double* q) {
    const double w = q[0], x = q[1], y = q[2], z = q[3];
    const double R[9] = {1 - 2 * (y * y + z * z), 2 * (x * y - w * z),     2 * (x * z + w * y),
                         2 * (x * y + w * z),     1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                         2 * (x * z - w * y),     2 * (y * z + w * x),     1 - 2 * (x * x + y * y)};
    double e = 0.0;
    for (size_t v = 0; v + 2 < m.V.size(); v += 3)
        for (int r = 0; r < 3; r++)
            e = std::max(e, std::fabs(R[3 * r] * m.V[v] + R[3 * r + 1] * m.V[v + 1] + R[3 * r + 2] * m.V[v + 2]));
    return e;
}

// Standard normal by Marsaglia's polar method.
double normal(Pcg32& rng) {
    for (;;) {
        const double v1 = 2.0 * rng.uniform() - 1.0, v2 = 2.0 * rng.uniform() - 1.0;
        const double s = v1 * v1 + v2 * v2;
        if (s > 0.0 && s < 1.0) return v1 * std::sqrt(-2.0 * m_log(s) / s);
    }
}

}  // namespace

static bool file_exists(const std::string& path) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    std::fclose(f);
    return true;
}

// ------------------------------------------- scenes of the caller's meshes --
// Meshes are centred at their centre of mass (model/mesh.cpp:77) with the
// volume mass model of a closed surface or the surface model of a thin shell
// (model/mesh.cpp:93-130, thickness 0.01); bodies as Particle's constructor
// sets them up (model/particle.cpp:7-40); the trees are built at the end from
// one PCG32 stream seeded (42, 54), in mesh order.
int builder_add_mesh(SceneBuilder& b, const double* V, int nv, const int32_t* F, int nf, bool surface, double* com,
                     std::string* err) {
    if (b.finished || !V || !F || nv < 3 || nf < 1) {
        if (err) *err = b.finished ? "scene already finished" : "a mesh needs 3 vertices and a face";
        return -1;
    }
    Mesh m;
    m.V.assign(V, V + 3 * (size_t)nv);
    m.F.assign(F, F + 3 * (size_t)nf);
    for (int32_t f : m.F)
        if (f < 0 || f >= nv) {
            if (err) *err = "face index out of range";
            return -1;
        }
    for (double x : m.V)
        if (!std::isfinite(x)) {
            if (err) *err = "non-finite vertex";
            return -1;
        }
    MassProps mp = surface ? mass_surface(m, 0.01) : mass_volume(m);
    if (!(mp.volume > 0.0) || !std::isfinite(mp.volume)) {
        if (err) *err = surface ? "the surface has no area" : "the mesh encloses no volume (open or inside out)";
        return -1;
    }
    for (int k = 0; k < 3; k++) com[k] = mp.com[k];
    shift_vertices(m, mp.com);
    mp.com[0] = mp.com[1] = mp.com[2] = 0.0;
    b.meshes.push_back(m);
    b.mass.push_back(mp);
    return (int)b.meshes.size() - 1;
}

bool builder_add_body(SceneBuilder& b, int mesh, bool is_static, double density, double geo_eps, double mu,
                      const double* x, const double* q, const double* v, std::string* err) {
    if (b.finished || mesh < 0 || mesh >= (int)b.meshes.size() || !x || !q || !v) {
        if (err) *err = b.finished ? "scene already finished" : "unknown mesh or null argument";
        return false;
    }
    if (!(density > 0.0) || !(geo_eps >= 0.0) || !(mu >= 0.0) || !(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3] > 0.0)) {
        if (err) *err = "density must be positive, geo_eps and mu non-negative, the quaternion non-zero";
        return false;
    }
    add_body(b.s, mesh, b.meshes[mesh], b.mass[mesh], is_static, density, geo_eps, mu, x, q, v, b.s.opt_dt);
    return true;
}

bool builder_finish(SceneBuilder& b, std::string* err) {
    if (b.finished) return true;
    if (b.s.n_bodies() == 0) {
        if (err) *err = "a scene needs a body";
        return false;
    }
    Pcg32 tree_rng;
    tree_rng.seed(42u, 54u);  // common/cli_options.h:45
    for (const Mesh& m : b.meshes)
        if (scene_add_mesh(b.s, m, tree_rng, err) < 0) return false;
    b.finished = true;
    return true;
}

// The trees of every mesh, in creation order: loaded from o.tree_file when
// it exists (checked against the meshes' triangle counts), else built and,
// with a tree_file, saved there.  Meshes draw from one PCG32 stream in order,
// except configuration 5, whose per-body meshes (all but the box) draw from
// their own streams (42, 55 + k) and are built on all host cores.
bool finish_trees(Scene& s, const std::vector<Mesh>& meshes, const SceneOpts& o, Pcg32& tree_rng,
                  std::string* err) {
    TreeSet ts;
    const bool have_file = !o.tree_file.empty() && file_exists(o.tree_file);
    if (have_file) {
        if (!load_trees(o.tree_file.c_str(), ts, err)) return false;
        if (ts.mesh_ntris.size() != meshes.size()) {
            if (err) *err = o.tree_file + ": " + std::to_string(ts.mesh_ntris.size()) + " trees for " +
                            std::to_string(meshes.size()) + " meshes";
            return false;
        }
        for (size_t k = 0; k < meshes.size(); k++)
            if (ts.mesh_ntris[k] != meshes[k].nf()) {
                if (err) *err = o.tree_file + ": tree " + std::to_string(k) + " is for another mesh";
                return false;
            }
        s.mesh_node_off = ts.mesh_node_off;
        s.nodes = ts.nodes;
        s.ntris = ts.ntris;
        s.tris = ts.tris;
        s.eps = ts.eps;
        s.inner_eps = ts.inner_eps;
        s.mesh_ntris = ts.mesh_ntris;
        return true;
    }
    if (o.config == 5) {
        if (scene_add_mesh(s, meshes[0], tree_rng, err) < 0) return false;
        std::vector<Mesh> bodies(meshes.begin() + 1, meshes.end());
        std::vector<Tree> trees;
        if (!build_trees_parallel(bodies, 55u, trees, err)) return false;
        for (size_t k = 0; k < trees.size(); k++) scene_add_tree(s, trees[k], bodies[k].nf());
    } else {
        for (const Mesh& m : meshes)
            if (scene_add_mesh(s, m, tree_rng, err) < 0) return false;
    }
    if (!o.tree_file.empty()) {
        ts.mesh_node_off = s.mesh_node_off;
        ts.mesh_ntris = s.mesh_ntris;
        ts.nodes = s.nodes;
        ts.ntris = s.ntris;
        ts.tris = s.tris;
        ts.eps = s.eps;
        ts.inner_eps = s.inner_eps;
        if (!save_trees(ts, o.tree_file.c_str(), err)) return false;
    }
    return true;
}

bool make_scene(const SceneOpts& o, Scene& s, std::string* err) {
    s = Scene();
    Pcg32 rng;
    rng.seed(0x9E3779B97F4A7C15ULL ^ o.seed, 0xD2 + (uint64_t)o.config);
    Pcg32 tree_rng;
    tree_rng.seed(42u, 54u);  // common/cli_options.h:45
    std::vector<Mesh> meshes;  // in creation order; mesh id = index, trees built at the end
    const double density = 1000.0;
    int nx, ny, nz;
    double spacing, half, geo_eps, z0, sigma, mu, ground_w;
    float dt;
    if (o.config == 1) {  // 64 unit cubes
        nx = 4, ny = 4, nz = 4, spacing = 1.5, half = 0.5, sigma = 0.5, dt = 1.0f / 120.0f;
    } else if (o.config == 2) {  // 1,024 convex hulls of 64 points, radius 0.6
        nx = 8, ny = 8, nz = 16, spacing = 1.4, half = 0.6, sigma = 0.5, dt = 1.0f / 240.0f;
    } else if (o.config == 3) {  // mixed shapes (one scene of the batched configuration)
        nx = 8, ny = 8, nz = 4, spacing = 1.4, half = 0.6, sigma = 0.5, dt = 1.0f / 240.0f;
    } else if (o.config == 5) {  // noisy icospheres, subdivision 3
        nx = 16, ny = 16, nz = 64, spacing = 1.2, half = 0.5, sigma = 0.5, dt = 1.0f / 240.0f;
    } else {
        if (err) *err = "unknown scene config";
        return false;
    }
    if (o.nx > 0) nx = o.nx;
    if (o.ny > 0) ny = o.ny;
    if (o.nz > 0) nz = o.nz;
    if (o.spacing > 0) spacing = o.spacing;
    if (o.speed_sigma >= 0) sigma = o.speed_sigma;
    if (o.dt > 0) dt = o.dt;
    mu = o.mu > 0 ? o.mu : (o.config == 5 ? 0.6 : 0.5);
    geo_eps = 0.25 * half;
    // Lowest layer clears the largest half-diagonal plus the contact margin.
    z0 = (o.config == 1 ? 0.8660254037844386 * 2 * half : half) + geo_eps + 0.25;
    ground_w = std::max(100.0, 2.0 * spacing * std::max(nx, ny) + 20.0);
    s.opt_dt = dt;
    s.gravity_z = o.gravity_z;

    // Ground plane: static, surface mass model (model/mesh.cpp:93-130).  The
    // noisy-icosphere configuration pours its bodies into a static open box
    // (40 x 40 m floor, 20 m walls) instead, centred at its centre of mass
    // like every other mesh.
    const double zero3[3] = {0, 0, 0}, ident[4] = {1, 0, 0, 0};
    {
        Mesh g = o.config == 5 ? make_open_box(40.0, 20.0) : make_plane(ground_w);
        MassProps gmp = mass_surface(g, 0.01);
        double at[3] = {0, 0, 0};
        if (o.config == 5) {
            for (int k = 0; k < 3; k++) at[k] = gmp.com[k];
            shift_vertices(g, gmp.com);
            gmp.com[0] = gmp.com[1] = gmp.com[2] = 0.0;
        }
        const int gm = (int)meshes.size();
        meshes.push_back(g);
        add_body(s, gm, g, gmp, true, density, geo_eps, mu, at, ident, zero3, dt);
    }

    int shared_mesh = -1;
    Mesh shared;
    MassProps shared_mp;
    if (o.config == 1) {
        shared = make_cube(half);
        shared_mp = mass_volume(shared);
        shift_vertices(shared, shared_mp.com);
        shared_mp.com[0] = shared_mp.com[1] = shared_mp.com[2] = 0.0;
        shared_mesh = (int)meshes.size();
        meshes.push_back(shared);
    }
    constexpr int kMixHulls = 4;
    int mix_mesh[2 + kMixHulls];
    Mesh mix_geom[2 + kMixHulls];
    MassProps mix_mp[2 + kMixHulls];
    for (int k = 0; k < 2 + kMixHulls; k++) mix_mesh[k] = -1;
    const double cx = 0.5 * (nx - 1) * spacing, cy = 0.5 * (ny - 1) * spacing;
    int body = 0;
    for (int iz = 0; iz < nz; iz++)
        for (int iy = 0; iy < ny; iy++)
            for (int ix = 0; ix < nx; ix++, body++) {
                if (o.count > 0 && body >= o.count) break;
                Mesh m;
                MassProps mp;
                int mesh_id = shared_mesh;
                if (o.config != 1) {
                    int kind = o.config == 3 ? body % 3 : (o.config == 2 ? 1 : 2);
                    // The mixed configuration shares meshes as the reference
                    // shares MeshData: one cube, one icosphere and a pool of
                    // kMixHulls hulls per scene, each built on first use.
                    const int slot = kind == 0 ? 0 : (kind == 2 ? 1 : 2 + (body / 3) % kMixHulls);
                    if (o.config == 3 && mix_mesh[slot] >= 0) {
                        m = mix_geom[slot];
                        mp = mix_mp[slot];
                        mesh_id = mix_mesh[slot];
                    } else {
                        if (kind == 0)
                            m = make_cube(0.5);
                        else if (kind == 1)
                            m = make_hull(o.hull_points, half, rng);
                        else
                            m = make_icosphere(o.config == 5 ? 3 : 2, half, o.config == 5 ? 0.2 : 0.0, &rng);
                        mp = mass_volume(m);
                        shift_vertices(m, mp.com);
                        mp.com[0] = mp.com[1] = mp.com[2] = 0.0;
                        mesh_id = (int)meshes.size();
                        meshes.push_back(m);
                        if (o.config == 3) {
                            mix_mesh[slot] = mesh_id;
                            mix_geom[slot] = m;
                            mix_mp[slot] = mp;
                        }
                    }
                } else {
                    m = shared;
                    mp = shared_mp;
                }
                double x[3] = {ix * spacing - cx, iy * spacing - cy, z0 + iz * spacing};
                // Orientations are uniform, redrawn while the rotated mesh
                // reaches past half the spacing along a grid axis, where it
                // could start interpenetrating a neighbour (unit cubes at
                // 1.5 m spacing can: their half-diagonal is 0.87 m).
                double q[4];
                for (int attempt = 0;; attempt++) {
                    random_quat(rng, q);
                    if (attempt >= 1000 || max_axis_extent(m, q) <= 0.5 * spacing) break;
                }
                double v[3];
                for (int k = 0; k < 3; k++) v[k] = sigma * normal(rng);
                add_body(s, mesh_id, m, mp, false, density, geo_eps, mu, x, q, v, dt);
            }
    return finish_trees(s, meshes, o, tree_rng, err);
    return true;
}

}  // namespace d2g
