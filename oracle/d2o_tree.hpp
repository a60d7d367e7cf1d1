// Oracle (test infrastructure only): the surrogate-tree construction of the
// reference, restated in plain C++ so that the product's host builder can be
// checked node for node against it.  Follows
//   model/surrogate_tree.cpp:39-112      SurrogateTree::buildSurrogateTreeKMean
//   model/construct_surrogate_tree.h:8-168  divideAndFit
//   model/construct_surrogate_tree.h:172-185 calcEpss
//   model/fit_surrogate_triangle.h:247-299  selectSurrogateTriangle
//   common/triangle.h:21-23, 280-471     Triangle::area, Triangle::distToPoint
//   common/pcg_basic.cpp:42-110          PCG32 (O'Neill's published generator)
// and the declared evaluation order of d2o_geom.hpp (left-to-right sums, no
// contraction).  Two places where the reference is undefined are declared:
//   * selectSurrogateTriangle keeps its caller's default-constructed
//     (uninitialised) triangle when every random draw is degenerate, because
//     its enumeration fallback tests `area() == -1`, which never holds; here
//     the enumeration it intends runs (first triple a < b < c with positive
//     area);
//   * divideAndFit leaves `best_group` uninitialised when no distance is
//     below infinity (NaN geometry); here it stays group 0.
#pragma once
#include <cmath>
#include <cstdint>
#include <deque>
#include <limits>
#include <stdexcept>
#include <tuple>
#include <vector>

#include "d2o_geom.hpp"

namespace d2o {

// ------------------------------------------------------------- PCG32 ------
// common/pcg_basic.cpp:60-67 pcg32_random_r and :79-110 pcg32_boundedrand_r.
struct Pcg32 {
    uint64_t state = 0, inc = 1;
    uint32_t next() {
        const uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        const uint32_t x = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        const uint32_t r = (uint32_t)(old >> 59u);
        return (x >> r) | (x << ((0u - r) & 31u));
    }
    // uniform in [0, bound): draws below (2^32 - bound) mod bound are rejected
    uint32_t below(uint32_t bound) {
        const uint32_t cut = (0u - bound) % bound;
        for (;;) {
            const uint32_t r = next();
            if (r >= cut) return r % bound;
        }
    }
};

// ------------------------------------------- point-triangle distance ------
// common/triangle.h:280-471 Triangle::distToPoint: the closest point by the
// seven-region classification of the (s, t) parameter plane (Eberly's method).
inline double tri_point_dist(const Tri& T, V3 X) {
    const V3 AX = X - T.A, AB = T.B - T.A, AC = T.C - T.A;
    const double a00 = dot(AB, AB), a01 = dot(AB, AC), a11 = dot(AC, AC);
    const double b0 = -dot(AX, AB), b1 = -dot(AX, AC);
    const double det = a00 * a11 - a01 * a01;
    double s = a01 * b1 - a11 * b0;
    double t = a01 * b0 - a00 * b1;
    // the parameter on the edge B-C from the projected numerator, or a vertex
    auto on_bc = [&](double num, double& first, double& second) {
        const double den = (a00 - 2.0 * a01) + a11;
        if (num >= den) {
            first = 1.0;
            second = 0.0;
        } else {
            first = num / den;
            second = 1.0 - first;
        }
    };
    auto on_ac = [&](double& tt) {  // s = 0: the edge A-C
        if (b1 >= 0.0)
            tt = 0.0;
        else if (-b1 >= a11)
            tt = 1.0;
        else
            tt = -b1 / a11;
    };
    auto on_ab = [&](double& ss) {  // t = 0: the edge A-B
        if (b0 >= 0.0)
            ss = 0.0;
        else if (-b0 >= a00)
            ss = 1.0;
        else
            ss = -b0 / a00;
    };
    if (s + t <= det) {
        if (s < 0.0) {
            if (t < 0.0) {  // below both edges at A
                if (b0 < 0.0) {
                    t = 0.0;
                    if (-b0 >= a00)
                        s = 1.0;
                    else
                        s = -b0 / a00;
                } else {
                    s = 0.0;
                    on_ac(t);
                }
            } else {
                s = 0.0;
                on_ac(t);
            }
        } else if (t < 0.0) {
            t = 0.0;
            on_ab(s);
        } else {  // inside
            const double inv = 1.0 / det;
            s *= inv;
            t *= inv;
        }
    } else {
        if (s < 0.0) {
            const double p = a01 + b0, q = a11 + b1;
            if (q > p) {
                on_bc(q - p, s, t);
            } else {
                s = 0.0;
                if (q <= 0.0)
                    t = 1.0;
                else if (b1 >= 0.0)
                    t = 0.0;
                else
                    t = -b1 / a11;
            }
        } else if (t < 0.0) {
            const double p = a01 + b1, q = a00 + b0;
            if (q > p) {
                on_bc(q - p, t, s);
            } else {
                t = 0.0;
                if (q <= 0.0)
                    s = 1.0;
                else if (b0 >= 0.0)
                    s = 0.0;
                else
                    s = -b0 / a00;
            }
        } else {
            const double num = ((a11 + b1) - a01) - b0;
            if (num <= 0.0) {
                s = 0.0;
                t = 1.0;
            } else {
                on_bc(num, s, t);
            }
        }
    }
    const V3 closest = (T.A + s * AB) + t * AC;
    return norm(X - closest);
}

// --------------------------------------------- selectSurrogateTriangle ----
// model/fit_surrogate_triangle.h:247-299: the largest-area triangle among
// floor(log2(n) * 10) random vertex triples (n = 3 x group triangles), or the
// only triple when n == 3.  Returns false when no triangle has positive area.
inline bool surrogate_of(const std::vector<V3>& pts, Pcg32& rng, Tri& out) {
    const int n = (int)pts.size();
    Tri best{V3{0, 0, 0}, V3{0, 0, 0}, V3{0, 0, 0}};
    if (n > 3) {
        double best_area = -1.0;
        const int attempts = (int)(std::log2((double)n) * 10);
        for (int k = 0; k < attempts; k++) {
            const int i = (int)rng.below((uint32_t)n);
            const int j = (int)rng.below((uint32_t)n);
            const int l = (int)rng.below((uint32_t)n);
            const Tri trial{pts[i], pts[j], pts[l]};
            const double area = tri_area(trial);
            if (area > best_area && area > 0.0) {
                best = trial;
                best_area = area;
            }
        }
        if (!(tri_area(best) > 0.0)) {  // the intended enumeration (declared above)
            for (int i = 0; i < n; i++)
                for (int j = i + 1; j < n; j++)
                    for (int l = j + 1; l < n; l++) {
                        const Tri trial{pts[i], pts[j], pts[l]};
                        if (tri_area(trial) > 0.0) {
                            out = trial;
                            return true;
                        }
                    }
        }
    } else {
        best = Tri{pts[0], pts[1], pts[2]};
    }
    out = best;
    return tri_area(best) > 0.0;
}

inline std::vector<V3> vertices_of(const std::vector<Tri>& tris, const std::vector<int>& ids) {
    std::vector<V3> pts;
    pts.reserve(3 * ids.size());
    for (int id : ids) {
        pts.push_back(tris[id].A);
        pts.push_back(tris[id].B);
        pts.push_back(tris[id].C);
    }
    return pts;
}

inline Tri surrogate_or_throw(const std::vector<Tri>& tris, const std::vector<int>& ids, Pcg32& rng) {
    Tri s;
    if (!surrogate_of(vertices_of(tris, ids), rng, s)) throw std::runtime_error("No valid surrogate triangle was found");
    return s;
}

// ------------------------------------------------------- divideAndFit -----
// model/construct_surrogate_tree.h:8-168.  Groups start from the MESH's first
// `k` triangles (not the group's), 20 rounds of: assign each triangle to the
// group triangle nearest to its farthest vertex (first of equals), refit every
// non-empty group; with `force`, empty groups are then filled by splitting the
// largest group (a recursive unforced divideAndFit over it), and failing that
// by moving single triangles out of the largest group.
inline void divide_and_fit(const std::vector<Tri>& tris, const std::vector<int>& ids, int k, bool force, Pcg32& rng,
                           std::vector<Tri>& gtri, std::vector<std::vector<int>>& gids) {
    if (k > (int)ids.size()) throw std::invalid_argument("There must be more triangles than branches");
    gtri.assign(k, Tri{});
    gids.assign(k, std::vector<int>());
    for (int g = 0; g < k; g++) gtri[g] = tris[g];
    auto largest_and_empty = [&](int& largest, std::vector<int>& empty) {
        size_t most = 0;
        largest = 0;
        empty.clear();
        for (int g = 0; g < k; g++) {
            if (gids[g].size() > most) {
                most = gids[g].size();
                largest = g;
            }
            if (gids[g].empty()) empty.push_back(g);
        }
    };
    for (int round = 0; round < 20; round++) {
        for (auto& v : gids) v.clear();
        for (int id : ids) {
            double best = std::numeric_limits<double>::infinity();
            int pick = 0;
            for (int g = 0; g < k; g++) {
                const double da = tri_point_dist(gtri[g], tris[id].A);
                const double db = tri_point_dist(gtri[g], tris[id].B);
                const double dc = tri_point_dist(gtri[g], tris[id].C);
                const double far = dmax(dmax(da, db), dc);
                if (far < best) {
                    pick = g;
                    best = far;
                }
            }
            gids[pick].push_back(id);
        }
        for (int g = 0; g < k; g++)
            if (!gids[g].empty()) gtri[g] = surrogate_or_throw(tris, gids[g], rng);
        if (!force) continue;
        bool improving = true, enough = false;
        while (improving && !enough) {
            int largest;
            std::vector<int> empty;
            largest_and_empty(largest, empty);
            if (empty.empty()) {
                enough = true;
                break;
            }
            const int parts = (int)std::min(gids[largest].size(), empty.size() + 1);
            std::vector<Tri> sub_tri;
            std::vector<std::vector<int>> sub_ids;
            divide_and_fit(tris, gids[largest], parts, false, rng, sub_tri, sub_ids);
            int filled = 0;
            for (int s = 0; s < (int)sub_tri.size(); s++) {
                const int dst = s == 0 ? largest : empty[s - 1];
                if (!sub_ids[s].empty()) {
                    filled++;
                    gids[dst] = sub_ids[s];
                    gtri[dst] = sub_tri[s];
                }
            }
            improving = filled > 1;
        }
        if (!enough) {
            // one triangle per empty group, taken from the back of the largest
            // group while it keeps more than one (the bound is re-evaluated
            // as the group shrinks, as the reference's loop condition is);
            // the pass that finds no empty group still refits the largest
            // group before the loop ends (a do-while)
            std::vector<int> empty;
            do {
                int largest;
                largest_and_empty(largest, empty);
                for (size_t z = 0; z < std::min(empty.size(), gids[largest].size() - 1); z++) {
                    const int id = gids[largest].back();
                    gids[empty[z]].push_back(id);
                    gids[largest].pop_back();
                    gtri[empty[z]] = tris[id];
                }
                gtri[largest] = surrogate_or_throw(tris, gids[largest], rng);
            } while (!empty.empty());
        }
    }
}

// model/construct_surrogate_tree.h:172-185 calcEpss: the smallest and largest
// distance from the surrogate to the group's triangle vertices.
inline void group_eps(const Tri& s, const std::vector<Tri>& tris, const std::vector<int>& ids, double& inner,
                      double& outer) {
    inner = std::numeric_limits<double>::infinity();
    outer = 0.0;
    for (int id : ids) {
        const double a = tri_point_dist(s, tris[id].A);
        const double b = tri_point_dist(s, tris[id].B);
        const double c = tri_point_dist(s, tris[id].C);
        inner = dmin(inner, dmin(a, dmin(b, c)));
        outer = dmax(outer, dmax(a, dmax(b, c)));
    }
}

// ------------------------------------------------------- tree layout ------
// The flattened tree in the library's layout: per node (child_first local to
// the tree or -1, num_children, is_inner, depth), triangle count, up to 8
// triangles of 9 doubles, eps[8], inner_eps[8].
struct FlatTree {
    std::vector<int32_t> nodes, ntris;
    std::vector<double> tris, eps, inner_eps;
    int size() const { return (int)ntris.size(); }
};

// model/surrogate_tree.cpp:39-112: breadth-first over groups (FIFO queue of
// (triangle ids, depth, parent)); a group of fewer than 8 triangles is a leaf
// holding them with eps 0, any other is split by divideAndFit into 8
// surrogates whose groups are queued in order; a parent's first child is the
// first of its groups to leave the queue, so children are contiguous.
inline FlatTree build_surrogate_tree(const std::vector<Tri>& tris, Pcg32& rng) {
    FlatTree T;
    std::deque<std::tuple<std::vector<int>, int, int>> queue;
    std::vector<int> all(tris.size());
    for (size_t i = 0; i < tris.size(); i++) all[i] = (int)i;
    queue.emplace_back(all, 0, -1);
    while (!queue.empty()) {
        auto [ids, depth, parent] = queue.front();
        queue.pop_front();
        const int id = T.size();
        T.ntris.push_back(0);
        T.tris.resize(72 * (size_t)(id + 1), 0.0);
        T.eps.resize(8 * (size_t)(id + 1), 0.0);
        T.inner_eps.resize(8 * (size_t)(id + 1), 0.0);
        auto put = [&](int slot, const Tri& t) {
            const V3 v[3] = {t.A, t.B, t.C};
            for (int q = 0; q < 3; q++) {
                T.tris[72 * (size_t)id + 9 * slot + 3 * q] = v[q].x;
                T.tris[72 * (size_t)id + 9 * slot + 3 * q + 1] = v[q].y;
                T.tris[72 * (size_t)id + 9 * slot + 3 * q + 2] = v[q].z;
            }
        };
        if (ids.size() < 8) {
            for (size_t i = 0; i < ids.size(); i++) put((int)i, tris[ids[i]]);
            T.ntris[id] = (int)ids.size();
            T.nodes.insert(T.nodes.end(), {-1, 0, 0, depth});
        } else {
            std::vector<Tri> gtri;
            std::vector<std::vector<int>> gids;
            divide_and_fit(tris, ids, 8, true, rng, gtri, gids);
            for (int g = 0; g < (int)gtri.size(); g++) {
                double inner, outer;
                group_eps(gtri[g], tris, gids[g], inner, outer);
                put(g, gtri[g]);
                T.eps[8 * (size_t)id + g] = outer;
                T.inner_eps[8 * (size_t)id + g] = inner;
            }
            T.ntris[id] = (int)gtri.size();
            T.nodes.insert(T.nodes.end(), {-1, (int32_t)gtri.size(), 1, depth});
            for (int g = 0; g < (int)gtri.size(); g++) queue.emplace_back(gids[g], depth + 1, id);
        }
        if (parent >= 0 && T.nodes[4 * (size_t)parent] == -1) T.nodes[4 * (size_t)parent] = id;
    }
    return T;
}

}  // namespace d2o
