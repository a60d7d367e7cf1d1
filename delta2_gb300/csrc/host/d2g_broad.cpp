// Host broad phase: candidate body pairs for the narrow phase and CCD.
//
// Restates the reference's Embree-based broad phase
// (collision_detection/broad_phase_embree.cpp:87-116 bounds, :186-238
// filter, :266-289 driver) without Embree: float boxes per body (the mesh's
// local box through the float transform for static bodies; the bounding-
// sphere box at the last, current and future positions for moving bodies;
// both grown by geo_eps), an inclusive overlap test, then the swept
// bounding-sphere first-contact time within max(last_dt).  Embree reports
// pairs in a thread-dependent order; here they come in ascending (i, j).
#include <algorithm>
#include <limits>
#include <string>
#include <vector>

#include "../../../include/d2g.h"
#include "../d2g_geom.cuh"

namespace d2g {

void set_error(const std::string& msg);

namespace {
struct FBox {
    float lo[3], hi[3];
};

FBox bounds(const d2g_bodies* b, const float* aabb, int i) {
    FBox r;
    for (int k = 0; k < 3; k++) {
        r.lo[k] = std::numeric_limits<float>::infinity();
        r.hi[k] = -std::numeric_limits<float>::infinity();
    }
    auto extend = [&](const float* lo, const float* hi) {
        for (int k = 0; k < 3; k++) {
            r.lo[k] = std::min(r.lo[k], lo[k]);
            r.hi[k] = std::max(r.hi[k], hi[k]);
        }
    };
    if (b->is_static[i]) {
        const State s = load_state(b->cur + 14 * (size_t)i);
        double Td[16];
        transformation(s.q, s.x, Td);
        float T[16];
        for (int k = 0; k < 16; k++) T[k] = (float)Td[k];
        const float* a = aabb + 6 * (size_t)i;
        for (int xi = 0; xi < 2; xi++)
            for (int yi = 0; yi < 2; yi++)
                for (int zi = 0; zi < 2; zi++) {
                    const float v[3] = {xi ? a[3] : a[0], yi ? a[4] : a[1], zi ? a[5] : a[2]};
                    float o[4];
                    for (int rr = 0; rr < 4; rr++)
                        o[rr] = ((T[4 * rr] * v[0] + T[4 * rr + 1] * v[1]) + T[4 * rr + 2] * v[2]) + T[4 * rr + 3] * 1.0f;
                    const float w[3] = {o[0] / o[3], o[1] / o[3], o[2] / o[3]};
                    extend(w, w);
                }
    } else {
        const float br = (float)b->bounding_radius[i];
        const double* st[3] = {b->last + 14 * (size_t)i, b->cur + 14 * (size_t)i, b->fut + 14 * (size_t)i};
        for (int s = 0; s < 3; s++) {
            const float t[3] = {(float)st[s][8], (float)st[s][9], (float)st[s][10]};
            const float lo[3] = {-br + t[0], -br + t[1], -br + t[2]};
            const float hi[3] = {br + t[0], br + t[1], br + t[2]};
            extend(lo, hi);
        }
    }
    const float e = (float)b->geo_eps[i];
    for (int k = 0; k < 3; k++) {
        r.lo[k] = r.lo[k] - e;
        r.hi[k] = r.hi[k] + e;
    }
    return r;
}
}  // namespace

// Candidate pairs as (i, j), i < j, ascending.  Boxes are swept along x in
// order of their lower x bound (ties by index); every pair whose boxes
// overlap on all three axes is then filtered exactly as the all-pairs loop
// does, so the pair set is the same.  Returns D2G_ERR_STATE when a state
// interpolation is invalid (the reference throws there).
int broad_phase_pairs(const d2g_bodies* b, const float* local_aabb, std::vector<int32_t>& out) {
    out.clear();
    const int n = b->n;
    std::vector<FBox> box(n);
    std::vector<int32_t> order;
    order.reserve(n);
    for (int i = 0; i < n; i++) {
        box[i] = bounds(b, local_aabb, i);
        bool finite = true;
        for (int k = 0; k < 3; k++) finite = finite && box[i].lo[k] == box[i].lo[k] && box[i].hi[k] == box[i].hi[k];
        if (finite) order.push_back(i);  // a NaN box overlaps nothing
    }
    std::sort(order.begin(), order.end(), [&](int32_t x, int32_t y) {
        return box[x].lo[0] < box[y].lo[0] || (box[x].lo[0] == box[y].lo[0] && x < y);
    });
    std::vector<std::pair<int32_t, int32_t>> cand;
    for (size_t u = 0; u < order.size(); u++) {
        const int p = order[u];
        for (size_t v = u + 1; v < order.size(); v++) {
            const int q = order[v];
            if (box[q].lo[0] > box[p].hi[0]) break;
            const int i = p < q ? p : q, j = p < q ? q : p;
            if (b->is_static[i] && b->is_static[j]) continue;
            bool ov = true;
            for (int k = 0; k < 3; k++) ov = ov && box[i].lo[k] <= box[j].hi[k] && box[j].lo[k] <= box[i].hi[k];
            if (ov) cand.emplace_back(i, j);
        }
    }
    std::sort(cand.begin(), cand.end());
    for (const auto& c : cand) {
        const int i = c.first, j = c.second;
        State as = load_state(b->cur + 14 * (size_t)i), bs = load_state(b->cur + 14 * (size_t)j);
        if (!b->is_static[i] && !b->is_static[j]) {
            const State al = load_state(b->last + 14 * (size_t)i), bl = load_state(b->last + 14 * (size_t)j);
            State o;
            if (as.time < bs.time) {
                if (!interpolate(bs, bl, as.time, o)) {
                    set_error("invalid state interpolation in the broad phase (bodies " + std::to_string(i) + ", " +
                              std::to_string(j) + ")");
                    return D2G_ERR_STATE;
                }
                bs = o;
            } else {
                if (!interpolate(as, al, bs.time, o)) {
                    set_error("invalid state interpolation in the broad phase (bodies " + std::to_string(i) + ", " +
                              std::to_string(j) + ")");
                    return D2G_ERR_STATE;
                }
                as = o;
            }
        }
        const double t = sphere_sphere_first_intersect(as.x, as.v, b->bounding_radius[i] + b->geo_eps[i], bs.x, bs.v,
                                                       b->bounding_radius[j] + b->geo_eps[j]);
        if (t >= 0.0 && t < dmax(b->last_dt[i], b->last_dt[j])) {
            out.push_back(i);
            out.push_back(j);
        }
    }
    return D2G_OK;
}
}  // namespace d2g

extern "C" int d2g_broad_phase(const d2g_bodies* b, const float* local_aabb, int32_t* pairs, int32_t capacity,
                               int32_t* n_pairs) {
    using namespace d2g;
    if (!b || !local_aabb || !n_pairs || b->n < 0 || !b->bounding_radius) {
        set_error("invalid broad-phase arguments");
        return D2G_ERR_INVALID;
    }
    std::vector<int32_t> out;
    const int rc = broad_phase_pairs(b, local_aabb, out);
    if (rc) return rc;
    const int cnt = (int)(out.size() / 2);
    *n_pairs = cnt;
    if (pairs)
        for (int k = 0; k < cnt && k < capacity; k++) {
            pairs[2 * k] = out[2 * k];
            pairs[2 * k + 1] = out[2 * k + 1];
        }
    if (pairs && cnt > capacity) {
        set_error("broad-phase pair capacity too small");
        return D2G_CAPACITY;
    }
    return D2G_OK;
}
