// Broad phase and cluster separation on the GPU.
//
// Broad phase: restates broadPhaseEmbree(ParticleHandler&)
// (collision_detection/broad_phase_embree.cpp:87-116 bounds, :186-238
// filter, :266-289 driver) as a sort-and-sweep instead of Embree's BVH:
//   1. one thread per body: the float box (the mesh's local box through the
//      float transform for static bodies; the bounding-sphere box at the
//      last, current and future positions for moving ones; grown by
//      geo_eps), with the same float operations, in the same order, as the
//      host restatement (csrc/host/d2g_broad.cpp);
//   2. a stable radix sort of the boxes by lower x (ties by index);
//   3. one thread per sorted box sweeps forward while the next lower x is
//      within its upper x and keeps the pairs whose boxes overlap on all
//      three axes (inclusive, as Embree's box test) and are not both static;
//   4. one thread per candidate: the reference's swept-sphere filter in FP64
//      (interpolate the later body back to the earlier body's time, first
//      contact within max(last_dt));
//   5. the surviving pairs sorted ascending by (i, j).
// The pair set is the all-pairs set; Embree's thread-dependent order is
// replaced by ascending (i, j), as on the host.
//
// Cluster separation: restates separateCollisionClusters
// (collision_detection/separate_clusters.cpp:355-459).  Components over
// moving-moving pairs by a lock-free union-find whose roots are the
// components' smallest indices; clusters are numbered in order of those
// indices, which is the breadth-first labelling from the lowest unlabelled
// index.  A cluster's particles are its members ascending, then the static
// bodies it interacts with in order of their first interaction; its
// interactions are the broad-phase pairs in order.  Minimum current time,
// minimum last_dt and the sleeping flag per cluster come from one thread per
// cluster over its members in order.
#include <cub/cub.cuh>

#include "d2g_geom.cuh"
#include "d2g_internal.hpp"

namespace d2g {

namespace {

constexpr int kBlock = 128;
inline int nblocks(long long n, int b = kBlock) { return (int)((n + b - 1) / b); }

#define RC(x)                          \
    do {                               \
        if (int rc_ = (x)) return rc_; \
    } while (0)
#define BLAUNCH(kern, n, ...)                                          \
    do {                                                               \
        kern<<<nblocks(n), kBlock, 0, ctx->stream>>>(__VA_ARGS__);     \
        ctx->eng.launches++;                                           \
    } while (0)

__device__ __forceinline__ float fmin_ref(float a, float b) { return (b < a) ? b : a; }  // std::min
__device__ __forceinline__ float fmax_ref(float a, float b) { return (a < b) ? b : a; }  // std::max

// Float box of body i (broad_phase_embree.cpp:87-116; model/mesh.cpp:137-155).
__global__ void k_bp_boxes(int n, const uint8_t* __restrict__ is_static, const double* __restrict__ last,
                           const double* __restrict__ cur, const double* __restrict__ fut,
                           const double* __restrict__ radius, const double* __restrict__ geo_eps,
                           const float* __restrict__ aabb, const int32_t* __restrict__ scene,
                           float* __restrict__ box, unsigned long long* __restrict__ key, int32_t* __restrict__ idx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float lo[3], hi[3];
    for (int k = 0; k < 3; k++) {
        lo[k] = __int_as_float(0x7f800000);
        hi[k] = -__int_as_float(0x7f800000);
    }
    if (is_static[i]) {
        const State s = load_state(cur + 14 * (size_t)i);
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
                    for (int r = 0; r < 4; r++)
                        o[r] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(T[4 * r], v[0]), __fmul_rn(T[4 * r + 1], v[1])),
                                                   __fmul_rn(T[4 * r + 2], v[2])),
                                         __fmul_rn(T[4 * r + 3], 1.0f));
                    for (int k = 0; k < 3; k++) {
                        const float w = __fdiv_rn(o[k], o[3]);
                        lo[k] = fmin_ref(lo[k], w);
                        hi[k] = fmax_ref(hi[k], w);
                    }
                }
    } else {
        const float br = (float)radius[i];
        const double* st[3] = {last + 14 * (size_t)i, cur + 14 * (size_t)i, fut + 14 * (size_t)i};
        for (int s = 0; s < 3; s++)
            for (int k = 0; k < 3; k++) {
                const float t = (float)st[s][8 + k];
                lo[k] = fmin_ref(lo[k], __fadd_rn(-br, t));
                hi[k] = fmax_ref(hi[k], __fadd_rn(br, t));
            }
    }
    const float e = (float)geo_eps[i];
    bool finite = true;
    for (int k = 0; k < 3; k++) {
        lo[k] = __fsub_rn(lo[k], e);
        hi[k] = __fadd_rn(hi[k], e);
        box[6 * (size_t)i + k] = lo[k];
        box[6 * (size_t)i + 3 + k] = hi[k];
        finite = finite && lo[k] == lo[k] && hi[k] == hi[k];
    }
    // scene, then an order-preserving key of lower x (NaN boxes sort last in
    // their scene and overlap nothing)
    const uint32_t u = __float_as_uint(lo[0]);
    const uint32_t xk = finite ? ((u & 0x80000000u) ? ~u : (u | 0x80000000u)) : 0xffffffffu;
    key[i] = ((unsigned long long)(uint32_t)scene[i] << 32) | xk;
    idx[i] = finite ? i : -1 - i;
}

__device__ __forceinline__ bool boxes_overlap(const float* a, const float* b) {
    bool ov = true;
    for (int k = 0; k < 3; k++) ov = ov && a[k] <= b[3 + k] && b[k] <= a[3 + k];
    return ov;
}

// Sweep along x over the sorted boxes, as ranges: the boxes that can overlap
// sorted box u are the positions after u, in its scene, among the finite boxes,
// up to the first whose lower x exceeds u's upper x (lower x is sorted, so
// both ends are binary searches).  r[u] = the range's length.
__global__ void k_bp_range(int n, const int32_t* __restrict__ order, const float* __restrict__ box,
                           const unsigned long long* __restrict__ key_s, long long* __restrict__ r) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= n) return;
    const int p = order[u];
    if (p < 0) {  // a NaN box overlaps nothing
        r[u] = 0;
        return;
    }
    const unsigned long long lim = key_s[u] | 0xffffffffULL;  // the NaN-box key of this scene
    int lo = u + 1, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (key_s[mid] < lim)
            lo = mid + 1;
        else
            hi = mid;
    }
    const float hx = box[6 * (size_t)p + 3];
    hi = lo;
    lo = u + 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (box[6 * (size_t)order[mid]] > hx)
            hi = mid;
        else
            lo = mid + 1;
    }
    r[u] = lo - u - 1;
}

// The reference's swept-sphere filter of one candidate (i < j)
// (broad_phase_embree.cpp:196-216): 1 keep, 0 drop, -1 invalid interpolation.
__device__ int bp_filter_one(int i, int j, const uint8_t* __restrict__ is_static, const double* __restrict__ last,
                             const double* __restrict__ cur, const double* __restrict__ radius,
                             const double* __restrict__ geo_eps, const double* __restrict__ last_dt) {
    State as = load_state(cur + 14 * (size_t)i), bs = load_state(cur + 14 * (size_t)j);
    if (!is_static[i] && !is_static[j]) {
        State o;
        if (as.time < bs.time) {
            if (!interpolate(bs, load_state(last + 14 * (size_t)j), as.time, o)) return -1;
            bs = o;
        } else {
            if (!interpolate(as, load_state(last + 14 * (size_t)i), bs.time, o)) return -1;
            as = o;
        }
    }
    const double t =
        sphere_sphere_first_intersect(as.x, as.v, radius[i] + geo_eps[i], bs.x, bs.v, radius[j] + geo_eps[j]);
    return (t >= 0.0 && t < dmax(last_dt[i], last_dt[j])) ? 1 : 0;
}

// One thread per range element (grid-stride over the total read from
// roff[n]): the box test of the two sorted positions, the static-static skip
// and the swept-sphere filter; kept pairs append their key (i << 32 | j) at a
// warp-aggregated counter (the keys are sorted afterwards, so the append
// order does not matter).  Keys beyond cap are counted but not written.
__global__ void k_bp_pairs(int n, const long long* __restrict__ roff, const int32_t* __restrict__ order,
                           const float* __restrict__ box, const uint8_t* __restrict__ is_static,
                           const double* __restrict__ last, const double* __restrict__ cur,
                           const double* __restrict__ radius, const double* __restrict__ geo_eps,
                           const double* __restrict__ last_dt, unsigned long long* __restrict__ out, int cap,
                           int32_t* __restrict__ count, int32_t* __restrict__ err) {
    const long long total = roff[n];
    const int lane = threadIdx.x & 31;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < total;
         base += (long long)gridDim.x * blockDim.x) {
        const long long k = base + threadIdx.x;
        bool keep = false;
        unsigned long long key = 0;
        if (k < total) {
            int lo = 0, hi = n;  // roff[lo] <= k < roff[hi]
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (roff[mid] <= k)
                    lo = mid;
                else
                    hi = mid;
            }
            const int p = order[lo], q = order[lo + 1 + (int)(k - roff[lo])];
            if (!(is_static[p] && is_static[q]) && boxes_overlap(box + 6 * (size_t)p, box + 6 * (size_t)q)) {
                const int i = p < q ? p : q, j = p < q ? q : p;
                const int f = bp_filter_one(i, j, is_static, last, cur, radius, geo_eps, last_dt);
                if (f < 0) atomicExch(err, 1);
                keep = f > 0;
                key = ((unsigned long long)(uint32_t)i << 32) | (uint32_t)j;
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);  // base is uniform over the block
        if (m) {
            const int lead = __ffs(m) - 1;
            int pos = 0;
            if (lane == lead) pos = atomicAdd(count, __popc(m));
            pos = __shfl_sync(0xffffffffu, pos, lead) + __popc(m & ((1u << lane) - 1u));
            if (keep && pos < cap) out[pos] = key;
        }
    }
}

__global__ void k_bp_unpack(int n, const unsigned long long* __restrict__ key, int32_t* __restrict__ pairs) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    pairs[2 * (size_t)k] = (int32_t)(key[k] >> 32);
    pairs[2 * (size_t)k + 1] = (int32_t)(key[k] & 0xffffffffu);
}

// ------------------------------------------------------------ clustering ---
__device__ __forceinline__ int uf_find(const int32_t* parent, int x) {
    for (int it = 0; it < (1 << 24); it++) {  // chains are short; the bound only guards bad input
        const int p = ((volatile const int32_t*)parent)[x];
        if (p == x) return x;
        x = p;
    }
    return x;
}

__global__ void k_uf_init(int n, int32_t* __restrict__ parent) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) parent[i] = i;
}

// Union of the two moving bodies of each pair: the larger root is hooked under
// the smaller, so every component's root is its smallest index.
__global__ void k_uf_union(int n_pairs, const int32_t* __restrict__ pairs, const uint8_t* __restrict__ is_static,
                           int32_t* __restrict__ parent, int32_t* __restrict__ err) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_pairs) return;
    int a = pairs[2 * (size_t)k], b = pairs[2 * (size_t)k + 1];
    if (is_static[a] || is_static[b]) return;
    for (int it = 0; it < (1 << 20); it++) {  // retries only when another thread hooked a root first
        a = uf_find(parent, a);
        b = uf_find(parent, b);
        if (a == b) return;
        if (a > b) {
            const int t = a;
            a = b;
            b = t;
        }
        if (atomicCAS(&parent[b], b, a) == b) return;
    }
    atomicExch(err, 2);
}

// Root of every body; a moving root starts a cluster.
__global__ void k_uf_roots(int n, int32_t* __restrict__ parent, const uint8_t* __restrict__ is_static,
                           int32_t* __restrict__ is_root) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int r = uf_find(parent, i);
    is_root[i] = (r == i && !is_static[i]) ? 1 : 0;
    parent[i] = r;  // every body now points at its root (roots are unchanged)
}

// Cluster id of every moving body (-1 for static bodies): the number of
// moving roots with a smaller index than its root.
__global__ void k_cl_ids(int n, const int32_t* __restrict__ root, const int32_t* __restrict__ root_off,
                         const uint8_t* __restrict__ is_static, int32_t* __restrict__ cid) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) cid[i] = is_static[i] ? -1 : root_off[root[i]];
}

// Per pair: its cluster (of the moving body) for the interaction lists; for
// a static-moving pair the (cluster, static body) key with the pair position.
__global__ void k_cl_pair_keys(int n_pairs, const int32_t* __restrict__ pairs, const uint8_t* __restrict__ is_static,
                               const int32_t* __restrict__ cid, int32_t* __restrict__ pair_cid,
                               unsigned long long* __restrict__ st_key, int32_t* __restrict__ st_pos) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_pairs) return;
    const int a = pairs[2 * (size_t)k], b = pairs[2 * (size_t)k + 1];
    const bool sa = is_static[a], sb = is_static[b];
    const int c = sa ? cid[b] : cid[a];
    pair_cid[k] = c;
    // dynamic-dynamic pairs get a key above every static entry
    st_key[k] = (sa != sb) ? (((unsigned long long)(uint32_t)c << 32) | (uint32_t)(sa ? a : b)) : ~0ULL;
    st_pos[k] = k;
}

// First entry of each (cluster, static body) group after the stable sort by
// key: its first interaction.  Flags them and re-keys by (cluster, position).
__global__ void k_cl_static_first(int n, const unsigned long long* __restrict__ key,
                                  const int32_t* __restrict__ pos, int32_t* __restrict__ flag,
                                  unsigned long long* __restrict__ key2, int32_t* __restrict__ body) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const bool first = key[k] != ~0ULL && (k == 0 || key[k - 1] != key[k]);
    flag[k] = first ? 1 : 0;
    key2[k] = ((key[k] >> 32) << 32) | (uint32_t)pos[k];
    body[k] = (int32_t)(key[k] & 0xffffffffu);
}

__global__ void k_cl_compact2(int n, const int32_t* __restrict__ flag, const int32_t* __restrict__ off,
                              const unsigned long long* __restrict__ key2, const int32_t* __restrict__ body,
                              unsigned long long* __restrict__ okey, int32_t* __restrict__ obody) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n && flag[k]) {
        okey[off[k]] = key2[k];
        obody[off[k]] = body[k];
    }
}

// Counts of moving members (from the member sort) and static members per cluster.
__global__ void k_cl_count(int n_members, const int32_t* __restrict__ member_cid, int n_static,
                           const unsigned long long* __restrict__ static_key, int32_t* __restrict__ n_dyn,
                           int32_t* __restrict__ n_stat) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n_members) atomicAdd(&n_dyn[member_cid[k]], 1);
    if (k < n_static) atomicAdd(&n_stat[(int)(static_key[k] >> 32)], 1);
}

// Particles of each cluster: moving members ascending (the members are
// sorted by cluster, stable in index), then its static bodies in order.
__global__ void k_cl_fill(int n_members, const int32_t* __restrict__ member_cid, const int32_t* __restrict__ member,
                          const int32_t* __restrict__ dyn_off, int n_static,
                          const unsigned long long* __restrict__ static_key, const int32_t* __restrict__ static_body,
                          const int32_t* __restrict__ static_off, const int32_t* __restrict__ part_off,
                          const int32_t* __restrict__ n_dyn, int32_t* __restrict__ parts) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n_members) {
        const int c = member_cid[k];
        parts[part_off[c] + (k - dyn_off[c])] = member[k];
    }
    if (k < n_static) {
        const int c = (int)(static_key[k] >> 32);
        parts[part_off[c] + n_dyn[c] + (k - static_off[c])] = static_body[k];
    }
}

// Minimum current time, minimum last_dt and the sleeping flag of each
// cluster over its moving members in order (separate_clusters.cpp:386-395),
// one warp per cluster.  The reference's running minimum from +inf keeps the
// first of equal values and never takes a NaN; that is the leftmost minimum
// over (value, member position), reduced with shuffles.
__device__ __forceinline__ void lmin(double& v, int& i, double ov, int oi) {
    if (ov < v || (ov == v && oi < i)) {
        v = ov;
        i = oi;
    }
}
__global__ void k_cl_meta(int n_clusters, const int32_t* __restrict__ part_off, const int32_t* __restrict__ n_dyn,
                          const int32_t* __restrict__ parts, const double* __restrict__ cur,
                          const double* __restrict__ last_dt, const uint8_t* __restrict__ sleeping,
                          double* __restrict__ mct, double* __restrict__ step, int32_t* __restrict__ sleep) {
    const int c = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (c >= n_clusters) return;  // uniform per warp
    const double inf = __longlong_as_double(0x7ff0000000000000LL);
    double m = inf, st = inf;
    int mi = 0x7fffffff, si = 0x7fffffff;
    bool awake = false;
    const int i0 = part_off[c], i1 = part_off[c] + n_dyn[c];
    for (int i = i0 + lane; i < i1; i += 32) {
        const int g = parts[i];
        const double t = cur[14 * (size_t)g], l = last_dt[g];
        if (t < m) {
            m = t;
            mi = i;
        }
        if (l < st) {
            st = l;
            si = i;
        }
        if (!sleeping[g]) awake = true;
    }
    for (int o = 16; o > 0; o >>= 1) {
        lmin(m, mi, __shfl_down_sync(0xffffffffu, m, o), __shfl_down_sync(0xffffffffu, mi, o));
        lmin(st, si, __shfl_down_sync(0xffffffffu, st, o), __shfl_down_sync(0xffffffffu, si, o));
    }
    const bool any_awake = __any_sync(0xffffffffu, awake);
    if (lane == 0) {
        mct[c] = m;
        step[c] = st;
        sleep[c] = any_awake ? 0 : 1;
    }
}

// separate_clusters.cpp:445-456: every moving body rolled back to its
// cluster's minimum current time.
__global__ void k_cl_rollback(int n, const int32_t* __restrict__ cid, const double* __restrict__ mct,
                              const double* __restrict__ last, double* __restrict__ cur, int32_t* __restrict__ err) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n || cid[g] < 0) return;
    State r;
    if (!interpolate(load_state(cur + 14 * (size_t)g), load_state(last + 14 * (size_t)g), mct[cid[g]], r)) {
        atomicExch(err, 1);
        return;
    }
    store_state(cur + 14 * (size_t)g, r);
}

__global__ void k_iota32(int n, int32_t* __restrict__ v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = i;
}

__global__ void k_cl_sum(int n, const int32_t* __restrict__ a, const int32_t* __restrict__ b,
                         int32_t* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = a[i] + b[i];
}

__global__ void k_cl_body_keys(int n, const int32_t* __restrict__ cid, uint32_t* __restrict__ key,
                               int32_t* __restrict__ idx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    key[i] = (uint32_t)cid[i];  // static bodies (-1) sort last
    idx[i] = i;
}

__global__ void k_cl_pair_count(int n_pairs, const int32_t* __restrict__ pair_cid, int32_t* __restrict__ cnt) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n_pairs) atomicAdd(&cnt[pair_cid[k]], 1);
}

__global__ void k_cl_pair_gather(int n_pairs, const int32_t* __restrict__ order, const int32_t* __restrict__ pairs,
                                 int32_t* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_pairs) return;
    out[2 * (size_t)k] = pairs[2 * (size_t)order[k]];
    out[2 * (size_t)k + 1] = pairs[2 * (size_t)order[k] + 1];
}

// exclusive scan of in[0..n) into out[0..n], out[n] = total
int bscan(d2g_ctx* ctx, const int32_t* in, int32_t* out, int n) {
    Engine& E = ctx->eng;
    D2G_CUDA(cudaMemsetAsync(out, 0, sizeof(int32_t), ctx->stream));
    if (n == 0) return D2G_OK;
    size_t bytes = 0;
    D2G_CUDA(cub::DeviceScan::InclusiveSum(nullptr, bytes, in, out + 1, n, ctx->stream));
    RC(E.cub_tmp.ensure(bytes + 16));
    D2G_CUDA(cub::DeviceScan::InclusiveSum(E.cub_tmp.p, bytes, in, out + 1, n, ctx->stream));
    return D2G_OK;
}

template <class K, class V>
int sort_pairs(d2g_ctx* ctx, const K* kin, K* kout, const V* vin, V* vout, int n, int end_bit) {
    if (n <= 0) return D2G_OK;
    Engine& E = ctx->eng;
    size_t bytes = 0;
    D2G_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, bytes, kin, kout, vin, vout, n, 0, end_bit, ctx->stream));
    RC(E.cub_tmp.ensure(bytes + 16));
    D2G_CUDA(cub::DeviceRadixSort::SortPairs(E.cub_tmp.p, bytes, kin, kout, vin, vout, n, 0, end_bit, ctx->stream));
    return D2G_OK;
}

int read_ints(d2g_ctx* ctx, const int32_t* const* src, int k, int32_t* dst) {
    for (int i = 0; i < k; i++)
        D2G_CUDA(cudaMemcpyAsync(ctx->h_pinned + i, src[i], sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    D2G_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < k; i++) dst[i] = ctx->h_pinned[i];
    return D2G_OK;
}

}  // namespace

// Broad phase over the context's device bodies; the pairs (ascending) are
// left in E.bp_pairs.  d_err receives 1 on an invalid interpolation.
int run_broad_phase(d2g_ctx* ctx, const float* d_aabb, int* n_out, int32_t* d_err) {
    Engine& E = ctx->eng;
    const int n = ctx->n_bodies;
    RC(E.bp_box.ensure(6 * (size_t)n + 6));
    RC(E.bp_key.ensure(n + 1));
    RC(E.bp_key_s.ensure(n + 1));
    RC(E.bp_idx.ensure(n + 1));
    RC(E.bp_order.ensure(n + 1));
    RC(E.bp_range.ensure(n + 1));
    RC(E.bp_roff.ensure(n + 1));
    RC(E.bp_count.ensure(1));
    BLAUNCH(k_bp_boxes, n, n, ctx->is_static.p, ctx->last.p, ctx->cur.p, ctx->fut.p, ctx->bounding_radius.p,
            ctx->geo_eps.p, d_aabb, ctx->scene.p, E.bp_box.p, E.bp_key.p, E.bp_idx.p);
    int scene_bits = 0;
    while (scene_bits < 31 && (1 << scene_bits) < ctx->n_scenes) scene_bits++;
    RC(sort_pairs(ctx, E.bp_key.p, E.bp_key_s.p, E.bp_idx.p, E.bp_order.p, n, 32 + scene_bits));
    if (n > 0) BLAUNCH(k_bp_range, n, n, E.bp_order.p, E.bp_box.p, E.bp_key_s.p, E.bp_range.p);
    // 64-bit exclusive scan of the range lengths: roff[n] = total range elements
    D2G_CUDA(cudaMemsetAsync(E.bp_roff.p, 0, sizeof(long long), ctx->stream));
    if (n > 0) {
        size_t bytes = 0;
        D2G_CUDA(cub::DeviceScan::InclusiveSum(nullptr, bytes, E.bp_range.p, E.bp_roff.p + 1, n, ctx->stream));
        RC(E.cub_tmp.ensure(bytes + 16));
        D2G_CUDA(cub::DeviceScan::InclusiveSum(E.cub_tmp.p, bytes, E.bp_range.p, E.bp_roff.p + 1, n, ctx->stream));
    }
    // kept pairs: at most the previous capacity; on overflow grow and run again
    RC(E.bp_pkey2.ensure(4 * (size_t)n + 1024));
    int dev_sms = 0;
    D2G_CUDA(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device));
    int n_pairs = 0;
    for (int pass = 0; pass < 2; pass++) {
        const int cap = (int)std::min<size_t>(E.bp_pkey2.cap, (size_t)INT32_MAX);
        D2G_CUDA(cudaMemsetAsync(E.bp_count.p, 0, sizeof(int32_t), ctx->stream));
        k_bp_pairs<<<dev_sms * 8, 256, 0, ctx->stream>>>(
            n, E.bp_roff.p, E.bp_order.p, E.bp_box.p, ctx->is_static.p, ctx->last.p, ctx->cur.p,
            ctx->bounding_radius.p, ctx->geo_eps.p, ctx->last_dt.p, E.bp_pkey2.p, cap, E.bp_count.p, d_err);
        ctx->eng.launches++;
        const int32_t* src = E.bp_count.p;
        RC(read_ints(ctx, &src, 1, &n_pairs));
        if (n_pairs <= cap) break;
        RC(E.bp_pkey2.ensure((size_t)n_pairs + 1));
    }
    RC(E.bp_pkey.ensure(n_pairs + 1));
    if (n_pairs > 0) {
        size_t bytes = 0;
        D2G_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, bytes, E.bp_pkey2.p, E.bp_pkey.p, n_pairs, 0, 64,
                                                ctx->stream));
        RC(E.cub_tmp.ensure(bytes + 16));
        D2G_CUDA(cub::DeviceRadixSort::SortKeys(E.cub_tmp.p, bytes, E.bp_pkey2.p, E.bp_pkey.p, n_pairs, 0, 64,
                                                ctx->stream));
    }
    RC(E.bp_pairs.ensure(2 * (size_t)n_pairs + 2));
    if (n_pairs > 0) BLAUNCH(k_bp_unpack, n_pairs, n_pairs, E.bp_pkey.p, E.bp_pairs.p);
    *n_out = n_pairs;
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

// Cluster separation over the broad-phase pairs d_pairs (ascending).  Results
// in E.cl_*: per body cid; per cluster part_off / parts (moving members
// first, n_dyn of them), pair_off / pairs, mct, step, sleep.
int run_clusters(d2g_ctx* ctx, const int32_t* d_pairs, int n_pairs, int n_dyn_total, int* n_clusters_out,
                 int* n_parts_out, int32_t* d_err) {
    Engine& E = ctx->eng;
    const int n = ctx->n_bodies;
    const size_t np1 = (size_t)n_pairs + 1;
    RC(E.uf_parent.ensure(n + 1));
    RC(E.uf_root.ensure(n + 1));
    RC(E.uf_roff.ensure(n + 1));
    RC(E.cl_cid.ensure(n + 1));
    RC(E.cl_ukey.ensure(n + 1));
    RC(E.cl_ukey_s.ensure(n + 1));
    RC(E.cl_uidx.ensure(n + 1));
    RC(E.cl_member.ensure(n + 1));
    RC(E.cl_pair_cid.ensure(np1));
    RC(E.cl_pkey_s.ensure(np1));
    RC(E.cl_piota.ensure(np1));
    RC(E.cl_porder.ensure(np1));
    RC(E.cl_pairs.ensure(2 * np1));
    RC(E.cl_st_key.ensure(np1));
    RC(E.cl_st_key_s.ensure(np1));
    RC(E.cl_st_key2.ensure(np1));
    RC(E.cl_st_key3.ensure(np1));
    RC(E.cl_st_key4.ensure(np1));
    RC(E.cl_st_pos.ensure(np1));
    RC(E.cl_st_pos_s.ensure(np1));
    RC(E.cl_st_flag.ensure(np1));
    RC(E.cl_st_off.ensure(np1));
    RC(E.cl_st_body.ensure(np1));
    RC(E.cl_st_body3.ensure(np1));
    RC(E.cl_st_body4.ensure(np1));
    BLAUNCH(k_uf_init, n, n, E.uf_parent.p);
    if (n_pairs > 0) BLAUNCH(k_uf_union, n_pairs, n_pairs, d_pairs, ctx->is_static.p, E.uf_parent.p, d_err);
    BLAUNCH(k_uf_roots, n, n, E.uf_parent.p, ctx->is_static.p, E.uf_root.p);
    RC(bscan(ctx, E.uf_root.p, E.uf_roff.p, n));
    BLAUNCH(k_cl_ids, n, n, E.uf_parent.p, E.uf_roff.p, ctx->is_static.p, E.cl_cid.p);
    // moving members sorted by cluster, ascending within (stable)
    BLAUNCH(k_cl_body_keys, n, n, E.cl_cid.p, E.cl_ukey.p, E.cl_uidx.p);
    RC(sort_pairs(ctx, E.cl_ukey.p, E.cl_ukey_s.p, E.cl_uidx.p, E.cl_member.p, n, 32));
    const int32_t* member_cid = (const int32_t*)E.cl_ukey_s.p;
    if (n_pairs > 0) {
        BLAUNCH(k_cl_pair_keys, n_pairs, n_pairs, d_pairs, ctx->is_static.p, E.cl_cid.p, E.cl_pair_cid.p,
                E.cl_st_key.p, E.cl_st_pos.p);
        // interactions grouped by cluster, broad-phase order within (stable)
        BLAUNCH(k_iota32, n_pairs, n_pairs, E.cl_piota.p);
        RC(sort_pairs(ctx, (const uint32_t*)E.cl_pair_cid.p, E.cl_pkey_s.p, E.cl_piota.p, E.cl_porder.p, n_pairs,
                      32));
        BLAUNCH(k_cl_pair_gather, n_pairs, n_pairs, E.cl_porder.p, d_pairs, E.cl_pairs.p);
        // static bodies: first interaction of each (cluster, static body)
        RC(sort_pairs(ctx, E.cl_st_key.p, E.cl_st_key_s.p, E.cl_st_pos.p, E.cl_st_pos_s.p, n_pairs, 64));
        BLAUNCH(k_cl_static_first, n_pairs, n_pairs, E.cl_st_key_s.p, E.cl_st_pos_s.p, E.cl_st_flag.p,
                E.cl_st_key2.p, E.cl_st_body.p);
    }
    RC(bscan(ctx, E.cl_st_flag.p, E.cl_st_off.p, n_pairs));
    int vals[2];
    const int32_t* srcs[2] = {E.uf_roff.p + n, E.cl_st_off.p + n_pairs};
    RC(read_ints(ctx, srcs, 2, vals));
    const int nc = vals[0], n_st = vals[1];
    if (n_st > 0) {
        BLAUNCH(k_cl_compact2, n_pairs, n_pairs, E.cl_st_flag.p, E.cl_st_off.p, E.cl_st_key2.p, E.cl_st_body.p,
                E.cl_st_key3.p, E.cl_st_body3.p);
        RC(sort_pairs(ctx, E.cl_st_key3.p, E.cl_st_key4.p, E.cl_st_body3.p, E.cl_st_body4.p, n_st, 64));
    }
    const size_t nc1 = (size_t)nc + 1;
    RC(E.cl_n_dyn.ensure(nc1));
    RC(E.cl_n_stat.ensure(nc1));
    RC(E.cl_n_all.ensure(nc1));
    RC(E.cl_dyn_off.ensure(nc1));
    RC(E.cl_stat_off.ensure(nc1));
    RC(E.cl_part_off.ensure(nc1));
    RC(E.cl_pair_cnt.ensure(nc1));
    RC(E.cl_pair_off.ensure(nc1));
    RC(E.cl_mct.ensure(nc1));
    RC(E.cl_step.ensure(nc1));
    RC(E.cl_sleep.ensure(nc1));
    const int n_parts = n_dyn_total + n_st;
    RC(E.cl_parts.ensure((size_t)n_parts + 1));
    if (nc > 0) {
        D2G_CUDA(cudaMemsetAsync(E.cl_n_dyn.p, 0, sizeof(int32_t) * nc, ctx->stream));
        D2G_CUDA(cudaMemsetAsync(E.cl_n_stat.p, 0, sizeof(int32_t) * nc, ctx->stream));
        D2G_CUDA(cudaMemsetAsync(E.cl_pair_cnt.p, 0, sizeof(int32_t) * nc, ctx->stream));
        const int m = n_dyn_total > n_st ? n_dyn_total : n_st;
        BLAUNCH(k_cl_count, m, n_dyn_total, member_cid, n_st, E.cl_st_key4.p, E.cl_n_dyn.p, E.cl_n_stat.p);
        BLAUNCH(k_cl_sum, nc, nc, E.cl_n_dyn.p, E.cl_n_stat.p, E.cl_n_all.p);
        RC(bscan(ctx, E.cl_n_dyn.p, E.cl_dyn_off.p, nc));
        RC(bscan(ctx, E.cl_n_stat.p, E.cl_stat_off.p, nc));
        RC(bscan(ctx, E.cl_n_all.p, E.cl_part_off.p, nc));
        BLAUNCH(k_cl_fill, m, n_dyn_total, member_cid, E.cl_member.p, E.cl_dyn_off.p, n_st, E.cl_st_key4.p,
                E.cl_st_body4.p, E.cl_stat_off.p, E.cl_part_off.p, E.cl_n_dyn.p, E.cl_parts.p);
        BLAUNCH(k_cl_meta, 32LL * nc, nc, E.cl_part_off.p, E.cl_n_dyn.p, E.cl_parts.p, ctx->cur.p, ctx->last_dt.p,
                ctx->sleeping.p, E.cl_mct.p, E.cl_step.p, E.cl_sleep.p);
        if (n_pairs > 0) BLAUNCH(k_cl_pair_count, n_pairs, n_pairs, E.cl_pair_cid.p, E.cl_pair_cnt.p);
        RC(bscan(ctx, E.cl_pair_cnt.p, E.cl_pair_off.p, nc));
    } else {
        D2G_CUDA(cudaMemsetAsync(E.cl_part_off.p, 0, sizeof(int32_t), ctx->stream));
        D2G_CUDA(cudaMemsetAsync(E.cl_pair_off.p, 0, sizeof(int32_t), ctx->stream));
    }
    *n_clusters_out = nc;
    *n_parts_out = n_parts;
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

// Moving bodies back to their clusters' minimum current time (after run_clusters).
int run_cluster_rollback(d2g_ctx* ctx, int32_t* d_err) {
    Engine& E = ctx->eng;
    BLAUNCH(k_cl_rollback, ctx->n_bodies, ctx->n_bodies, E.cl_cid.p, E.cl_mct.p, ctx->last.p, ctx->cur.p, d_err);
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

}  // namespace d2g
