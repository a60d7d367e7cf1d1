// Level-synchronous surrogate-tree traversal on the GPU, for all body pairs
// of a call at once.
//
// The reference walks one body pair at a time, level by level
// (collision_detection/full_tree_comparison.h:13-219).  Here every frontier
// holds the node pairs of ALL body pairs, sorted by body pair and, within a
// pair, in the reference's order; every expansion is an ordered compaction
// (prefix sums), so the contacts of each pair come out in exactly the order
// the reference's sequential loops produce them.  Each level of each stage
// is three kinds of launches:
//   1. a cheap filter over all primitive slots (swept boxes in the CCD soup
//      stage), compacted into a dense work list;
//   2. one thread per primitive test (triangle-triangle CCD, point-triangle
//      CCD, edge-edge CCD or discrete triangle distance) writing its result
//      and hit flag;
//   3. ordered compaction of the contacts of leaf-leaf node pairs and
//      expansion of the node pairs that hit into the next frontiers.
// All arithmetic is FP64 with -fmad=false, in the order declared in
// d2g_geom.cuh, so results equal the CPU restatement bit for bit.
#include <cub/cub.cuh>

#include <mutex>
#include <string>

#include "d2g_geom.cuh"
#include "d2g_internal.hpp"

namespace d2g {

namespace {

constexpr int kBlock = 128;

inline int nblocks(long long n, int b = kBlock) { return (int)((n + b - 1) / b); }

__device__ __forceinline__ int4 ld_node(const int4* nodes, int g) { return nodes[g]; }

// ------------------------------------------------------------- CCD prep ----
// Projects both futures over the pair's max_time (model/state.cpp:90-102,
// full_tree_comparison.h:78-79) and forms the pose matrices.
// Per pair: the futures over max_time, the pose matrices (pair_mats) and the
// root frontier entry.  Four lanes per pair: lanes 1 and 3 extrapolate a and
// b, lane k forms transform k (a start, a end, b start, b end) and then the
// product inverse(transform k^2) * transform k, so the four 4x4 inverses and
// products run side by side.
__global__ void k_ccd_prep(int n, const int32_t* __restrict__ pairs, const double* __restrict__ max_time,
                           const double* __restrict__ cur, const double* __restrict__ ii,
                           const int32_t* __restrict__ mesh, const int32_t* __restrict__ mesh_node_off,
                           const double* __restrict__ geo_eps, double* __restrict__ pm, double* __restrict__ pfut,
                           float* __restrict__ search, Entry* __restrict__ soup) {
    const int p = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 2);
    const int k = threadIdx.x & 3;
    if (p >= n) return;  // uniform per quad
    const unsigned qm = 0xFu << (threadIdx.x & 28);
    const int body = pairs[2 * p + (k >> 1)];
    const State c = load_state(cur + 14 * (size_t)body);
    State st = c;
    if (k & 1) {
        st = extrapolate(c, max_time[p], ii + 9 * (size_t)body);
        store_state(pfut + 28 * (size_t)p + 14 * (k >> 1), st);
    }
    double* M = pm + (size_t)PM_SIZE * p;
    double T[16], O[16], inv[16], R[16];
    transformation(st.q, st.x, T);
#pragma unroll
    for (int i = 0; i < 16; i++) {
        M[16 * k + i] = T[i];
        O[i] = __shfl_xor_sync(qm, T[i], 2);
    }
    mat_inverse(O, inv);
    mat_mul(inv, T, R);
#pragma unroll
    for (int i = 0; i < 16; i++) M[PM_ABS + 16 * k + i] = R[i];
    if (k == 0) {
        const int a = pairs[2 * p], b = pairs[2 * p + 1];
        search[p] = (float)(geo_eps[a] + geo_eps[b]);
        Entry e;
        e.pair = p;
        e.na = mesh_node_off[mesh[a]];
        e.nb = mesh_node_off[mesh[b]];
        soup[p] = e;
    }
}

// Discrete narrow phase prep: future transforms of a and b (comparison_dist.h:225,229).
__global__ void k_np_prep(int n, const int32_t* __restrict__ pairs, const double* __restrict__ fut,
                          const int32_t* __restrict__ mesh, const int32_t* __restrict__ mesh_node_off,
                          const double* __restrict__ geo_eps, double* __restrict__ pm, float* __restrict__ search,
                          Entry* __restrict__ front, float* __restrict__ pm32) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int a = pairs[2 * p], b = pairs[2 * p + 1];
    const State fa = load_state(fut + 14 * (size_t)a);
    const State fb = load_state(fut + 14 * (size_t)b);
    double* M = pm + 32 * (size_t)p;
    transformation(fa.q, fa.x, M);
    transformation(fb.q, fb.x, M + 16);
    if (pm32)  // rows 0-2 of both poses in FP32, for the candidate prefilter
        for (int k = 0; k < 12; k++) {
            pm32[24 * (size_t)p + k] = (float)M[k];
            pm32[24 * (size_t)p + 12 + k] = (float)M[16 + k];
        }
    search[p] = (float)(geo_eps[a] + geo_eps[b]);
    Entry e;
    e.pair = p;
    e.na = mesh_node_off[mesh[a]];
    e.nb = mesh_node_off[mesh[b]];
    front[p] = e;
}

// ------------------------------------------------------------ soup stage ---
__global__ void k_compact(int n, const int32_t* __restrict__ flags, const int32_t* __restrict__ off,
                          int32_t* __restrict__ items) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (flags[i]) items[off[i]] = i;
}

__device__ __forceinline__ void put_result(PrimResult& r, double dist, V3 A, V3 B, double toc) {
    r.dist = dist;
    r.P[0] = A.x;
    r.P[1] = A.y;
    r.P[2] = A.z;
    r.Q[0] = B.x;
    r.Q[1] = B.y;
    r.Q[2] = B.z;
    r.toc = toc;
}

// ------------------------------------------- flattened primitive tests -----
// One level of the CCD as two homogeneous work lists: every point-triangle
// test and every edge-edge test of the level, from the soup stage (the 15
// sub-tests of each surviving triangle pair, continuous_comparison.h:692-777)
// and from the connected stage (all tests of each leaf pair, :855-907).
// Point-triangle list: 6 per soup triangle pair, then 6*na*nb per leaf pair;
// edge-edge list: 9 per soup triangle pair, then 9*na*nb per leaf pair.  The
// soup sub-results are folded afterwards in the reference's order.
constexpr int kPrimBlock = 64;

__global__ void k_conn_nn(int n, const Entry* __restrict__ conn, const int32_t* __restrict__ ntris,
                          int32_t* __restrict__ cnt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Entry e = conn[i];
    cnt[i] = ntris[e.na] * ntris[e.nb];
}

__global__ void k_scale(int n, const int32_t* __restrict__ in, int32_t m, int32_t* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = m * in[i];
}

// Last entry e with m*off[e] <= k (off[0] == 0).
__device__ __forceinline__ int find_entry(const int32_t* __restrict__ off, int n_entries, int m, int k) {
    int lo = 0, hi = n_entries;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (m * off[mid] <= k)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

__device__ __forceinline__ void store_prim(PrimResult* __restrict__ r, double dist, V3 A, V3 B, double toc) {
    r->dist = dist;
    r->P[0] = A.x;
    r->P[1] = A.y;
    r->P[2] = A.z;
    r->Q[0] = B.x;
    r->Q[1] = B.y;
    r->Q[2] = B.z;
    r->toc = toc;
}

// ---------------------------------------------- FP32 candidate filtering ---
// Every primitive CCD test returns a distance between a point of a box built
// from its inputs and a point of a second box: for edgeEdgeCCD the world
// positions of the two edges' endpoints at the start and the end; for
// pointTriCCDLinear the point carried into the triangle's frame at the start
// and the end, then through the triangle body's start and end transforms, and
// the triangle's vertices through the same two transforms (the returned
// points are lerps of those).  A box gap above the hit threshold means the
// test cannot hit (a soup sub-test with such a distance can never be the best
// of a triangle pair that hits), so the test is recorded as no contact (+inf)
// and left out of the FP64 work list.  The gap is computed in FP32 and only
// used beyond a margin (1 mm plus 4e-6 of the largest coordinate involved)
// far above the FP32 and FP64 rounding at scene scale.

struct Box32 {
    float lo[3], hi[3];
};
__device__ __forceinline__ void box_init(Box32& b) {
    for (int k = 0; k < 3; k++) {
        b.lo[k] = 3.4e38f;
        b.hi[k] = -3.4e38f;
    }
}
// adds M (3x4 rows, FP32) applied to (x, y, z); returns the point in o
__device__ __forceinline__ void box_add(Box32& b, const float* M, float x, float y, float z, float* o, float& mag) {
    for (int r = 0; r < 3; r++) {
        const float v = M[4 * r] * x + M[4 * r + 1] * y + M[4 * r + 2] * z + M[4 * r + 3];
        o[r] = v;
        b.lo[r] = fminf(b.lo[r], v);
        b.hi[r] = fmaxf(b.hi[r], v);
        mag = fmaxf(mag, fabsf(v));
    }
}
__device__ __forceinline__ float box_gap(const Box32& a, const Box32& b) {
    float g2 = 0.f;
    for (int k = 0; k < 3; k++) {
        const float g = fmaxf(b.lo[k] - a.hi[k], a.lo[k] - b.hi[k]);
        if (g > 0.f) g2 += g * g;
    }
    return sqrtf(g2);
}

// Indices of PM_* matrices in the FP32 pose block (8 x 12 floats per pair).
__device__ __forceinline__ const float* pm32_of(const float* pm32, int pair, int which) {
    return pm32 + (size_t)96 * pair + 12 * which;
}
enum { P32_AS = 0, P32_AE, P32_BS, P32_BE, P32_ABS, P32_ABE, P32_BAS, P32_BAE };

__global__ void k_ccd_pm32(int n, const double* __restrict__ pm, float* __restrict__ pm32) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * 96) return;
    const int p = i / 96, w = (i % 96) / 12, r = i % 12;
    pm32[i] = (float)pm[(size_t)PM_SIZE * p + 16 * w + r];
}

// The swept-AABB prefilter of every (triangle of a, triangle of b) slot of a
// soup node pair (continuous_comparison.h:804-812), one warp per node pair:
// lanes 0-7 form the swept boxes of a's triangles, lanes 8-15 those of b's,
// once each, and every lane then tests two of the 64 slots from shuffled
// boxes.  flags[64 * entry + 8 * ta + tb] = 1 where the boxes overlap.  The
// boxes are first formed in FP32 (FP32 poses and triangles): a slot whose
// boxes are apart, or overlap, by more than a margin (1e-4 m plus 4e-6 of the
// largest coordinate, far above the FP32 rounding of the box edges) has the
// answer the FP64 boxes give; a warp with any slot inside the margin (or a
// NaN) forms the FP64 boxes and decides those slots exactly.
__global__ void k_soup_filter(int n_soup, const Entry* __restrict__ soup, const int32_t* __restrict__ pairs,
                              const double* __restrict__ pm, const float* __restrict__ pm32,
                              const int32_t* __restrict__ ntris, const double* __restrict__ tris,
                              const float* __restrict__ tri32, const double* __restrict__ geo_eps,
                              const uint8_t* __restrict__ skip, const uint8_t* __restrict__ eskip,
                              int32_t* __restrict__ flags) {
    const int w = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= n_soup) return;  // uniform per warp
    const Entry e = soup[w];
    // a pair the root certificate proved contact-free, or a node pair its
    // separation witness proved clear: no slot goes on
    if ((skip && skip[e.pair]) || (eskip && eskip[w])) {
        flags[64 * (size_t)w + lane] = 0;
        flags[64 * (size_t)w + lane + 32] = 0;
        return;
    }
    const int na = ntris[e.na], nb = ntris[e.nb];
    const bool side_b = lane >= 8;
    const int t = lane & 7;
    const bool own = lane < 16 && t < (side_b ? nb : na);
    const int body = pairs[2 * e.pair + (side_b ? 1 : 0)];
    const int node = side_b ? e.nb : e.na;
    Box32 b32;
    box_init(b32);
    float mag = 0.f;
    if (own) {
        const float* tv = tri32 + ((size_t)node * 8 + t) * 9;
        const float* MS = pm32_of(pm32, e.pair, side_b ? P32_BS : P32_AS);
        const float* ME = pm32_of(pm32, e.pair, side_b ? P32_BE : P32_AE);
        float o[3];
#pragma unroll
        for (int v = 0; v < 3; v++) {
            box_add(b32, MS, tv[3 * v], tv[3 * v + 1], tv[3 * v + 2], o, mag);
            box_add(b32, ME, tv[3 * v], tv[3 * v + 1], tv[3 * v + 2], o, mag);
        }
        const float e32 = (float)geo_eps[body];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            b32.lo[k] -= e32;
            b32.hi[k] += e32;
        }
        mag += e32;
    }
    int res[2];
    bool border = false;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int sl = lane + 32 * h, ta = sl >> 3, tb = sl & 7;
        float alo[3], ahi[3], blo[3], bhi[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            alo[k] = __shfl_sync(0xffffffffu, b32.lo[k], ta);
            ahi[k] = __shfl_sync(0xffffffffu, b32.hi[k], ta);
            blo[k] = __shfl_sync(0xffffffffu, b32.lo[k], 8 + tb);
            bhi[k] = __shfl_sync(0xffffffffu, b32.hi[k], 8 + tb);
        }
        const float m = 1e-4f + 4e-6f * fmaxf(__shfl_sync(0xffffffffu, mag, ta), __shfl_sync(0xffffffffu, mag, 8 + tb));
        res[h] = 0;
        if (ta < na && tb < nb) {
            bool apart = false, over = true;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                apart = apart || blo[k] > ahi[k] + m || alo[k] > bhi[k] + m;
                over = over && blo[k] < ahi[k] - m && alo[k] < bhi[k] - m;
            }
            res[h] = apart ? 0 : (over ? 1 : 2);
            border = border || res[h] == 2;
        }
    }
    if (__any_sync(0xffffffffu, border)) {
        Box bx;
#pragma unroll
        for (int k = 0; k < 3; k++) bx.lo[k] = bx.hi[k] = 0.0;
        if (own) {
            const double* M = pm + (size_t)PM_SIZE * e.pair;
            const Tri tri = load_tri(tris + (size_t)node * 72 + t * 9);
            bx = side_b ? swept_box(tri, M + PM_BS, M + PM_BE, geo_eps[body])
                        : swept_box(tri, M + PM_AS, M + PM_AE, geo_eps[body]);
        }
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int sl = lane + 32 * h, ta = sl >> 3, tb = sl & 7;
            Box A, B;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                A.lo[k] = __shfl_sync(0xffffffffu, bx.lo[k], ta);
                A.hi[k] = __shfl_sync(0xffffffffu, bx.hi[k], ta);
                B.lo[k] = __shfl_sync(0xffffffffu, bx.lo[k], 8 + tb);
                B.hi[k] = __shfl_sync(0xffffffffu, bx.hi[k], 8 + tb);
            }
            if (res[h] == 2) res[h] = box_overlap(A, B) ? 1 : 0;
        }
    }
    flags[64 * (size_t)w + lane] = res[0];
    flags[64 * (size_t)w + lane + 32] = res[1];
}


__global__ void k_add_u64(unsigned long long* __restrict__ v, unsigned long long x) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *v += x;
}

// ------------------------------------------------- learned proposal --------
// Features of a CCD pair query for the proposal network, from the bodies'
// current states: B's pose in A's frame (R_a^T R_b row major, R_a^T (x_b -
// x_a)), the relative motion over the query's horizon in A's frame
// (R_a^T (v_b - v_a) max_time, R_a^T (w_b - w_a) max_time with w = R I^-1 R^T L)
// and the two bounding radii; FP64, stored as FP32.
__global__ void k_ccd_features(int n, const int32_t* __restrict__ pairs, const double* __restrict__ max_time,
                               const double* __restrict__ cur, const double* __restrict__ ii,
                               const double* __restrict__ radius, float* __restrict__ feat) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int ia = pairs[2 * p], ib = pairs[2 * p + 1];
    const State a = load_state(cur + 14 * (size_t)ia), b = load_state(cur + 14 * (size_t)ib);
    double Ra[9], Rb[9], Ia[9], Ib[9];
    qmat(a.q, Ra);
    qmat(b.q, Rb);
    world_inv_inertia(a.q, ii + 9 * (size_t)ia, Ia);
    world_inv_inertia(b.q, ii + 9 * (size_t)ib, Ib);
    const V3 wa = m3_vec(Ia, a.L), wb = m3_vec(Ib, b.L);
    const double mt = max_time[p];
    float* f = feat + 20 * (size_t)p;
    auto at = [&](V3 v, int r) { return (Ra[r] * v.x + Ra[3 + r] * v.y) + Ra[6 + r] * v.z; };  // (R_a^T v)_r
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) f[3 * r + c] = (float)((Ra[r] * Rb[c] + Ra[3 + r] * Rb[3 + c]) + Ra[6 + r] * Rb[6 + c]);
    for (int r = 0; r < 3; r++) {
        f[9 + r] = (float)at(b.x - a.x, r);
        f[12 + r] = (float)(at(b.v - a.v, r) * mt);
        f[15 + r] = (float)(at(wb - wa, r) * mt);
    }
    f[18] = (float)radius[ia];
    f[19] = (float)radius[ib];
}

// The root certificate of a pair query the network predicts contact-free: a
// warp per pair proves that no slot of the root node pair can hit, so the
// query has no contacts (compareTreesFullContinuous expands only node pairs
// with hits).  A slot is proven clear when the reference's swept-box test
// rejects it (continuous_comparison.h:804-812; decided in FP32 beyond a
// margin, as the swept-box filter decides it, else in FP64), or when the
// two triangles' vertices, each on a straight line from its start to its end
// position, stay apart over the motion:
//   * along an axis n fixed at the start (the centroid difference, either
//     face normal), min_j n.b_j(t) - max_i n.a_i(t) is concave in t, so its
//     minimum over [0, 1] is at t = 0 or 1; the gap over |n| bounds every
//     edge-edge distance edgeEdgeCCD evaluates (points of the two edges at
//     one time), and the point-to-triangle distances at t = 0 and 1;
//   * pointTriCCDLinear returns 0 only when a vertex's start and end lie on
//     opposite sides of the other triangle's plane (its start and end frames),
//     and otherwise the vertex's distance to that plane at t = 0 or 1 when its
//     projection falls inside (decided with float barycentrics) or nothing:
//     so every vertex must keep its side, and the gap carries a margin for a
//     projection the float test puts inside by mistake (6e-7 of the
//     triangle's size times its conditioning (L0 L1 / 2 area)^2).
// A query whose every root slot is proven clear is skipped: it would produce
// no contact.  Any slot not proven leaves the query to the exact traversal.
// stats: [2] predicted clear, [3] certified, [4] not certified, [5] seen.
__device__ __forceinline__ double axis_gap(V3 n, const V3* A0, const V3* A1, const V3* B0, const V3* B1) {
    double g = -1e300;
    for (int sg = 0; sg < 2; sg++) {
        const V3 m = sg ? -n : n;
        double gmin = 1e300;
        for (int t = 0; t < 2; t++) {
            const V3* A = t ? A1 : A0;
            const V3* B = t ? B1 : B0;
            const double amax = fmax(fmax(dot(m, A[0]), dot(m, A[1])), dot(m, A[2]));
            const double bmin = fmin(fmin(dot(m, B[0]), dot(m, B[1])), dot(m, B[2]));
            gmin = fmin(gmin, bmin - amax);
        }
        g = fmax(g, gmin);
    }
    const double nn = norm(n);
    return nn > 0.0 ? g / nn : -1e300;
}
// every vertex of P keeps a side of T's plane (start and end frames), with
// distances far above rounding
__device__ __forceinline__ bool keeps_side(const V3* P0, const V3* P1, const V3* T0, const V3* T1, double tol) {
    const V3 n0 = cross(T0[1] - T0[0], T0[2] - T0[0]), n1 = cross(T1[1] - T1[0], T1[2] - T1[0]);
    const double l0 = norm(n0), l1 = norm(n1);
    if (!(l0 > 0.0) || !(l1 > 0.0)) return false;
    for (int i = 0; i < 3; i++) {
        const double h0 = dot(n0, P0[i] - T0[0]) / l0, h1 = dot(n1, P1[i] - T1[0]) / l1;
        if (!(h0 * h1 > 0.0) || !(fabs(h0) > tol) || !(fabs(h1) > tol)) return false;
    }
    return true;
}
__device__ __forceinline__ double tri_conditioning(const V3* T, double& lmax) {
    const double l0 = norm(T[1] - T[0]), l1 = norm(T[2] - T[0]), l2 = norm(T[2] - T[1]);
    lmax = fmax(fmax(l0, l1), l2);
    const double a2 = norm(cross(T[1] - T[0], T[2] - T[0]));
    if (!(a2 > 0.0)) return 1e300;
    const double k = (l0 * l1) / a2;
    return k * k;
}
// ------------------------------------------------ separation witnesses -----
// Temporal coherence of the CCD traversal (the separation witnesses of
// collision_detection/contact_state.cpp:14-150 and full_tree_comparison.cpp:
// 7-198, rebuilt so that results cannot change).  A witness is an axis, in
// body a's frame, that separated a soup node pair at an earlier call.  At the
// next call the node pair is skipped when that axis (through a's current
// rotation) still proves every slot of the pair clear over the query's motion,
// by the same proof as the root certificate (swept-box rejection, or
// side-keeping vertices and a separating gap beyond the search distance);
// a skipped node pair has no hit, so the reference would neither expand it
// nor emit from it.  Node pairs without hits get a new witness (the axis
// between their buckets' vertex centroids) when it proves them clear.  A
// stale or foreign witness can only fail its check.  Table: open addressing,
// 64-bit keys (bodies < 2^19, node ids local to their tree < 2^12; other
// node pairs get no witness), at most 32 probes.
__device__ __forceinline__ unsigned long long witness_key(int a, int b, int la, int lb) {
    if (a < 0 || b < 0 || a >= (1 << 19) || b >= (1 << 19) || la < 0 || lb < 0 || la >= 4096 || lb >= 4096)
        return 0ull;
    return (1ull << 63) | ((unsigned long long)a << 43) | ((unsigned long long)b << 24) |
           ((unsigned long long)la << 12) | (unsigned long long)lb;
}
__device__ __forceinline__ unsigned int witness_hash(unsigned long long k, int log2cap) {
    return (unsigned int)((k * 0x9E3779B97F4A7C15ull) >> (64 - log2cap));
}

// Every slot of node pair (na, nb) proven clear (warp-collective).  Lanes
// 0-7 hold a's triangles and lanes 8-15 b's: each forms its triangle's world
// vertices at the start and end and the reference's swept box once; every
// lane then takes two slots, rejected by the boxes or proven by the
// certificate from shuffled vertices.  With `axis` non-null only that world
// axis is tried (a witness); otherwise the slot's centroid difference and
// both face normals.
__device__ bool slots_clear(int na_node, int nb_node, const double* M, const float* pm32, int pair,
                            const int32_t* ntris, const double* tris, const float* tri32, double eps_a, double eps_b,
                            double S, const V3* axis) {
    const int lane = threadIdx.x & 31;
    const int na = ntris[na_node], nb = ntris[nb_node];
    const bool side_b = lane >= 8;
    const int t = lane & 7;
    const bool own = lane < 16 && t < (side_b ? nb : na);
    // The swept boxes first in FP32, as the swept-box filter forms them: a slot
    // whose boxes are apart by more than the margin is rejected as the FP64
    // boxes would reject it; only when some slot is not the warp goes on in FP64.
    bool apart32[2];
    {
        Box32 b32;
        box_init(b32);
        float mag = 0.f;
        if (own) {
            const float* tv = tri32 + ((size_t)(side_b ? nb_node : na_node) * 8 + t) * 9;
            const float* MS = pm32_of(pm32, pair, side_b ? P32_BS : P32_AS);
            const float* ME = pm32_of(pm32, pair, side_b ? P32_BE : P32_AE);
            float o[3];
            for (int v = 0; v < 3; v++) {
                box_add(b32, MS, tv[3 * v], tv[3 * v + 1], tv[3 * v + 2], o, mag);
                box_add(b32, ME, tv[3 * v], tv[3 * v + 1], tv[3 * v + 2], o, mag);
            }
            const float e32 = (float)(side_b ? eps_b : eps_a);
            for (int k = 0; k < 3; k++) {
                b32.lo[k] -= e32;
                b32.hi[k] += e32;
            }
            mag += e32;
        }
        bool any_near = false;
        for (int h = 0; h < 2; h++) {
            const int sl = lane + 32 * h, ta = sl >> 3, tb = sl & 7;
            bool apart = false;
            const float m = 1e-4f + 4e-6f * fmaxf(__shfl_sync(0xffffffffu, mag, ta),
                                                  __shfl_sync(0xffffffffu, mag, 8 + tb));
            for (int k = 0; k < 3; k++) {
                const float alo = __shfl_sync(0xffffffffu, b32.lo[k], ta), ahi = __shfl_sync(0xffffffffu, b32.hi[k], ta);
                const float blo = __shfl_sync(0xffffffffu, b32.lo[k], 8 + tb),
                            bhi = __shfl_sync(0xffffffffu, b32.hi[k], 8 + tb);
                apart = apart || blo > ahi + m || alo > bhi + m;
            }
            apart32[h] = apart;
            any_near = any_near || (ta < na && tb < nb && !apart);
        }
        if (!__any_sync(0xffffffffu, any_near)) return true;  // every slot rejected by the swept boxes
    }
    V3 v0[3], v1[3];
    Box bx;
    for (int k = 0; k < 3; k++) bx.lo[k] = bx.hi[k] = 0.0;
    for (int i = 0; i < 3; i++) v0[i] = v1[i] = mk(0, 0, 0);
    if (own) {
        const Tri T = load_tri(tris + (size_t)(side_b ? nb_node : na_node) * 72 + t * 9);
        const double* MS = M + (side_b ? PM_BS : PM_AS);
        const double* ME = M + (side_b ? PM_BE : PM_AE);
        bx = swept_box(T, MS, ME, side_b ? eps_b : eps_a);
        v0[0] = xform_rigid(T.A, MS);
        v0[1] = xform_rigid(T.B, MS);
        v0[2] = xform_rigid(T.C, MS);
        v1[0] = xform_rigid(T.A, ME);
        v1[1] = xform_rigid(T.B, ME);
        v1[2] = xform_rigid(T.C, ME);
    }
    auto sh3 = [&](V3 v, int src) {
        return mk(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src),
                  __shfl_sync(0xffffffffu, v.z, src));
    };
    bool clear = true;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int sl = lane + 32 * h, ta = sl >> 3, tb = sl & 7;
        Box A, B;
        for (int k = 0; k < 3; k++) {
            A.lo[k] = __shfl_sync(0xffffffffu, bx.lo[k], ta);
            A.hi[k] = __shfl_sync(0xffffffffu, bx.hi[k], ta);
            B.lo[k] = __shfl_sync(0xffffffffu, bx.lo[k], 8 + tb);
            B.hi[k] = __shfl_sync(0xffffffffu, bx.hi[k], 8 + tb);
        }
        V3 A0[3], A1[3], B0[3], B1[3];
        for (int i = 0; i < 3; i++) {
            A0[i] = sh3(v0[i], ta);
            A1[i] = sh3(v1[i], ta);
            B0[i] = sh3(v0[i], 8 + tb);
            B1[i] = sh3(v1[i], 8 + tb);
        }
        if (ta >= na || tb >= nb || !clear || apart32[h] || !box_overlap(A, B)) continue;
        double mag = 0.0;
        for (int i = 0; i < 3; i++)
            mag = fmax(mag, fmax(fmax(fmax(fabs(A0[i].x), fabs(A0[i].y)), fabs(A0[i].z)),
                                 fmax(fmax(fabs(B0[i].x), fabs(B0[i].y)), fabs(B0[i].z))));
        double la, lb;
        const double ka = tri_conditioning(A0, la), kb = tri_conditioning(B0, lb);
        if (!(ka < 1e4) || !(kb < 1e4)) {
            clear = false;
            continue;
        }
        const double tol = 1e-9 + 1e-12 * mag;
        const double margin = (1e-5 + 1e-9 * mag) + 6e-7 * fmax(ka * la, kb * lb);
        if (!keeps_side(A0, A1, B0, B1, tol) || !keeps_side(B0, B1, A0, A1, tol)) {
            clear = false;
            continue;
        }
        double g;
        if (axis) {
            g = axis_gap(*axis, A0, A1, B0, B1);
        } else {
            const V3 ca = (A0[0] + A0[1]) + A0[2], cb = (B0[0] + B0[1]) + B0[2];
            g = axis_gap(cb - ca, A0, A1, B0, B1);
            g = fmax(g, axis_gap(cross(A0[1] - A0[0], A0[2] - A0[0]), A0, A1, B0, B1));
            g = fmax(g, axis_gap(cross(B0[1] - B0[0], B0[2] - B0[0]), A0, A1, B0, B1));
        }
        if (!(g >= S + margin)) clear = false;
    }
    return __all_sync(0xffffffffu, clear);
}

__global__ void k_root_certify(int n, const int32_t* __restrict__ pairs, const double* __restrict__ pm,
                               const float* __restrict__ pm32, const float* __restrict__ tri32,
                               const int32_t* __restrict__ mesh, const int32_t* __restrict__ mesh_node_off,
                               const int32_t* __restrict__ ntris, const double* __restrict__ tris,
                               const double* __restrict__ geo_eps, const float* __restrict__ search,
                               const float* __restrict__ pred, float logit_cut, uint8_t* __restrict__ skip,
                               unsigned long long* __restrict__ stats) {
    const int p = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (p >= n) return;  // uniform per warp
    const bool gated = pred[2 * (size_t)p + 1] < logit_cut;  // NaN: not gated
    if (!gated) {
        if (lane == 0) skip[p] = 0;
        return;
    }
    const int ia = pairs[2 * p], ib = pairs[2 * p + 1];
    const bool all = slots_clear(mesh_node_off[mesh[ia]], mesh_node_off[mesh[ib]], pm + (size_t)PM_SIZE * p, pm32, p,
                                 ntris, tris, tri32, geo_eps[ia], geo_eps[ib], (double)search[p], nullptr);
    if (lane == 0) {
        skip[p] = all ? 1 : 0;
        atomicAdd(stats + 2, 1ull);
        atomicAdd(stats + (all ? 3 : 4), 1ull);
    }
}

__global__ void k_witness_check(int n, const Entry* __restrict__ soup, const int32_t* __restrict__ pairs,
                                const double* __restrict__ pm, const float* __restrict__ pm32,
                                const float* __restrict__ tri32, const int32_t* __restrict__ mesh,
                                const int32_t* __restrict__ mesh_node_off, const int32_t* __restrict__ ntris,
                                const double* __restrict__ tris, const double* __restrict__ geo_eps,
                                const float* __restrict__ search, const WitnessSlot* __restrict__ table,
                                int log2cap, uint8_t* __restrict__ wflag, unsigned long long* __restrict__ stats) {
    const int w = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= n) return;  // uniform per warp
    const Entry e = soup[w];
    const int a = pairs[2 * e.pair], b = pairs[2 * e.pair + 1];
    const unsigned long long key =
        witness_key(a, b, e.na - mesh_node_off[mesh[a]], e.nb - mesh_node_off[mesh[b]]);
    int found = -1;
    if (key) {
        const unsigned int mask = (1u << log2cap) - 1u;
        unsigned int h = witness_hash(key, log2cap);
        for (int probe = 0; probe < 32; probe++, h = (h + 1) & mask) {
            const unsigned long long k = table[h].key;
            if (k == key) {
                found = (int)h;
                break;
            }
            if (k == 0ull) break;
        }
    }
    bool clear = false;
    if (found >= 0) {
        const double* M = pm + (size_t)PM_SIZE * e.pair;
        const WitnessSlot& W = table[found];
        // the axis through a's rotation at the start (rows 0-2 of its start transform)
        const V3 loc = mk((double)W.ax, (double)W.ay, (double)W.az);
        const V3 n_world = mk((M[PM_AS + 0] * loc.x + M[PM_AS + 1] * loc.y) + M[PM_AS + 2] * loc.z,
                              (M[PM_AS + 4] * loc.x + M[PM_AS + 5] * loc.y) + M[PM_AS + 6] * loc.z,
                              (M[PM_AS + 8] * loc.x + M[PM_AS + 9] * loc.y) + M[PM_AS + 10] * loc.z);
        clear = norm(n_world) > 0.0 && slots_clear(e.na, e.nb, M, pm32, e.pair, ntris, tris, tri32, geo_eps[a],
                                                   geo_eps[b], (double)search[e.pair], &n_world);
    }
    if (lane == 0) {
        wflag[w] = clear ? 1 : 0;
        if (clear) atomicAdd(stats + 6, 1ull);
    }
}

__global__ void k_witness_make(int n, const Entry* __restrict__ soup, const int32_t* __restrict__ entry_hits,
                               const uint8_t* __restrict__ wflag, const uint8_t* __restrict__ skip,
                               const int32_t* __restrict__ pairs, const double* __restrict__ pm,
                               const float* __restrict__ pm32, const float* __restrict__ tri32,
                               const int32_t* __restrict__ mesh, const int32_t* __restrict__ mesh_node_off,
                               const int32_t* __restrict__ ntris, const double* __restrict__ tris,
                               const double* __restrict__ geo_eps, const float* __restrict__ search,
                               WitnessSlot* __restrict__ table, int log2cap, unsigned long long* __restrict__ stats) {
    const int w = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= n) return;  // uniform per warp
    const Entry e = soup[w];
    if (entry_hits[w] > 0 || wflag[w] || (skip && skip[e.pair])) return;
    const int a = pairs[2 * e.pair], b = pairs[2 * e.pair + 1];
    const unsigned long long key =
        witness_key(a, b, e.na - mesh_node_off[mesh[a]], e.nb - mesh_node_off[mesh[b]]);
    if (!key) return;
    const double* M = pm + (size_t)PM_SIZE * e.pair;
    // the axis between the two buckets' vertex centroids at the start
    const int na = ntris[e.na], nb = ntris[e.nb];
    V3 c = mk(0, 0, 0);
    if (lane < 16) {
        const int t = lane & 7;
        const bool side_b = lane >= 8;
        if (t < (side_b ? nb : na)) {
            const Tri T = load_tri(tris + (size_t)(side_b ? e.nb : e.na) * 72 + t * 9);
            const double* Ms = M + (side_b ? PM_BS : PM_AS);
            const V3 s = (xform_rigid(T.A, Ms) + xform_rigid(T.B, Ms)) + xform_rigid(T.C, Ms);
            c = s * (side_b ? 1.0 / nb : -1.0 / na);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        c.x += __shfl_xor_sync(0xffffffffu, c.x, o);
        c.y += __shfl_xor_sync(0xffffffffu, c.y, o);
        c.z += __shfl_xor_sync(0xffffffffu, c.z, o);
    }
    if (!(norm(c) > 0.0) ||
        !slots_clear(e.na, e.nb, M, pm32, e.pair, ntris, tris, tri32, geo_eps[a], geo_eps[b], (double)search[e.pair],
                     &c))
        return;
    if (lane == 0) {
        // store the axis in a's frame: R_a^T n
        const V3 loc = mk((M[PM_AS + 0] * c.x + M[PM_AS + 4] * c.y) + M[PM_AS + 8] * c.z,
                          (M[PM_AS + 1] * c.x + M[PM_AS + 5] * c.y) + M[PM_AS + 9] * c.z,
                          (M[PM_AS + 2] * c.x + M[PM_AS + 6] * c.y) + M[PM_AS + 10] * c.z);
        const unsigned int mask = (1u << log2cap) - 1u;
        unsigned int h = witness_hash(key, log2cap);
        for (int probe = 0; probe < 32; probe++, h = (h + 1) & mask) {
            const unsigned long long old = atomicCAS(&table[h].key, 0ull, key);
            if (old == 0ull || old == key) {
                table[h].ax = (float)loc.x;
                table[h].ay = (float)loc.y;
                table[h].az = (float)loc.z;
                atomicAdd(stats + 7, 1ull);
                break;
            }
        }
    }
}

// Point-triangle work item j (the decoding of k_prim_pt): which pair, which
// point (body-local), which triangle (body-local) and which transforms.
struct PtWork {
    int pair, pt_node, pt_tri, pt_vert, tri_node, tri_idx, mC, mT;  // mC: point frame pair, mT: triangle body
    PrimResult* out;
    int32_t* hit;
};
__device__ __forceinline__ PtWork decode_pt(int j, int n_tp, const int32_t* items, const Entry* soup,
                                            const Entry* conn, const int32_t* nn_off, int n_conn,
                                            const int32_t* ntris, PrimResult* sub, PrimResult* cres, int32_t* chit) {
    PtWork w;
    w.hit = nullptr;
    if (j < 6 * n_tp) {
        const int k = j / 6, q = j % 6;
        const int slot = items[k];
        const Entry e = soup[slot >> 6];
        const int i = q >> 1;
        w.pair = e.pair;
        if (q & 1) {
            w.pt_node = e.nb, w.pt_tri = slot & 7, w.tri_node = e.na, w.tri_idx = (slot >> 3) & 7;
            w.mC = P32_BAS, w.mT = P32_AS;
        } else {
            w.pt_node = e.na, w.pt_tri = (slot >> 3) & 7, w.tri_node = e.nb, w.tri_idx = slot & 7;
            w.mC = P32_ABS, w.mT = P32_BS;
        }
        w.pt_vert = i;
        w.out = sub + 15 * (size_t)k + 5 * i + (q & 1);
        return w;
    }
    const int jp = j - 6 * n_tp;
    const int ei = find_entry(nn_off, n_conn, 6, jp);
    const Entry e = conn[ei];
    const int l = jp - 6 * nn_off[ei];
    const int na = ntris[e.na], nb = ntris[e.nb];
    const int n1 = 3 * na * nb;
    w.pair = e.pair;
    if (l < n1) {
        const int vi = l / nb, jj = l % nb;
        w.pt_node = e.na, w.pt_tri = vi / 3, w.pt_vert = vi % 3, w.tri_node = e.nb, w.tri_idx = jj;
        w.mC = P32_ABS, w.mT = P32_BS;
    } else {
        const int m = l - n1;
        const int vi = m / na, jj = m % na;
        w.pt_node = e.nb, w.pt_tri = vi / 3, w.pt_vert = vi % 3, w.tri_node = e.na, w.tri_idx = jj;
        w.mC = P32_BAS, w.mT = P32_AS;
    }
    const size_t item = 15 * (size_t)nn_off[ei] + l;
    w.out = cres + item;
    w.hit = chit + item;
    return w;
}

// Edge-edge work item j, as the edge-edge mask and CCD kernels decode it.
struct EeWork {
    int pair, na, nb, aTri, aEdge, bTri, bEdge;
    PrimResult* out;
    int32_t* hit;
};
__device__ __forceinline__ EeWork decode_ee(int j, int n_tp, const int32_t* items, const Entry* soup,
                                            const Entry* conn, const int32_t* nn_off, int n_conn,
                                            const int32_t* ntris, PrimResult* sub, PrimResult* cres, int32_t* chit) {
    EeWork w;
    w.hit = nullptr;
    Entry e;
    if (j < 9 * n_tp) {
        const int k = j / 9, q = j % 9;
        const int slot = items[k];
        e = soup[slot >> 6];
        w.aTri = (slot >> 3) & 7;
        w.bTri = slot & 7;
        w.aEdge = q / 3;
        w.bEdge = q % 3;
        w.out = sub + 15 * (size_t)k + 5 * w.aEdge + 2 + w.bEdge;
    } else {
        const int jp = j - 9 * n_tp;
        const int ei = find_entry(nn_off, n_conn, 9, jp);
        e = conn[ei];
        const int m = jp - 9 * nn_off[ei];
        const int na = ntris[e.na], nb = ntris[e.nb];
        const int ea = m / (3 * nb), eb = m % (3 * nb);
        w.aTri = ea / 3;
        w.aEdge = ea % 3;
        w.bTri = eb / 3;
        w.bEdge = eb % 3;
        const size_t item = 15 * (size_t)nn_off[ei] + 6 * (size_t)na * nb + m;
        w.out = cres + item;
        w.hit = chit + item;
    }
    w.pair = e.pair;
    w.na = e.na;
    w.nb = e.nb;
    return w;
}

__device__ __forceinline__ void record_no_contact(PrimResult* out, int32_t* hit) {
    store_prim(out, 1.0 / 0.0, mk(0, 0, 0), mk(0, 0, 0), 1.0);
    if (hit) *hit = 0;
}

// A warp's surviving tests appended to list (lane order within the warp,
// warps in arrival order; the tests' results do not depend on the order), the
// list's length in *count.
__device__ __forceinline__ void warp_append(int j, bool keep, int32_t* list, int32_t* count) {
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == 0) base = atomicAdd(count, __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (keep) list[base + __popc(m & ((1u << lane) - 1u))] = j;
}

__global__ void __launch_bounds__(kBlock) k_ccd_mask_pt(int n_tp, int n_total, const int32_t* __restrict__ items,
                                                        const Entry* __restrict__ soup, const Entry* __restrict__ conn,
                                                        const int32_t* __restrict__ nn_off, int n_conn,
                                                        const float* __restrict__ pm32,
                                                        const int32_t* __restrict__ ntris,
                                                        const float* __restrict__ tri32,
                                                        const float* __restrict__ search, PrimResult* __restrict__ sub,
                                                        PrimResult* __restrict__ cres, int32_t* __restrict__ chit,
                                                        int32_t* __restrict__ list, int32_t* __restrict__ count,
                                                        int use_bounds) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    bool keep = false;
    if (j < n_total) {
        const PtWork w = decode_pt(j, n_tp, items, soup, conn, nn_off, n_conn, ntris, sub, cres, chit);
        const float* pt = tri32 + ((size_t)w.pt_node * 8 + w.pt_tri) * 9 + 3 * w.pt_vert;
        const float* tv = tri32 + ((size_t)w.tri_node * 8 + w.tri_idx) * 9;
        const float *Cs = pm32_of(pm32, w.pair, w.mC), *Ce = pm32_of(pm32, w.pair, w.mC + 1);
        const float *tS = pm32_of(pm32, w.pair, w.mT), *tE = pm32_of(pm32, w.pair, w.mT + 1);
        float mag = 0.f, ps[3], pe[3], o[3];
        Box32 bp, bq, scratch;
        box_init(bp);
        box_init(bq);
        box_init(scratch);
        box_add(scratch, Cs, pt[0], pt[1], pt[2], ps, mag);
        box_add(scratch, Ce, pt[0], pt[1], pt[2], pe, mag);
        box_add(bp, tS, ps[0], ps[1], ps[2], o, mag);
        box_add(bp, tS, pe[0], pe[1], pe[2], o, mag);
        box_add(bp, tE, ps[0], ps[1], ps[2], o, mag);
        box_add(bp, tE, pe[0], pe[1], pe[2], o, mag);
        for (int v = 0; v < 3; v++) {
            box_add(bq, tS, tv[3 * v], tv[3 * v + 1], tv[3 * v + 2], o, mag);
            box_add(bq, tE, tv[3 * v], tv[3 * v + 1], tv[3 * v + 2], o, mag);
        }
        const float thr = search[w.pair];
        keep = !use_bounds || !(box_gap(bp, bq) > thr + (1e-3f + 4e-6f * (mag + thr)));  // NaN keeps the test
        if (!keep) record_no_contact(w.out, w.hit);
    }
    warp_append(j, keep, list, count);
}

__global__ void __launch_bounds__(kBlock) k_ccd_mask_ee(int n_tp, int n_total, const int32_t* __restrict__ items,
                                                        const Entry* __restrict__ soup, const Entry* __restrict__ conn,
                                                        const int32_t* __restrict__ nn_off, int n_conn,
                                                        const float* __restrict__ pm32,
                                                        const int32_t* __restrict__ ntris,
                                                        const float* __restrict__ tri32,
                                                        const float* __restrict__ search, PrimResult* __restrict__ sub,
                                                        PrimResult* __restrict__ cres, int32_t* __restrict__ chit,
                                                        int32_t* __restrict__ list, int32_t* __restrict__ count,
                                                        int use_bounds) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    bool keep = false;
    if (j < n_total) {
        const EeWork w = decode_ee(j, n_tp, items, soup, conn, nn_off, n_conn, ntris, sub, cres, chit);
        const float* ta = tri32 + ((size_t)w.na * 8 + w.aTri) * 9;
        const float* tb = tri32 + ((size_t)w.nb * 8 + w.bTri) * 9;
        const int a0 = w.aEdge, a1 = w.aEdge == 2 ? 0 : w.aEdge + 1;
        const int b0 = w.bEdge, b1 = w.bEdge == 2 ? 0 : w.bEdge + 1;
        float mag = 0.f, o[3];
        Box32 ba, bb;
        box_init(ba);
        box_init(bb);
        for (int m = 0; m < 2; m++) {
            const float* MA = pm32_of(pm32, w.pair, P32_AS + m);
            const float* MB = pm32_of(pm32, w.pair, P32_BS + m);
            box_add(ba, MA, ta[3 * a0], ta[3 * a0 + 1], ta[3 * a0 + 2], o, mag);
            box_add(ba, MA, ta[3 * a1], ta[3 * a1 + 1], ta[3 * a1 + 2], o, mag);
            box_add(bb, MB, tb[3 * b0], tb[3 * b0 + 1], tb[3 * b0 + 2], o, mag);
            box_add(bb, MB, tb[3 * b1], tb[3 * b1 + 1], tb[3 * b1 + 2], o, mag);
        }
        const float thr = search[w.pair];
        keep = !use_bounds || !(box_gap(ba, bb) > thr + (1e-3f + 4e-6f * (mag + thr)));
        if (!keep) record_no_contact(w.out, w.hit);
    }
    warp_append(j, keep, list, count);
}

__global__ void __launch_bounds__(kPrimBlock) k_prim_pt(int n_tp, int n_total, const int32_t* __restrict__ items,
                                                        const Entry* __restrict__ soup, const Entry* __restrict__ conn,
                                                        const int32_t* __restrict__ nn_off, int n_conn,
                                                        const double* __restrict__ pm,
                                                        const int32_t* __restrict__ ntris,
                                                        const double* __restrict__ tris,
                                                        const float* __restrict__ search,
                                                        PrimResult* __restrict__ sub, PrimResult* __restrict__ cres,
                                                        int32_t* __restrict__ chit, const int32_t* __restrict__ list,
                                                        const int32_t* __restrict__ n_list) {
    // work item list[kk] (every item when list is null)
    const int kk = blockIdx.x * blockDim.x + threadIdx.x;
    if (kk >= n_total || (n_list && kk >= *n_list)) return;
    const int j = list ? list[kk] : kk;
    if (j < 6 * n_tp) {
        const int k = j / 6, w = j % 6;
        const int slot = items[k];
        const Entry e = soup[slot >> 6];
        const double* M = pm + (size_t)PM_SIZE * e.pair;
        const Tri ta = load_tri(tris + (size_t)e.na * 72 + ((slot >> 3) & 7) * 9);
        const Tri tb = load_tri(tris + (size_t)e.nb * 72 + (slot & 7) * 9);
        const int i = w >> 1;
        const Ccd r = (w & 1) ? point_tri_ccd(tvert(tb, i), M + PM_BAS, M + PM_BAE, ta, M + PM_AS, M + PM_AE)
                              : point_tri_ccd(tvert(ta, i), M + PM_ABS, M + PM_ABE, tb, M + PM_BS, M + PM_BE);
        store_prim(sub + 15 * (size_t)k + 5 * i + (w & 1), r.dist, r.P, r.Q, r.toc);
        return;
    }
    const int jp = j - 6 * n_tp;
    const int ei = find_entry(nn_off, n_conn, 6, jp);
    const Entry e = conn[ei];
    const int l = jp - 6 * nn_off[ei];
    const int na = ntris[e.na], nb = ntris[e.nb];
    const double* M = pm + (size_t)PM_SIZE * e.pair;
    const double* pa = tris + (size_t)e.na * 72;
    const double* pb = tris + (size_t)e.nb * 72;
    const int n1 = 3 * na * nb;
    Ccd r;
    V3 A, B;
    if (l < n1) {
        const int vi = l / nb, jj = l % nb;
        r = point_tri_ccd(tvert(load_tri(pa + (vi / 3) * 9), vi % 3), M + PM_ABS, M + PM_ABE, load_tri(pb + jj * 9),
                          M + PM_BS, M + PM_BE);
        A = r.P;
        B = r.Q;
    } else {
        const int m = l - n1;
        const int vi = m / na, jj = m % na;
        r = point_tri_ccd(tvert(load_tri(pb + (vi / 3) * 9), vi % 3), M + PM_BAS, M + PM_BAE, load_tri(pa + jj * 9),
                          M + PM_AS, M + PM_AE);
        A = r.Q;
        B = r.P;
    }
    const size_t item = 15 * (size_t)nn_off[ei] + l;
    store_prim(cres + item, r.dist, A, B, r.toc);
    chit[item] = r.dist < (double)search[e.pair] ? 1 : 0;
}

// Edge-edge CCD in two kernels over the level's surviving tests.  GB300's
// FP64 pipe takes one warp instruction per 64 cycles per SM sub-partition
// (SMSP), dependent or not and whatever the number of active lanes (a
// division costs ~9 such slots, a square root ~10), and a level has only a
// few thousand surviving tests, so a warp's time is the instruction count of
// its longest lane and the level's time that of its slowest warp.  62% of the
// tests end within two Newton iterations and 20% run all ten, so:
//   k_ee_first   one test per lane: edges, FP64 box-gap skip, the bisection
//                (its cost is about two Newton iterations) or at most two
//                Newton iterations; the tests still running are saved and
//                listed.
//   k_ee_rest4   the listed tests on four lanes each (below): the remaining
//                iterations with about half the instructions per iteration,
//                on few enough warps that each has an SMSP to itself.
// Each test performs exactly the operations of edge_edge_ccd, in order.
// The first pass's iteration cap is the context setting D2G_TUNE_EE_FIRST_ITERS (default 2).
constexpr int kEeRec = 10;  // saved test: t, min_dist, P, Q, toc, iterations done (the edges are recomputed)
struct EeArgs {
    int n_tp, n_conn;
    const int32_t* items;
    const Entry* soup;
    const Entry* conn;
    const int32_t* nn_off;
    const int32_t* ntris;
    const float* search;
    PrimResult* sub;
    PrimResult* cres;
    int32_t* chit;
    const double* pm;
    const double* tris;
    double* rec;     // kEeRec per listed test
    int32_t* work;   // the listed test's work item
    int32_t* count;  // [0] listed tests
    int first_iters;  // Newton iterations in the first pass
    int certificates;  // conservative-advancement cut-off of the first pass (results unchanged)
    unsigned long long* ca_stats;  // [0] tests cut, [1] Newton iterations they did not run
};

// Conservative advancement over an edge-edge test's linear motion: every
// endpoint moves on a straight line, so the points of the two edges at any
// time t' are within V |t' - t| of where they were at time t, V being the
// largest relative endpoint displacement |(aE.i - aS.i) - (bE.j - bS.j)| over
// the four endpoint pairs (a point of an edge is a convex combination of its
// endpoints, and so is its displacement).  Every distance edgeEdgeCCD
// evaluates after time t is therefore at least dist(t) - V max(t, 1 - t).
// When that and every distance evaluated so far are at least the search
// distance (plus a margin far above FP64 rounding), the test cannot hit, and
// a sub-test that cannot hit is never the best of a triangle pair that hits:
// it is recorded as no contact, as the FP32 and box bounds record theirs.
__device__ __forceinline__ double ee_motion_bound(const Edge& aS, const Edge& aE, const Edge& bS, const Edge& bE) {
    const V3 da0 = aE.A - aS.A, da1 = aE.B - aS.B, db0 = bE.A - bS.A, db1 = bE.B - bS.B;
    const V3 d00 = da0 - db0, d01 = da0 - db1, d10 = da1 - db0, d11 = da1 - db1;
    const double m = fmax(fmax(dot(d00, d00), dot(d01, d01)), fmax(dot(d10, d10), dot(d11, d11)));
    return sqrt(m);
}

__device__ __forceinline__ void ee_store_at(const EeArgs& a, int o, float thr, const Ccd& r) {
    if (o < 0) {  // leaf-pair test: P and Q swapped (continuous_comparison.h:881-896)
        store_prim(a.cres + (-1 - o), r.dist, r.Q, r.P, r.toc);
        a.chit[-1 - o] = r.dist < (double)thr ? 1 : 0;
    } else {
        store_prim(a.sub + o, r.dist, r.P, r.Q, r.toc);
    }
}

__global__ void __launch_bounds__(kPrimBlock) k_ee_first(int n_total, const int32_t* __restrict__ list,
                                                         const int32_t* __restrict__ n_list,
                                                         const double* __restrict__ pm,
                                                         const double* __restrict__ tris, EeArgs a) {
    const int kk = blockIdx.x * blockDim.x + threadIdx.x;
    bool keep = false;
    int o = 0;
    float thr = 0.f;
    Edge aS, aE, bS, bE;
    Ccd r;
    double min_dist = DBL_MAX, t = 0.0;
    int iters = 0;
    if (kk < n_total && kk < *n_list) {
        const int j = list[kk];
        const EeWork w = decode_ee(j, a.n_tp, a.items, a.soup, a.conn, a.nn_off, a.n_conn, a.ntris, a.sub, a.cres,
                                   a.chit);
        o = w.hit ? -1 - (int)(w.out - a.cres) : (int)(w.out - a.sub);
        thr = a.search[w.pair];
        const double* M = pm + (size_t)PM_SIZE * w.pair;
        const Edge ea = tedge(load_tri(tris + (size_t)w.na * 72 + w.aTri * 9), w.aEdge);
        const Edge eb = tedge(load_tri(tris + (size_t)w.nb * 72 + w.bTri * 9), w.bEdge);
        aS.A = xform_rigid(ea.A, M + PM_AS);
        aS.B = xform_rigid(ea.B, M + PM_AS);
        aE.A = xform_rigid(ea.A, M + PM_AE);
        aE.B = xform_rigid(ea.B, M + PM_AE);
        bS.A = xform_rigid(eb.A, M + PM_BS);
        bS.B = xform_rigid(eb.B, M + PM_BS);
        bE.A = xform_rigid(eb.A, M + PM_BE);
        bE.B = xform_rigid(eb.B, M + PM_BE);
        // Every distance edgeEdgeCCD can return is between points of the two
        // swept segments, which lie in the boxes of their four endpoint
        // positions.  A box gap beyond the search distance (plus 1e-7 m, far
        // above FP64 rounding at scene scale) means no hit, and such a
        // sub-test can never be the best of a triangle pair that hits: skip
        // it, recording +inf.
        const double lim = (double)thr + 1e-7;
        double gap2 = 0.0;
        {
            const double ax[4] = {aS.A.x, aS.B.x, aE.A.x, aE.B.x}, ay[4] = {aS.A.y, aS.B.y, aE.A.y, aE.B.y},
                         az[4] = {aS.A.z, aS.B.z, aE.A.z, aE.B.z};
            const double bx[4] = {bS.A.x, bS.B.x, bE.A.x, bE.B.x}, by[4] = {bS.A.y, bS.B.y, bE.A.y, bE.B.y},
                         bz[4] = {bS.A.z, bS.B.z, bE.A.z, bE.B.z};
            const double* av[3] = {ax, ay, az};
            const double* bv[3] = {bx, by, bz};
#pragma unroll
            for (int d = 0; d < 3; d++) {
                const double alo = fmin(fmin(av[d][0], av[d][1]), fmin(av[d][2], av[d][3]));
                const double ahi = fmax(fmax(av[d][0], av[d][1]), fmax(av[d][2], av[d][3]));
                const double blo = fmin(fmin(bv[d][0], bv[d][1]), fmin(bv[d][2], bv[d][3]));
                const double bhi = fmax(fmax(bv[d][0], bv[d][1]), fmax(bv[d][2], bv[d][3]));
                const double g = fmax(blo - ahi, alo - bhi);
                if (g > 0.0) gap2 = gap2 + g * g;
            }
        }
        if (gap2 > lim * lim) {
            record_no_contact(w.out, w.hit);
        } else {
            r.P = mk(0, 0, 0);
            r.Q = mk(0, 0, 0);
            r.toc = 0.0;
            const double dot_start = ee_coplanarity(aS, bS);
            const double dot_end = ee_coplanarity(aE, bE);
            bool bisected = false;
            if (dot_start * dot_end < 0.0) {
                min_dist = ee_bisect(aS, aE, bS, bE, dot_start, r);
                bisected = true;
            }
            bool done = !(min_dist > 1e-8), cut = false;
            if (!done && !bisected) {
                double V = 0.0, lim = 0.0;
                if (a.certificates) {
                    V = ee_motion_bound(aS, aE, bS, bE);
                    const double mag = fmax(fmax(fmax(fabs(aS.A.x), fabs(aS.A.y)), fabs(aS.A.z)),
                                            fmax(fmax(fabs(bS.A.x), fabs(bS.A.y)), fabs(bS.A.z)));
                    lim = ((double)thr + 1e-6) + 1e-12 * (mag + V);
                }
                for (; iters < a.first_iters; iters++) {
                    const double t_at = t;
                    double d_at;
                    if (ee_newton_iter(aS, aE, bS, bE, t, min_dist, r, &d_at)) {
                        done = true;
                        break;
                    }
                    if (a.certificates && min_dist >= lim && d_at - V * fmax(t_at, 1.0 - t_at) >= lim) {
                        cut = true;
                        iters++;
                        break;
                    }
                }
            }
            if (cut) {
                record_no_contact(w.out, w.hit);
                atomicAdd(a.ca_stats, 1ull);
                atomicAdd(a.ca_stats + 1, (unsigned long long)(kEeNewtonIters - iters));
            } else if (done) {
                r.dist = min_dist;
                ee_store_at(a, o, thr, r);
            } else {
                keep = true;  // the remaining iterations run in k_ee_rest4
            }
        }
    }
    // warp-aggregated append of the tests still running
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (m) {
        const int lane = threadIdx.x & 31, lead = __ffs(m) - 1;
        int base = 0;
        if (lane == lead) base = atomicAdd(a.count, __popc(m));
        base = __shfl_sync(0xffffffffu, base, lead);
        if (keep) {
            const int slot = base + __popc(m & ((1u << lane) - 1u));
            double* R = a.rec + (size_t)kEeRec * slot;
            const double st[kEeRec] = {t, min_dist, r.P.x, r.P.y, r.P.z, r.Q.x, r.Q.y, r.Q.z, r.toc, (double)iters};
#pragma unroll
            for (int k = 0; k < kEeRec; k++) R[k] = st[k];
            a.work[slot] = list[kk];
        }
    }
}

// ---- the Newton phase on four lanes per test ------------------------------
// GB300 issues an FP64 warp instruction at the same cost whatever the number
// of active lanes, and a level has far fewer surviving edge-edge tests than
// the GPU has lanes, so a test's time is the number of FP64 instructions on
// its path.  Here each test runs on a quad of lanes: lane c < 3 holds
// component c of every point (lane 3 mirrors x), vector operations are one
// instruction for all three components, a dot product is one multiply and the
// two adds (x + y) + z of the reference's order, and independent divisions
// share one instruction stream on different lanes.  Scalars are computed
// identically on all four lanes, so every branch is uniform within a quad.
// Every value is produced by the same operations, in the same order, as in
// edge_edge_ccd.
struct Quad {
    unsigned m;  // the quad's lanes
    int base;    // its first lane
    int c;       // this lane's component (3: mirror of x)
};
__device__ __forceinline__ double q_at(const Quad& q, double v, int k) { return __shfl_sync(q.m, v, q.base + k); }
__device__ __forceinline__ double q_dot(const Quad& q, double a, double b) {
    const double p = a * b;
    const double px = q_at(q, p, 0), py = q_at(q, p, 1), pz = q_at(q, p, 2);
    return (px + py) + pz;
}
__device__ __forceinline__ double q_lerp(double A, double B, double t) {
    const double u = 1 - t;
    return A * u + B * t;
}
// components differ anywhere (vne)
__device__ __forceinline__ bool q_ne(const Quad& q, double a, double b) {
    const unsigned bal = __ballot_sync(q.m, q.c < 3 && a != b);
    return ((bal >> q.base) & 7u) != 0u;
}
// edge_constrain(A, B, pos)
__device__ __forceinline__ double q_constrain(const Quad& q, double A, double B, double pos) {
    const double ba = B - A;
    const double t = q_dot(q, pos - A, ba) / q_dot(q, ba, ba);
    return q_lerp(A, B, clamp01(t));
}
// edge_closest(SA, SB, EA, EB, P, Q): one component per lane
__device__ __forceinline__ double q_edge_closest(const Quad& q, double SA, double SB, double EA, double EB, double& P,
                                                 double& Qo) {
    const double segDC = EB - EA;
    const double lineDirSqrMag = q_dot(q, segDC, segDC);
    const double segAC = SA - EA;
    const double segBC = SB - EA;
    const double nA = q_dot(q, segAC, segDC), nB = q_dot(q, segBC, segDC);
    const double s2 = ((q.c & 1) ? nB : nA) / lineDirSqrMag;  // lanes 0, 2: A; 1, 3: B
    const double sA = q_at(q, s2, 0), sB = q_at(q, s2, 1);
    const double inPlaneA = SA - sA * segDC;
    const double inPlaneB = SB - sB * segDC;
    const double inPlaneBA = inPlaneB - inPlaneA;
    double t = q_dot(q, EA - inPlaneA, inPlaneBA) / q_dot(q, inPlaneBA, inPlaneBA);
    t = q_ne(q, inPlaneA, inPlaneB) ? t : 0.0;
    const double segABtoLineCD = q_lerp(SA, SB, clamp01(t));
    const double segCDtoSegAB = q_constrain(q, EA, EB, segABtoLineCD);
    const double segABtoSegCD = q_constrain(q, SA, SB, segCDtoSegAB);
    Qo = segCDtoSegAB;
    P = segABtoSegCD;
    const double d = Qo - P;
    return sqrt(q_dot(q, d, d));
}

__global__ void __launch_bounds__(kBlock) k_ee_rest4(EeArgs a) {
    const int n = a.count[0];
    Quad q;
    q.m = 0xFu << (threadIdx.x & 28);
    q.base = threadIdx.x & 28;
    q.c = threadIdx.x & 3;
    const int comp = q.c < 3 ? q.c : 0;
    const int n_quads = (gridDim.x * blockDim.x) >> 2;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 2; i < n; i += n_quads) {
        const double* R = a.rec + (size_t)kEeRec * i;
        const EeWork w = decode_ee(a.work[i], a.n_tp, a.items, a.soup, a.conn, a.nn_off, a.n_conn, a.ntris, a.sub,
                                   a.cres, a.chit);
        // this lane's component of the edges' endpoints at start and end
        // (xform_rigid's row `comp`, the same operations in the same order)
        const double* M = a.pm + (size_t)PM_SIZE * w.pair;
        const double* ta = a.tris + (size_t)w.na * 72 + w.aTri * 9;
        const double* tb = a.tris + (size_t)w.nb * 72 + w.bTri * 9;
        const double* va0 = ta + 3 * w.aEdge;
        const double* va1 = ta + 3 * (w.aEdge == 2 ? 0 : w.aEdge + 1);
        const double* vb0 = tb + 3 * w.bEdge;
        const double* vb1 = tb + 3 * (w.bEdge == 2 ? 0 : w.bEdge + 1);
        auto row = [&](const double* T, const double* v) {
            const double* m = T + 4 * comp;
            return ((m[0] * v[0] + m[1] * v[1]) + m[2] * v[2]) + m[3] * 1.0;
        };
        const double aSA = row(M + PM_AS, va0), aSB = row(M + PM_AS, va1);
        const double aEA = row(M + PM_AE, va0), aEB = row(M + PM_AE, va1);
        const double bSA = row(M + PM_BS, vb0), bSB = row(M + PM_BS, vb1);
        const double bEA = row(M + PM_BE, vb0), bEB = row(M + PM_BE, vb1);
        double t = R[0], min_dist = R[1];
        double rP = R[2 + comp], rQ = R[5 + comp], toc = R[8];
        for (int iter = (int)R[9]; iter < kEeNewtonIters; iter++) {
            const double atA = q_lerp(aSA, aEA, t), atB = q_lerp(aSB, aEB, t);
            const double btA = q_lerp(bSA, bEA, t), btB = q_lerp(bSB, bEB, t);
            double P, Qv;
            const double dist = q_edge_closest(q, atA, atB, btA, btB, P, Qv);
            if (dist < min_dist) {
                min_dist = dist;
                rP = P;
                rQ = Qv;
                toc = t;
            }
            // edge_project(atA, atB, P) and edge_project(btA, btB, Q), divided on lanes 0 / 1
            const double AB = atB - atA, CD = btB - btA;
            const double na = q_dot(q, P - atA, AB), da = q_dot(q, AB, AB);
            const double nb = q_dot(q, Qv - btA, CD), db = q_dot(q, CD, CD);
            const double pr = ((q.c & 1) ? nb : na) / ((q.c & 1) ? db : da);
            const double pa = q_at(q, pr, 0), pb = q_at(q, pr, 1);
            // ee_newton_terms, component per lane
            const double omt = 1 - t, ompa = 1 - pa, ompb = 1 - pb, pbm1 = pb - 1;
            const double f = ((pa * (aEB + aSB * omt) - pb * (bEB + bSB * omt)) + ompa * (aEA * t + aSA * omt)) -
                             ompb * (bEA * t + bSA * omt);
            const double g = ((-2 * aSB * pa + 2 * bSB * pb) + 2 * ompa * (aEA - aSA)) + 2 * (bEA - bSA) * pbm1;
            const double h = ((-aSB * pa / 2 + bSB * pb / 2) + ompa * (aEA - aSA) / 2) + (bEA - bSA) * pbm1 / 2;
            const double gf2 = g * f / 2, gh = g * h, ff = f * f;
            const double gf = (q_at(q, gf2, 0) + q_at(q, gf2, 1)) + q_at(q, gf2, 2);
            const double S = (q_at(q, ff, 0) + q_at(q, ff, 1)) + q_at(q, ff, 2);
            const double GH = (q_at(q, gh, 0) + q_at(q, gh, 1)) + q_at(q, gh, 2);
            const double sS = sqrt(S);
            // gf / sS, GH / sS and (-gf * gf) / pow15(S) on lanes 0, 1, 2
            const double num = q.c == 1 ? GH : (q.c == 2 ? (-gf) * gf : gf);
            const double den = q.c == 2 ? m_pow15(S) : sS;
            const double quo = num / den;
            const double t_diff = q_at(q, quo, 0);
            const double t_diff2 = q_at(q, quo, 1) + q_at(q, quo, 2);
            const double t_prev = t;
            t = t - t_diff / t_diff2;
            t = clamp01(t);
            if (t == t_prev || t != t) break;
        }
        const double Px = q_at(q, rP, 0), Py = q_at(q, rP, 1), Pz = q_at(q, rP, 2);
        const double Qx = q_at(q, rQ, 0), Qy = q_at(q, rQ, 1), Qz = q_at(q, rQ, 2);
        if (q.c == 0) {
            Ccd r;
            r.dist = min_dist;
            r.P = mk(Px, Py, Pz);
            r.Q = mk(Qx, Qy, Qz);
            r.toc = toc;
            ee_store_at(a, w.hit ? -1 - (int)(w.out - a.cres) : (int)(w.out - a.sub), a.search[w.pair], r);
        }
    }
}

// triTriCCDLinear's sequential (dist, toc) selection over its 15 sub-tests
// (continuous_comparison.h:682-778), then the soup hit test (:817) and the
// final-contact flag (a hit between two leaves, as k_final_flags sets it).
__global__ void k_soup_fold(int K, const int32_t* __restrict__ items, const Entry* __restrict__ soup,
                            const PrimResult* __restrict__ sub, const float* __restrict__ search,
                            PrimResult* __restrict__ res, int32_t* __restrict__ hit,
                            int32_t* __restrict__ entry_hits, const int4* __restrict__ nodes,
                            int32_t* __restrict__ flags) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    PrimResult best;
    best.dist = 1.0 / 0.0;
    best.P[0] = best.P[1] = best.P[2] = 0.0;
    best.Q[0] = best.Q[1] = best.Q[2] = 0.0;
    best.toc = 1.0;
    for (int s = 0; s < 15; s++) {
        const PrimResult c = sub[15 * (size_t)k + s];
        if (c.dist < best.dist || (c.dist == best.dist && c.toc < best.toc)) best = c;
    }
    res[k] = best;
    const int slot = items[k];
    const Entry e = soup[slot >> 6];
    const int h = best.dist < (double)search[e.pair] ? 1 : 0;
    hit[k] = h;
    if (h) atomicAdd(&entry_hits[slot >> 6], 1);
    flags[k] = (h && !ld_node(nodes, e.na).z && !ld_node(nodes, e.nb).z) ? 1 : 0;
}

// ----------------------------------------------------------- discrete -----
// All 64 slots of a node pair: triangle distance at the future poses and the
// hit test dist < float(search) + eps_a + eps_b (comparison_dist.h:223-236).
// Candidate slots of the discrete narrow phase.  A (node pair, ta, tb) slot
// can only hit (comparison_dist.h:231-233) when the triangles are closer than
// thr = search + eps_a + eps_b.  Lower bounds on that distance: the bounding
// spheres' |c_a - c_b| - r_a - r_b (centroid, radius rounded up), the gap
// between the boxes of the transformed triangles and, for slots those keep,
// the gaps along the eleven separating axes (two face normals, nine edge-edge
// cross products).  The largest is evaluated in FP32 and a slot is dropped
// only when it exceeds thr by a margin
// (1 mm plus 4e-6 of the magnitudes involved) far above the FP32 rounding of
// the bound and the FP64 rounding of the exact test, so every slot that hits
// survives.  Dropped slots produce nothing in the reference
// either.  One thread per slot; per warp a survivor mask and count.  The valid
// slots (ta < ntris_a, tb < ntris_b) are counted for the statistics.
__global__ void __launch_bounds__(kBlock) k_np_mask(int n_slots, const Entry* __restrict__ front,
                                                    const float* __restrict__ pm32, const int32_t* __restrict__ ntris,
                                                    const float4* __restrict__ sph, const float* __restrict__ tri32,
                                                    const float* __restrict__ eps_up,
                                                    const float* __restrict__ search, uint32_t* __restrict__ mask,
                                                    int32_t* __restrict__ cnt, int32_t* __restrict__ tri_pairs,
                                                    int use_bounds) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool valid = false, keep = false;
    if (i < n_slots) {
        const Entry e = front[i >> 6];
        const int ta = (i >> 3) & 7, tb = i & 7;
        valid = ta < ntris[e.na] && tb < ntris[e.nb];
        if (valid) {
            const float* A = pm32 + 24 * (size_t)e.pair;
            const float* B = A + 12;
            const float4 sa = sph[(size_t)e.na * 8 + ta], sb = sph[(size_t)e.nb * 8 + tb];
            const float dx = (A[0] * sa.x + A[1] * sa.y + A[2] * sa.z + A[3]) -
                             (B[0] * sb.x + B[1] * sb.y + B[2] * sb.z + B[3]);
            const float dy = (A[4] * sa.x + A[5] * sa.y + A[6] * sa.z + A[7]) -
                             (B[4] * sb.x + B[5] * sb.y + B[6] * sb.z + B[7]);
            const float dz = (A[8] * sa.x + A[9] * sa.y + A[10] * sa.z + A[11]) -
                             (B[8] * sb.x + B[9] * sb.y + B[10] * sb.z + B[11]);
            const float thr = search[e.pair] + eps_up[(size_t)e.na * 8 + ta] + eps_up[(size_t)e.nb * 8 + tb];
            const float mag = fabsf(A[3]) + fabsf(A[7]) + fabsf(A[11]) + fabsf(B[3]) + fabsf(B[7]) + fabsf(B[11]) +
                              fabsf(sa.x) + fabsf(sa.y) + fabsf(sa.z) + fabsf(sb.x) + fabsf(sb.y) + fabsf(sb.z) +
                              sa.w + sb.w + thr;
            float lb = sqrtf(dx * dx + dy * dy + dz * dz) - sa.w - sb.w;
            // the gap between the transformed triangles' boxes is a second lower bound
            const float* va = tri32 + ((size_t)e.na * 8 + ta) * 9;
            const float* vb = tri32 + ((size_t)e.nb * 8 + tb) * 9;
            float wa[3][3], wb[3][3];  // [vertex][axis]
#pragma unroll
            for (int v = 0; v < 3; v++)
#pragma unroll
                for (int r = 0; r < 3; r++) {
                    wa[v][r] = A[4 * r] * va[3 * v] + A[4 * r + 1] * va[3 * v + 1] + A[4 * r + 2] * va[3 * v + 2] +
                               A[4 * r + 3];
                    wb[v][r] = B[4 * r] * vb[3 * v] + B[4 * r + 1] * vb[3 * v + 1] + B[4 * r + 2] * vb[3 * v + 2] +
                               B[4 * r + 3];
                }
            float gap2 = 0.f;
#pragma unroll
            for (int r = 0; r < 3; r++) {
                const float alo = fminf(fminf(wa[0][r], wa[1][r]), wa[2][r]);
                const float ahi = fmaxf(fmaxf(wa[0][r], wa[1][r]), wa[2][r]);
                const float blo = fminf(fminf(wb[0][r], wb[1][r]), wb[2][r]);
                const float bhi = fmaxf(fmaxf(wb[0][r], wb[1][r]), wb[2][r]);
                const float g = fmaxf(blo - ahi, alo - bhi);
                if (g > 0.f) gap2 += g * g;
            }
            lb = fmaxf(lb, sqrtf(gap2));
            const float lim = thr + (1e-3f + 4e-6f * mag);
            if (!(lb > lim)) {
                // Separating axes: along any direction n the distance is at
                // least the gap between the projections divided by |n|,
                // whatever n is, so n computed in FP32 still bounds; the two
                // face normals and the nine edge-edge cross products.
                auto axis_gap = [&](float nx, float ny, float nz) {
                    const float nn = sqrtf(nx * nx + ny * ny + nz * nz);
                    if (!(nn > 1e-20f)) return 0.f;
                    float a0 = 3.4e38f, a1 = -3.4e38f, b0 = 3.4e38f, b1 = -3.4e38f;
#pragma unroll
                    for (int v = 0; v < 3; v++) {
                        const float pa = wa[v][0] * nx + wa[v][1] * ny + wa[v][2] * nz;
                        const float pb = wb[v][0] * nx + wb[v][1] * ny + wb[v][2] * nz;
                        a0 = fminf(a0, pa);
                        a1 = fmaxf(a1, pa);
                        b0 = fminf(b0, pb);
                        b1 = fmaxf(b1, pb);
                    }
                    return fmaxf(b0 - a1, a0 - b1) / nn;
                };
                float ea[3][3], eb[3][3];
#pragma unroll
                for (int k = 0; k < 3; k++)
#pragma unroll
                    for (int r = 0; r < 3; r++) {
                        ea[k][r] = wa[(k + 1) % 3][r] - wa[k][r];
                        eb[k][r] = wb[(k + 1) % 3][r] - wb[k][r];
                    }
                lb = fmaxf(lb, axis_gap(ea[0][1] * ea[1][2] - ea[0][2] * ea[1][1], ea[0][2] * ea[1][0] - ea[0][0] * ea[1][2],
                                        ea[0][0] * ea[1][1] - ea[0][1] * ea[1][0]));
                lb = fmaxf(lb, axis_gap(eb[0][1] * eb[1][2] - eb[0][2] * eb[1][1], eb[0][2] * eb[1][0] - eb[0][0] * eb[1][2],
                                        eb[0][0] * eb[1][1] - eb[0][1] * eb[1][0]));
#pragma unroll
                for (int x = 0; x < 3; x++)
#pragma unroll
                    for (int y = 0; y < 3; y++)
                        lb = fmaxf(lb, axis_gap(ea[x][1] * eb[y][2] - ea[x][2] * eb[y][1],
                                                ea[x][2] * eb[y][0] - ea[x][0] * eb[y][2],
                                                ea[x][0] * eb[y][1] - ea[x][1] * eb[y][0]));
            }
            keep = !use_bounds || !(lb > lim);  // NaN keeps the slot
        }
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    const unsigned v = __ballot_sync(0xffffffffu, valid);
    if ((threadIdx.x & 31) == 0 && i < n_slots) {
        mask[i >> 5] = m;
        cnt[i >> 5] = __popc(m);
        if (tri_pairs && v) atomicAdd(tri_pairs, __popc(v));  // statistics only
    }
}

// Ordered compaction of the surviving slots (slot order = the reference's
// triangle-pair order within each node pair).
__global__ void k_np_items(int n_slots, const uint32_t* __restrict__ mask, const int32_t* __restrict__ off,
                           int32_t* __restrict__ items) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_slots) return;
    const unsigned m = mask[i >> 5];
    const int lane = i & 31;
    if ((m >> lane) & 1u) items[off[i >> 5] + __popc(m & ((1u << lane) - 1u))] = i;
}

__global__ void __launch_bounds__(kBlock) k_np(int n_slots, const Entry* __restrict__ front,
                                               const int32_t* __restrict__ pairs, const double* __restrict__ pm,
                                               const int32_t* __restrict__ ntris, const double* __restrict__ tris,
                                               const double* __restrict__ eps, const double* __restrict__ inner_eps,
                                               const double* __restrict__ geo_eps,
                                               const float* __restrict__ search, PrimResult* __restrict__ res,
                                               double* __restrict__ res_eps, int32_t* __restrict__ hit,
                                               int32_t* __restrict__ entry_hits, const int32_t* __restrict__ items,
                                               const int32_t* __restrict__ n_items) {
    // Work item k tests slot items[k] (all slots when items is null); results
    // are stored per item.
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_slots) return;
    if (n_items && k >= *n_items) {
        hit[k] = 0;
        return;
    }
    const int i = items ? items[k] : k;
    const Entry e = front[i >> 6];
    const int ta = (i >> 3) & 7, tb = i & 7;
    int h = 0;
    if (ta < ntris[e.na] && tb < ntris[e.nb]) {
        const double* M = pm + 32 * (size_t)e.pair;
        const Tri A = tri_xform_rigid(load_tri(tris + (size_t)e.na * 72 + ta * 9), M);
        const Tri B = tri_xform_rigid(load_tri(tris + (size_t)e.nb * 72 + tb * 9), M + 16);
        V3 P, Q;
        const double d = tri_tri_dist(A, B, P, Q);
        const double ea = eps[(size_t)e.na * 8 + ta], eb = eps[(size_t)e.nb * 8 + tb];
        h = d < ((double)search[e.pair] + ea) + eb ? 1 : 0;
        if (h) {
            const int a = pairs[2 * e.pair], b = pairs[2 * e.pair + 1];
            put_result(res[k], d, P, Q, 0.0);
            res_eps[4 * (size_t)k + 0] = geo_eps[a] + ea;
            res_eps[4 * (size_t)k + 1] = geo_eps[b] + eb;
            res_eps[4 * (size_t)k + 2] = inner_eps[(size_t)e.na * 8 + ta];
            res_eps[4 * (size_t)k + 3] = inner_eps[(size_t)e.nb * 8 + tb];
            atomicAdd(&entry_hits[i >> 6], 1);
        }
    }
    hit[k] = h;
}

// Frontier entries of one body pair (pair index 0) from a list of node pairs.
__global__ void k_bucket_entries(int n, const int32_t* __restrict__ node_pairs, Entry* __restrict__ front) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Entry e;
    e.pair = 0;
    e.na = node_pairs[2 * i];
    e.nb = node_pairs[2 * i + 1];
    front[i] = e;
}

// --------------------------------------------------- finals / expansion ----
// Final-contact flag of each result: a hit inside a leaf-leaf node pair.
// `slot_entry` maps a result to its entry: item >> 6 through `items` when
// given (soup stage), else the slot index >> 6 (discrete stage).
__global__ void k_final_flags(int n, const int32_t* __restrict__ items, const Entry* __restrict__ front,
                              const int4* __restrict__ nodes, const int32_t* __restrict__ hit,
                              int32_t* __restrict__ flags) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int slot = items ? items[k] : k;
    int f = 0;
    if (hit[k]) {
        const Entry e = front[slot >> 6];
        f = (!ld_node(nodes, e.na).z && !ld_node(nodes, e.nb).z) ? 1 : 0;
    }
    flags[k] = f;
}

// Append flagged results as contact records (collision_detection/contact.h).
__global__ void k_emit(int n, const int32_t* __restrict__ flags, const int32_t* __restrict__ off,
                       const int32_t* __restrict__ items, int slot_shift, const Entry* __restrict__ front,
                       const int32_t* __restrict__ conn_off, int n_conn, const int32_t* __restrict__ pairs,
                       const PrimResult* __restrict__ res, const double* __restrict__ res_eps,
                       const double* __restrict__ geo_eps, double* __restrict__ rec, int32_t* __restrict__ rec_pair,
                       int base) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || !flags[k]) return;
    int ei;
    if (conn_off) {
        int lo = 0, hi = n_conn;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (conn_off[mid] <= k)
                lo = mid;
            else
                hi = mid;
        }
        ei = lo;
    } else {
        ei = (items ? items[k] : k) >> slot_shift;
    }
    const Entry e = front[ei];
    const int a = pairs[2 * e.pair], b = pairs[2 * e.pair + 1];
    const PrimResult& r = res[k];
    double* o = rec + 14 * (size_t)(base + off[k]);
    o[0] = r.P[0];
    o[1] = r.P[1];
    o[2] = r.P[2];
    o[3] = r.Q[0];
    o[4] = r.Q[1];
    o[5] = r.Q[2];
    if (res_eps) {
        o[6] = res_eps[4 * (size_t)k + 0];
        o[7] = res_eps[4 * (size_t)k + 1];
        o[8] = res_eps[4 * (size_t)k + 2];
        o[9] = res_eps[4 * (size_t)k + 3];
    } else {
        o[6] = geo_eps[a];
        o[7] = geo_eps[b];
        o[8] = 0.0;
        o[9] = 0.0;
    }
    o[10] = r.toc;
    o[11] = (double)a;
    o[12] = (double)b;
    o[13] = 0.0;
    rec_pair[base + off[k]] = e.pair;
}

// Expansion rule of full_tree_comparison.h:27-59: leaf-leaf keeps its hits,
// otherwise the shallower inner side (b on ties, the inner one when the other
// is a leaf) is replaced by its children.  `split` separates children into
// the soup (some inner node) and connected (both leaves) frontiers.
__global__ void k_expand_count(int n, const Entry* __restrict__ front, const int32_t* __restrict__ entry_hits,
                               const int4* __restrict__ nodes, int split, int32_t* __restrict__ cnt_s,
                               int32_t* __restrict__ cnt_c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int s = 0, c = 0;
    if (entry_hits[i] > 0) {
        const Entry e = front[i];
        const int4 A = ld_node(nodes, e.na), B = ld_node(nodes, e.nb);
        int rule;
        if (!A.z && !B.z)
            rule = 0;
        else if (!A.z)
            rule = 2;
        else if (!B.z)
            rule = 1;
        else
            rule = A.w < B.w ? 1 : 2;
        if (rule) {
            const int4 P = rule == 1 ? A : B;
            for (int ch = 0; ch < P.y; ch++) {
                const int ga = rule == 1 ? P.x + ch : e.na;
                const int gb = rule == 1 ? e.nb : P.x + ch;
                const bool inner = ld_node(nodes, ga).z || ld_node(nodes, gb).z;
                if (!split || inner)
                    s++;
                else
                    c++;
            }
        }
    }
    cnt_s[i] = s;
    cnt_c[i] = c;
}

__global__ void k_expand_write(int n, const Entry* __restrict__ front, const int32_t* __restrict__ entry_hits,
                               const int4* __restrict__ nodes, int split, const int32_t* __restrict__ off_s,
                               const int32_t* __restrict__ off_c, Entry* __restrict__ next_s,
                               Entry* __restrict__ next_c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || entry_hits[i] <= 0) return;
    const Entry e = front[i];
    const int4 A = ld_node(nodes, e.na), B = ld_node(nodes, e.nb);
    int rule;
    if (!A.z && !B.z)
        rule = 0;
    else if (!A.z)
        rule = 2;
    else if (!B.z)
        rule = 1;
    else
        rule = A.w < B.w ? 1 : 2;
    if (!rule) return;
    const int4 P = rule == 1 ? A : B;
    int s = off_s[i], c = off_c[i];
    for (int ch = 0; ch < P.y; ch++) {
        Entry x;
        x.pair = e.pair;
        x.na = rule == 1 ? P.x + ch : e.na;
        x.nb = rule == 1 ? e.nb : P.x + ch;
        const bool inner = ld_node(nodes, x.na).z || ld_node(nodes, x.nb).z;
        if (!split || inner)
            next_s[s++] = x;
        else
            next_c[c++] = x;
    }
}

// ---------------------------------------------------------- output sort ----
__global__ void k_iota(int n, int32_t* __restrict__ v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = i;
}
__global__ void k_count_pairs(int n, int p0, int n_pairs, const int32_t* __restrict__ rec_pair,
                              int32_t* __restrict__ cnt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int p = rec_pair[i] - p0;
    if (p >= 0 && p < n_pairs) atomicAdd(&cnt[p], 1);
}
__global__ void k_gather(int n, const int32_t* __restrict__ idx, const double* __restrict__ in,
                         double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int j = idx[i];
    if (j < 0 || j >= n) return;
    const double* s = in + 14 * (size_t)j;
    double* d = out + 14 * (size_t)i;
#pragma unroll
    for (int k = 0; k < 14; k++) d[k] = s[k];
}

// Future state left on each body: the projection of the last pair containing it.
__global__ void k_last_pair(int n, const int32_t* __restrict__ pairs, int32_t* __restrict__ last) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    atomicMax(&last[pairs[2 * p]], p);
    atomicMax(&last[pairs[2 * p + 1]], p);
}
__global__ void k_write_fut(int n, const int32_t* __restrict__ pairs, const int32_t* __restrict__ last,
                            const double* __restrict__ pfut, double* __restrict__ fut) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int a = pairs[2 * p], b = pairs[2 * p + 1];
    if (last[a] == p)
        for (int k = 0; k < 14; k++) fut[14 * (size_t)a + k] = pfut[28 * (size_t)p + k];
    if (last[b] == p)
        for (int k = 0; k < 14; k++) fut[14 * (size_t)b + k] = pfut[28 * (size_t)p + 14 + k];
}

__global__ void k_fill(int n, int32_t* __restrict__ v, int32_t x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = x;
}

// ------------------------------------------------------------ host side ----
#define LAUNCH(kern, n, ...)                                                \
    do {                                                                    \
        kern<<<nblocks(n), kBlock, 0, ctx->stream>>>(__VA_ARGS__);          \
        ctx->eng.launches++;                                                \
    } while (0)

// Profiling mode: an event pair around a dominant kernel's launch; the
// elapsed times are collected at the next stream synchronisation.
int prof_begin(d2g_ctx* ctx, int kind, long long items, cudaStream_t st = nullptr) {
    Engine& E = ctx->eng;
    if (!E.profiling) return -1;
    cudaEvent_t ev[2];
    for (int i = 0; i < 2; i++) {
        if (!E.event_pool.empty()) {
            ev[i] = E.event_pool.back();
            E.event_pool.pop_back();
        } else if (cudaEventCreate(&ev[i]) != cudaSuccess) {
            return -1;
        }
    }
    cudaEventRecord(ev[0], st ? st : ctx->stream);
    E.pending.push_back(Engine::Pending{kind, ev[0], ev[1], items});
    return (int)E.pending.size() - 1;
}
void prof_end(d2g_ctx* ctx, int idx, cudaStream_t st = nullptr) {
    if (idx >= 0) cudaEventRecord(ctx->eng.pending[idx].e1, st ? st : ctx->stream);
}
// Call only after the stream has been synchronised.
void prof_collect(d2g_ctx* ctx) {
    Engine& E = ctx->eng;
    for (auto& p : E.pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p.e0, p.e1) == cudaSuccess) {
            E.prof_ms[p.kind] += ms;
            E.prof_launches[p.kind] += 1;
            E.prof_items[p.kind] += p.items;
        }
        E.event_pool.push_back(p.e0);
        E.event_pool.push_back(p.e1);
    }
    E.pending.clear();
}

// Exclusive prefix sum of in[0..n) into out[0..n], out[n] = total.
// Exclusive prefix sums of up to two small int32 arrays in one launch, one
// 1024-thread block per array: out[0..n] with out[n] = total.  The array is
// staged in shared memory in chunks of kScanChunk (coalesced), each thread
// sums its kScanPer contiguous elements, and a shuffle scan over the thread
// sums gives every thread its offset.
constexpr int kScanThreads = 1024, kScanPer = 8, kScanChunk = kScanThreads * kScanPer;
static_assert(kScanThreads == 32 * 32, "the warp-sum scan assumes 32 warps");
constexpr int kScanOneBlock = 4 * kScanChunk;  // larger arrays go to cub
struct ScanSeg {  // up to four independent scans, one block each
    const int32_t* in[4];
    int32_t* out[4];
    int n[4];
};
__global__ void __launch_bounds__(kScanThreads) k_scan1(ScanSeg sg) {
    __shared__ int32_t buf[kScanChunk];
    __shared__ int32_t wsum[32];
    const int32_t* in = sg.in[blockIdx.x];
    int32_t* out = sg.out[blockIdx.x];
    const int n = sg.n[blockIdx.x];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    int carry = 0;
    for (int base = 0; base < n; base += kScanChunk) {
        const int m = min(kScanChunk, n - base);
        for (int i = tid; i < kScanChunk; i += kScanThreads) buf[i] = i < m ? in[base + i] : 0;
        __syncthreads();
        int v[kScanPer], sum = 0;
#pragma unroll
        for (int k = 0; k < kScanPer; k++) {
            v[k] = buf[tid * kScanPer + k];
            sum += v[k];
        }
        int x = sum;  // inclusive warp scan of the thread sums
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[w] = x;
        __syncthreads();
        if (w == 0) {
            int z = wsum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, z, o);
                if (lane >= o) z += y;
            }
            wsum[lane] = z;  // inclusive over warps
        }
        __syncthreads();
        int run = carry + (w > 0 ? wsum[w - 1] : 0) + (x - sum);
#pragma unroll
        for (int k = 0; k < kScanPer; k++) {
            buf[tid * kScanPer + k] = run;
            run += v[k];
        }
        const int chunk_total = wsum[31];
        __syncthreads();
        for (int i = tid; i < m; i += kScanThreads) out[base + i] = buf[i];
        carry += chunk_total;
        __syncthreads();
    }
    if (tid == 0) out[n] = carry;
}

int scan_on(cudaStream_t st, DBuf<uint8_t>& tmp, const int32_t* in, int32_t* out, int n) {
    if (n <= kScanOneBlock) {
        ScanSeg sg;
        sg.in[0] = sg.in[1] = in;
        sg.out[0] = sg.out[1] = out;
        sg.n[0] = sg.n[1] = n;
        k_scan1<<<1, kScanThreads, 0, st>>>(sg);
        return D2G_OK;
    }
    D2G_CUDA(cudaMemsetAsync(out, 0, sizeof(int32_t), st));
    size_t bytes = 0;
    D2G_CUDA(cub::DeviceScan::InclusiveSum(nullptr, bytes, in, out + 1, n, st));
    if (int rc = tmp.ensure(bytes + 16)) return rc;
    D2G_CUDA(cub::DeviceScan::InclusiveSum(tmp.p, bytes, in, out + 1, n, st));
    return D2G_OK;
}
int scan(d2g_ctx* ctx, const int32_t* in, int32_t* out, int n) {
    if (n <= kScanOneBlock) ctx->eng.launches++;  // this library's scan kernel (larger ones are cub's)
    return scan_on(ctx->stream, ctx->eng.cub_tmp, in, out, n);
}
// Two independent scans on the context's stream (one launch when both are small).
int scan2(d2g_ctx* ctx, const int32_t* in0, int32_t* out0, int n0, const int32_t* in1, int32_t* out1, int n1) {
    if (n0 <= kScanOneBlock && n1 <= kScanOneBlock) {
        ScanSeg sg;
        sg.in[0] = in0;
        sg.out[0] = out0;
        sg.n[0] = n0;
        sg.in[1] = in1;
        sg.out[1] = out1;
        sg.n[1] = n1;
        k_scan1<<<2, kScanThreads, 0, ctx->stream>>>(sg);
        ctx->eng.launches++;
        return D2G_OK;
    }
    if (int rc = scan(ctx, in0, out0, n0)) return rc;
    return scan(ctx, in1, out1, n1);
}

// Four scans in one launch when each fits one block, else one by one.
int scan4(d2g_ctx* ctx, const int32_t* const* in, int32_t* const* out, const int* n) {
    ScanSeg sg;
    bool one = true;
    for (int i = 0; i < 4; i++) {
        sg.in[i] = in[i];
        sg.out[i] = out[i];
        sg.n[i] = n[i];
        one = one && n[i] <= kScanOneBlock;
    }
    if (one) {
        k_scan1<<<4, kScanThreads, 0, ctx->stream>>>(sg);
        ctx->eng.launches++;
        return D2G_OK;
    }
    for (int i = 0; i < 4; i++)
        if (int rc = scan(ctx, in[i], out[i], n[i])) return rc;
    return D2G_OK;
}

// Read k device int32 scalars (after the stream's pending work).
int read_scalars(d2g_ctx* ctx, const int32_t* const* src, int k, int32_t* dst) {
    for (int i = 0; i < k; i++)
        D2G_CUDA(cudaMemcpyAsync(ctx->h_pinned + i, src[i], sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    D2G_CUDA(cudaStreamSynchronize(ctx->stream));
    prof_collect(ctx);
    for (int i = 0; i < k; i++) dst[i] = ctx->h_pinned[i];
    return D2G_OK;
}

#define RC(x)                     \
    do {                          \
        if (int rc_ = (x)) return rc_; \
    } while (0)

// Sort records by pair (stable) into rec_sorted and write offsets [n_pairs+1].
// Pairs [p0, p0 + n_pairs): the records' pair ids lie in that range and the
// offsets are indexed from p0.
int finish_records(d2g_ctx* ctx, int n_pairs, int n_rec, int p0 = 0) {
    Engine& E = ctx->eng;
    RC(E.out_off.ensure(n_pairs + 1));
    RC(E.pair_cnt.ensure(n_pairs + 1));
    RC(E.rec_sorted.ensure(14 * (size_t)n_rec + 14));
    D2G_CUDA(cudaMemsetAsync(E.pair_cnt.p, 0, sizeof(int32_t) * (n_pairs + 1), ctx->stream));
    if (n_rec > 0) {
        RC(E.rec_idx.ensure(n_rec));
        RC(E.rec_idx_sorted.ensure(n_rec));
        RC(E.rec_pair_sorted.ensure(n_rec));
        LAUNCH(k_iota, n_rec, n_rec, E.rec_idx.p);
        int bits = 1;
        while ((1LL << bits) < (long long)p0 + n_pairs + 1 && bits < 31) bits++;
        size_t bytes = 0;
        D2G_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, bytes, E.rec_pair.p, E.rec_pair_sorted.p, E.rec_idx.p,
                                                 E.rec_idx_sorted.p, n_rec, 0, bits, ctx->stream));
        RC(E.cub_tmp.ensure(bytes + 16));
        D2G_CUDA(cub::DeviceRadixSort::SortPairs(E.cub_tmp.p, bytes, E.rec_pair.p, E.rec_pair_sorted.p, E.rec_idx.p,
                                                 E.rec_idx_sorted.p, n_rec, 0, bits, ctx->stream));
        LAUNCH(k_gather, n_rec, n_rec, E.rec_idx_sorted.p, E.rec.p, E.rec_sorted.p);
        LAUNCH(k_count_pairs, n_rec, n_rec, p0, n_pairs, E.rec_pair.p, E.pair_cnt.p);
    }
    RC(scan(ctx, E.pair_cnt.p, E.out_off.p, n_pairs));
    return D2G_OK;
}

}  // namespace

// Profiling marks for kernels launched outside this file.
int prof_mark_begin(d2g_ctx* ctx, int kind, long long items) { return prof_begin(ctx, kind, items); }
void prof_mark_end(d2g_ctx* ctx, int idx) { prof_end(ctx, idx); }
void prof_mark_collect(d2g_ctx* ctx) { prof_collect(ctx); }

// Launch with an explicit block size.
#define LAUNCHB(kern, n, block, ...)                                                  \
    do {                                                                              \
        kern<<<nblocks(n, block), block, 0, ctx->stream>>>(__VA_ARGS__);              \
        ctx->eng.launches++;                                                          \
    } while (0)

// Append flagged results (already scanned into `off`) as contact records at `base`.
void emit_records(d2g_ctx* ctx, int n, const int32_t* flags, const int32_t* off, const int32_t* items, int shift,
                  const Entry* front, const int32_t* conn_off, int n_conn, const int32_t* d_pairs,
                  const PrimResult* res, int base) {
    Engine& E = ctx->eng;
    LAUNCH(k_emit, n, n, flags, off, items, shift, front, conn_off, n_conn, d_pairs, res, nullptr, ctx->geo_eps.p,
           E.rec.p, E.rec_pair.p, base);
}

// Grid of k_ee_rest4: it reads its list size from device memory, so the grid
// is fixed (every block resident, grid-stride; the first quads take the
// tests, so a short list occupies the first blocks, one warp per SMSP).
int ee_grid_size(d2g_ctx* ctx, int* grid) {
    Engine& E = ctx->eng;
    if (E.ee_grid == 0) {
        int dev_sms = 0, per_sm = 0;
        D2G_CUDA(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device));
        D2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ee_rest4, kBlock, 0));
        E.ee_grid = std::max(1, dev_sms * std::max(1, per_sm));
    }
    *grid = E.ee_grid;
    return D2G_OK;
}

// Bytes a traversal level may use for its buffers: a sixth of the device
// memory (the rest holds the scene, the contact records with their sorted
// copy, and other stages).  d2g_ctx_set_level_budget overrides it.
double level_budget(d2g_ctx* ctx) {
    Engine& E = ctx->eng;
    if (E.level_budget > 0) return (double)E.level_budget;
    if (E.device_bytes == 0) {  // queried once: the driver call is not free
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 1e30;
        E.device_bytes = total_b;
    }
    return (double)E.device_bytes / 6.0;
}

// The proposal's 20 features of n pair queries over the context's device
// bodies, into E.pp_feat.
int run_ccd_features(d2g_ctx* ctx, const int32_t* d_pairs, const double* d_max_time, int n) {
    Engine& E = ctx->eng;
    RC(E.pp_feat.ensure(20 * (size_t)n + 1));
    if (n > 0)
        LAUNCH(k_ccd_features, n, n, d_pairs, d_max_time, ctx->cur.p, ctx->inv_inertia.p, ctx->bounding_radius.p,
               E.pp_feat.p);
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

// The separation-witness table: allocated on first use and cleared when the
// witnesses written since the last clearing could fill half of it (stale
// entries only cost a failed check; clearing keeps the probes short).
int ensure_witness_table(d2g_ctx* ctx) {
    Engine& E = ctx->eng;
    const size_t cap = (size_t)1 << E.wt_log2cap;
    if (!E.wt_table.p || E.wt_inserts > (long long)(cap / 2)) {
        RC(E.wt_table.ensure(cap));
        D2G_CUDA(cudaMemsetAsync(E.wt_table.p, 0, sizeof(WitnessSlot) * cap, ctx->stream));
        E.wt_inserts = 0;
    }
    return D2G_OK;
}

// Body indices of a device pair list inside [0, n_bodies): one flag, one read.
__global__ void k_check_pairs(int n, const int32_t* __restrict__ pairs, int n_bodies, int32_t* __restrict__ bad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 2 * n) return;
    const int v = pairs[i];
    if (v < 0 || v >= n_bodies) atomicMin(bad, i >> 1);
}

int check_device_pairs(d2g_ctx* ctx, const int32_t* d_pairs, int n) {
    Engine& E = ctx->eng;
    if (n <= 0) return D2G_OK;
    RC(E.scratch_i32.ensure(1));
    ctx->h_pinned[0] = INT32_MAX;
    D2G_CUDA(cudaMemcpyAsync(E.scratch_i32.p, ctx->h_pinned, sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
    LAUNCH(k_check_pairs, 2LL * n, n, d_pairs, ctx->n_bodies, E.scratch_i32.p);
    int32_t bad = 0;
    const int32_t* src = E.scratch_i32.p;
    RC(read_scalars(ctx, &src, 1, &bad));
    if (bad != INT32_MAX) {
        set_error("device pair " + std::to_string(bad) + " names a body outside [0, " +
                  std::to_string(ctx->n_bodies) + ")");
        return D2G_ERR_INVALID;
    }
    return D2G_OK;
}

// The CCD counters live on the device across calls (one read when asked).
int ensure_ccd_stats(d2g_ctx* ctx) {
    Engine& E = ctx->eng;
    if (!E.ccd_stats.p) {
        RC(E.ccd_stats.ensure(kCcdStats));
        D2G_CUDA(cudaMemsetAsync(E.ccd_stats.p, 0, sizeof(unsigned long long) * kCcdStats, ctx->stream));
    }
    return D2G_OK;
}

int read_ccd_stats(d2g_ctx* ctx, int64_t* out, int n, bool reset) {
    Engine& E = ctx->eng;
    RC(ensure_ccd_stats(ctx));
    unsigned long long h[kCcdStats];
    D2G_CUDA(cudaMemcpyAsync(h, E.ccd_stats.p, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    if (reset) D2G_CUDA(cudaMemsetAsync(E.ccd_stats.p, 0, sizeof(h), ctx->stream));
    D2G_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < n && i < kCcdStats; i++) out[i] = (int64_t)h[i];
    return D2G_OK;
}

int run_ccd(d2g_ctx* ctx, const int32_t* d_pairs, const double* d_max_time, int n_pairs, int* n_out,
            int64_t* counters, const CcdSink* sink) {
    Engine& E = ctx->eng;
    cudaStream_t s = ctx->stream;
    int64_t c_node = 0, c_tri = 0, c_leaf = 0, c_levels = 0;
    RC(ensure_ccd_stats(ctx));
    if (E.witnesses) RC(ensure_witness_table(ctx));
    RC(E.pm.ensure((size_t)PM_SIZE * n_pairs + 1));
    RC(E.pfut.ensure(28 * (size_t)n_pairs + 1));
    RC(E.search.ensure(n_pairs + 1));
    RC(E.soup.ensure(n_pairs + 1));
    int ee_grid = 0;
    RC(ee_grid_size(ctx, &ee_grid));
    int n_rec = 0;
    long long n_streamed = 0;  // records handed to the sink
    if (n_pairs > 0)
        LAUNCH(k_ccd_prep, 4LL * n_pairs, n_pairs, d_pairs, d_max_time, ctx->cur.p, ctx->inv_inertia.p, ctx->mesh.p,
               ctx->mesh_node_off.p, ctx->geo_eps.p, E.pm.p, E.pfut.p, E.search.p, E.soup.p);
    RC(E.pm32c.ensure((size_t)96 * n_pairs + 1));
    if (n_pairs > 0) LAUNCH(k_ccd_pm32, 96LL * n_pairs, n_pairs, E.pm.p, E.pm32c.p);  // FP32 poses, once per call
    // The learned proposal: the network predicts which queries have no
    // contact; the root certificate proves it for those it can, and the
    // proven ones are skipped (their outputs are empty either way).
    const uint8_t* skip = nullptr;
    if (E.proposal && n_pairs > 0) {
        RC(E.pp_feat.ensure(20 * (size_t)n_pairs));
        RC(E.pp_skip.ensure(n_pairs + 1));
        LAUNCH(k_ccd_features, n_pairs, n_pairs, d_pairs, d_max_time, ctx->cur.p, ctx->inv_inertia.p,
               ctx->bounding_radius.p, E.pp_feat.p);
        const float* pred = nullptr;
        RC(mlp_forward_device(E.proposal, E.pp_feat.p, n_pairs, &pred));
        LAUNCH(k_root_certify, 32LL * n_pairs, n_pairs, d_pairs, E.pm.p, E.pm32c.p, ctx->tri32.p, ctx->mesh.p,
               ctx->mesh_node_off.p,
               ctx->ntris.p, ctx->tris.p, ctx->geo_eps.p, E.search.p, pred, E.proposal_logit, E.pp_skip.p,
               E.ccd_stats.p);
        LAUNCH(k_add_u64, 1, E.ccd_stats.p + 5, (unsigned long long)n_pairs);
        skip = E.pp_skip.p;
    }
    // Pair chunks: the traversal of a range of body pairs runs to the end
    // before the next range starts.  A level whose buffers would pass the
    // budget abandons its chunk (its records are dropped) and the chunk is
    // halved.  A pair's records come from one chunk and are sorted by pair at
    // the end, so the results do not depend on the chunking.
    RC(E.roots.ensure(n_pairs + 1));
    if (n_pairs > 0)
        D2G_CUDA(cudaMemcpyAsync(E.roots.p, E.soup.p, sizeof(Entry) * n_pairs, cudaMemcpyDeviceToDevice, s));
    const double budget = level_budget(ctx);
    // start from the chunk size that fitted last time (abandoning a chunk
    // wastes its finished levels), growing it when the last call used under
    // a third of the budget
    int chunk = E.ccd_chunk > 0 ? std::min(n_pairs, E.ccd_chunk) : n_pairs;
    double peak = 0.0;  // largest level need / budget among finished chunks
    for (int p0 = 0; p0 < n_pairs;) {
    const int p1 = std::min(n_pairs, p0 + chunk);
    const int rec_start = n_rec;
    int64_t k_node = 0, k_tri = 0, k_leaf = 0, k_levels = 0;
    bool abandon = false;
    double chunk_peak = 0.0;
    RC(E.soup.ensure((size_t)(p1 - p0) + 1));  // the frontiers swap every level: this one may be the smaller
    D2G_CUDA(cudaMemcpyAsync(E.soup.p, E.roots.p + p0, sizeof(Entry) * (p1 - p0), cudaMemcpyDeviceToDevice, s));
    int n_soup = p1 - p0, n_conn = 0;
    while (n_soup > 0 || n_conn > 0) {
        // past the budget, or past 32-bit slot indices (64 slots per node pair)
        if ((64.0 * 8.0 * 1.5 * n_soup > budget || 64LL * n_soup > (long long)INT32_MAX / 2) && p1 - p0 > 1) {
            abandon = true;
            break;
        }
        chunk_peak = std::max(chunk_peak, 64.0 * 8.0 * 1.5 * n_soup / budget);
        k_levels++;
        k_node += n_soup + n_conn;
        k_leaf += n_conn;
        // (1) soup swept-box filter and leaf-pair sizes, one synchronisation
        const int n_slots = 64 * n_soup;
        RC(E.flags.ensure(n_slots + 1));
        RC(E.flag_off.ensure(n_slots + 1));
        RC(E.entry_hits.ensure(n_soup + 1));
        RC(E.nn_cnt.ensure(n_conn + 1));
        RC(E.nn_off.ensure(n_conn + 1));
        RC(E.citem_off.ensure(n_conn + 1));
        if (n_soup > 0) {
            D2G_CUDA(cudaMemsetAsync(E.entry_hits.p, 0, sizeof(int32_t) * n_soup, s));
            const int pff = prof_begin(ctx, PROF_SOUP_FILTER, n_slots);
            const uint8_t* eskip = nullptr;
            if (E.witnesses) {
                RC(E.wt_flag.ensure(n_soup + 1));
                LAUNCH(k_witness_check, 32LL * n_soup, n_soup, E.soup.p, d_pairs, E.pm.p, E.pm32c.p, ctx->tri32.p,
                       ctx->mesh.p,
                       ctx->mesh_node_off.p, ctx->ntris.p, ctx->tris.p, ctx->geo_eps.p, E.search.p, E.wt_table.p,
                       E.wt_log2cap, E.wt_flag.p, E.ccd_stats.p);
                eskip = E.wt_flag.p;
            }
            LAUNCH(k_soup_filter, 32LL * n_soup, n_soup, E.soup.p, d_pairs, E.pm.p, E.pm32c.p, ctx->ntris.p,
                   ctx->tris.p, ctx->tri32.p, ctx->geo_eps.p, skip, eskip, E.flags.p);
            prof_end(ctx, pff);
        }
        if (n_conn > 0) LAUNCH(k_conn_nn, n_conn, n_conn, E.conn.p, ctx->ntris.p, E.nn_cnt.p);
        RC(scan2(ctx, E.flags.p, E.flag_off.p, n_slots, E.nn_cnt.p, E.nn_off.p, n_conn));
        int32_t tot1[2];
        const int32_t* src1[2] = {E.flag_off.p + n_slots, E.nn_off.p + n_conn};
        RC(read_scalars(ctx, src1, 2, tot1));
        const int K = tot1[0], P = tot1[1];  // soup triangle pairs, leaf-pair triangle pairs
        if (15LL * K + 15LL * P > (long long)INT32_MAX) {  // test indices are 32-bit
            if (p1 - p0 > 1) {
                abandon = true;
                break;
            }
            set_error("CCD level with " + std::to_string(K) + " + " + std::to_string(P) +
                      " triangle pairs exceeds the 32-bit test index range");
            return D2G_ERR_INVALID;
        }
        // bytes of the level's test buffers (x1.5 for the buffers' growth slack)
        if (1.5 * 1900.0 * ((double)K + (double)P) > budget && p1 - p0 > 1) {
            abandon = true;
            break;
        }
        chunk_peak = std::max(chunk_peak, 1.5 * 1900.0 * ((double)K + (double)P) / budget);
        k_tri += (int64_t)K + 15 * (int64_t)P;
        // (2) all primitive tests of the level
        RC(E.items.ensure(K + 1));
        RC(E.sub.ensure(15 * (size_t)K + 1));
        RC(E.res.ensure(K + 1));
        RC(E.hit.ensure(K + 1));
        RC(E.cres.ensure(15 * (size_t)P + 1));
        RC(E.chit.ensure(15 * (size_t)P + 1));
        RC(E.cflag_off.ensure(15 * (size_t)P + 1));
        if (n_soup > 0) LAUNCH(k_compact, n_slots, n_slots, E.flags.p, E.flag_off.p, E.items.p);
        const int n_pt = 6 * K + 6 * P, n_ee = 9 * K + 9 * P;
        // FP32 bounds drop the tests that cannot hit; the FP64 kernels run on
        // the survivors, which the bound kernels append to their lists
        RC(E.ccd_cnt.ensure(3));
        RC(E.ccd_list.ensure((size_t)n_pt + n_ee + 2));
        int32_t* cnt_pt = E.ccd_cnt.p;
        int32_t* cnt_ee = E.ccd_cnt.p + 1;
        int32_t* cnt_rest = E.ccd_cnt.p + 2;  // edge-edge tests continued by k_ee_rest4
        int32_t* list_pt = E.ccd_list.p;
        int32_t* list_ee = E.ccd_list.p + n_pt;
        D2G_CUDA(cudaMemsetAsync(E.ccd_cnt.p, 0, 3 * sizeof(int32_t), s));
        if (n_ee > 0) {
            RC(E.ee_rec.ensure((size_t)kEeRec * n_ee));
            RC(E.ee_work.ensure(n_ee));
        }
        // The point-triangle and edge-edge chains touch disjoint outputs: the
        // edge-edge chain runs on the second stream beside the other.
        const bool fork = n_pt > 0 && n_ee > 0;
        cudaStream_t s_ee = fork ? ctx->stream2 : s;
        if (fork) {
            D2G_CUDA(cudaEventRecord(ctx->ev_fork, s));
            D2G_CUDA(cudaStreamWaitEvent(s_ee, ctx->ev_fork, 0));
        }
        if (n_ee > 0) {
            k_ccd_mask_ee<<<nblocks(n_ee), kBlock, 0, s_ee>>>(K, n_ee, E.items.p, E.soup.p, E.conn.p, E.nn_off.p,
                                                            n_conn, E.pm32c.p, ctx->ntris.p, ctx->tri32.p,
                                                            E.search.p, E.sub.p, E.cres.p, E.chit.p, list_ee,
                                                            cnt_ee, E.fp32_bounds ? 1 : 0);
            const int pf = prof_begin(ctx, PROF_CONN, n_ee, s_ee);
            EeArgs ea;
            ea.n_tp = K;
            ea.n_conn = n_conn;
            ea.items = E.items.p;
            ea.soup = E.soup.p;
            ea.conn = E.conn.p;
            ea.nn_off = E.nn_off.p;
            ea.ntris = ctx->ntris.p;
            ea.search = E.search.p;
            ea.sub = E.sub.p;
            ea.cres = E.cres.p;
            ea.chit = E.chit.p;
            ea.pm = E.pm.p;
            ea.tris = ctx->tris.p;
            ea.rec = E.ee_rec.p;
            ea.work = E.ee_work.p;
            ea.count = cnt_rest;
            ea.first_iters = E.tune[D2G_TUNE_EE_FIRST_ITERS];
            ea.certificates = E.certificates ? 1 : 0;
            ea.ca_stats = E.ccd_stats.p;
            k_ee_first<<<nblocks(n_ee, kPrimBlock), kPrimBlock, 0, s_ee>>>(n_ee, list_ee, cnt_ee, E.pm.p,
                                                                          ctx->tris.p, ea);
            k_ee_rest4<<<ee_grid, kBlock, 0, s_ee>>>(ea);
            ctx->eng.launches += 2;
            prof_end(ctx, pf, s_ee);
            ctx->eng.launches += 1;  // the bound kernel
        }
        if (n_pt > 0) {
            LAUNCH(k_ccd_mask_pt, n_pt, K, n_pt, E.items.p, E.soup.p, E.conn.p, E.nn_off.p, n_conn, E.pm32c.p,
                   ctx->ntris.p, ctx->tri32.p, E.search.p, E.sub.p, E.cres.p, E.chit.p, list_pt, cnt_pt,
                   E.fp32_bounds ? 1 : 0);
            const int pf = prof_begin(ctx, PROF_SOUP_CCD, n_pt);
            LAUNCHB(k_prim_pt, n_pt, kPrimBlock, K, n_pt, E.items.p, E.soup.p, E.conn.p, E.nn_off.p, n_conn, E.pm.p,
                    ctx->ntris.p, ctx->tris.p, E.search.p, E.sub.p, E.cres.p, E.chit.p, list_pt, cnt_pt);
            prof_end(ctx, pf);
        }
        if (fork) {
            D2G_CUDA(cudaEventRecord(ctx->ev_join, s_ee));
            D2G_CUDA(cudaStreamWaitEvent(s, ctx->ev_join, 0));
        }
        // (3) soup fold and finals, leaf-pair finals, expansion; one synchronisation
        if (K > 0) {
            LAUNCH(k_soup_fold, K, K, E.items.p, E.soup.p, E.sub.p, E.search.p, E.res.p, E.hit.p, E.entry_hits.p,
                   ctx->nodes.p, E.flags.p);
        }
        RC(E.cnt_a.ensure(n_soup + 1));
        RC(E.cnt_b.ensure(n_soup + 1));
        RC(E.off_a.ensure(n_soup + 1));
        RC(E.off_b.ensure(n_soup + 1));
        if (n_soup > 0 && E.witnesses) {
            LAUNCH(k_witness_make, 32LL * n_soup, n_soup, E.soup.p, E.entry_hits.p, E.wt_flag.p, skip, d_pairs,
                   E.pm.p, E.pm32c.p, ctx->tri32.p, ctx->mesh.p, ctx->mesh_node_off.p, ctx->ntris.p, ctx->tris.p, ctx->geo_eps.p, E.search.p,
                   E.wt_table.p, E.wt_log2cap, E.ccd_stats.p);
            E.wt_inserts += n_soup;
        }
        if (n_soup > 0)
            LAUNCH(k_expand_count, n_soup, n_soup, E.soup.p, E.entry_hits.p, ctx->nodes.p, 1, E.cnt_a.p, E.cnt_b.p);
        {  // final flags of soup and leaf-pair tests, children of soup node pairs: one launch
            const int32_t* sin[4] = {E.flags.p, E.chit.p, E.cnt_a.p, E.cnt_b.p};
            int32_t* sout[4] = {E.flag_off.p, E.cflag_off.p, E.off_a.p, E.off_b.p};
            const int sn[4] = {K, 15 * P, n_soup, n_soup};
            RC(scan4(ctx, sin, sout, sn));
        }
        int32_t tot2[4];
        const int32_t* src2[4] = {E.flag_off.p + K, E.cflag_off.p + 15 * P, E.off_a.p + n_soup, E.off_b.p + n_soup};
        RC(read_scalars(ctx, src2, 4, tot2));
        const int fin_soup = tot2[0], fin_conn = tot2[1];
        RC(E.rec.ensure_keep(14 * (size_t)(n_rec + fin_soup + fin_conn + 1), 14 * (size_t)n_rec, s));
        RC(E.rec_pair.ensure_keep((size_t)(n_rec + fin_soup + fin_conn + 1), (size_t)n_rec, s));
        if (fin_soup > 0)
            emit_records(ctx, K, E.flags.p, E.flag_off.p, E.items.p, 6, E.soup.p, nullptr, 0, d_pairs, E.res.p, n_rec);
        n_rec += fin_soup;
        if (fin_conn > 0) {
            LAUNCH(k_scale, n_conn + 1, n_conn + 1, E.nn_off.p, 15, E.citem_off.p);
            emit_records(ctx, 15 * P, E.chit.p, E.cflag_off.p, nullptr, 0, E.conn.p, E.citem_off.p, n_conn, d_pairs,
                         E.cres.p, n_rec);
        }
        n_rec += fin_conn;
        RC(E.soup_next.ensure(tot2[2] + 1));
        RC(E.conn_next.ensure(tot2[3] + 1));
        if (n_soup > 0)
            LAUNCH(k_expand_write, n_soup, n_soup, E.soup.p, E.entry_hits.p, ctx->nodes.p, 1, E.off_a.p, E.off_b.p,
                   E.soup_next.p, E.conn_next.p);
        std::swap(E.soup, E.soup_next);
        std::swap(E.conn, E.conn_next);
        n_soup = tot2[2];
        n_conn = tot2[3];
    }
    if (abandon) {
        n_rec = rec_start;
        chunk = std::max(1, (p1 - p0) / 2);
        continue;
    }
    c_node += k_node;
    c_tri += k_tri;
    c_leaf += k_leaf;
    c_levels += k_levels;
    peak = std::max(peak, chunk_peak);
    if (sink) {  // the chunk's records, sorted by pair, go to the consumer and are dropped
        RC(finish_records(ctx, p1 - p0, n_rec, p0));
        RC(sink->consume(ctx, sink->user, p0, p1));
        n_streamed += n_rec;
        n_rec = 0;
    }
    p0 = p1;
    }
    if (n_pairs > 0) E.ccd_chunk = chunk >= n_pairs ? 0 : (peak < 1.0 / 3.0 ? 2 * chunk : chunk);
    if (!sink) RC(finish_records(ctx, n_pairs, n_rec));
    if (n_pairs > 0) {
        RC(E.last_pair.ensure(ctx->n_bodies + 1));
        LAUNCH(k_fill, ctx->n_bodies, ctx->n_bodies, E.last_pair.p, -1);
        LAUNCH(k_last_pair, n_pairs, n_pairs, d_pairs, E.last_pair.p);
        LAUNCH(k_write_fut, n_pairs, n_pairs, d_pairs, E.last_pair.p, E.pfut.p, ctx->fut.p);
    }
    D2G_CUDA(cudaGetLastError());
    *n_out = sink ? (int)n_streamed : n_rec;
    if (counters) {
        counters[0] = c_node;
        counters[1] = c_tri;
        counters[2] = c_leaf;
        counters[3] = c_levels;
    }
    return D2G_OK;
}

int run_narrowphase(d2g_ctx* ctx, const int32_t* d_pairs, int n_pairs, int* n_out, int64_t* counters) {
    Engine& E = ctx->eng;
    cudaStream_t s = ctx->stream;
    int64_t c_node = 0, c_tri = 0, c_leaf = 0, c_levels = 0;
    RC(E.pm.ensure(32 * (size_t)n_pairs + 1));
    RC(E.search.ensure(n_pairs + 1));
    RC(E.soup.ensure(n_pairs + 1));
    RC(E.np_tri.ensure(1));
    D2G_CUDA(cudaMemsetAsync(E.np_tri.p, 0, sizeof(int32_t), s));
    RC(E.pm32.ensure(24 * (size_t)n_pairs + 1));
    if (n_pairs > 0)
        LAUNCH(k_np_prep, n_pairs, n_pairs, d_pairs, ctx->fut.p, ctx->mesh.p, ctx->mesh_node_off.p,
                                                     ctx->geo_eps.p, E.pm.p, E.search.p, E.soup.p, E.pm32.p);
    int n_rec = 0;
    DBuf<double>& res_eps = E.pfut;  // reused as the per-slot eps record buffer
    // pair chunks, as in run_ccd: a level that would pass the byte budget
    // (~110 bytes per slot, 64 slots per node pair, x1.5 growth slack)
    // abandons its chunk, which is halved
    RC(E.roots.ensure(n_pairs + 1));
    if (n_pairs > 0)
        D2G_CUDA(cudaMemcpyAsync(E.roots.p, E.soup.p, sizeof(Entry) * n_pairs, cudaMemcpyDeviceToDevice, s));
    const double budget = level_budget(ctx);
    int chunk = E.np_chunk > 0 ? std::min(n_pairs, E.np_chunk) : n_pairs;  // as in run_ccd
    double peak = 0.0;
    for (int p0 = 0; p0 < n_pairs;) {
    const int p1 = std::min(n_pairs, p0 + chunk);
    const int rec_start = n_rec;
    const int32_t tri_start = (int32_t)c_tri;  // the device counter's value before this chunk
    int64_t k_node = 0, k_levels = 0;
    bool abandon = false;
    double chunk_peak = 0.0;
    RC(E.soup.ensure((size_t)(p1 - p0) + 1));  // the frontiers swap every level: this one may be the smaller
    D2G_CUDA(cudaMemcpyAsync(E.soup.p, E.roots.p + p0, sizeof(Entry) * (p1 - p0), cudaMemcpyDeviceToDevice, s));
    int n = p1 - p0;
    while (n > 0) {
        if ((1.5 * 110.0 * 64.0 * n > budget || 64LL * n > (long long)INT32_MAX / 2) && p1 - p0 > 1) {
            abandon = true;
            break;
        }
        chunk_peak = std::max(chunk_peak, 1.5 * 110.0 * 64.0 * n / budget);
        k_levels++;
        k_node += n;
        const int n_slots = 64 * n;
        RC(E.res.ensure(n_slots));
        RC(res_eps.ensure(4 * (size_t)n_slots));
        RC(E.hit.ensure(n_slots));
        RC(E.flags.ensure(n_slots));
        RC(E.entry_hits.ensure(n));
        D2G_CUDA(cudaMemsetAsync(E.entry_hits.p, 0, sizeof(int32_t) * n, s));
        const int n_words = n_slots / 32;
        RC(E.np_mask.ensure(n_words + 1));
        RC(E.np_cnt.ensure(n_words + 1));
        RC(E.np_off.ensure(n_words + 1));
        RC(E.items.ensure(n_slots + 1));
        LAUNCH(k_np_mask, n_slots, n_slots, E.soup.p, E.pm32.p, ctx->ntris.p, ctx->tri_sph.p, ctx->tri32.p, ctx->eps_up.p,
               E.search.p, E.np_mask.p, E.np_cnt.p, E.np_tri.p, E.fp32_bounds ? 1 : 0);
        RC(scan(ctx, E.np_cnt.p, E.np_off.p, n_words));
        LAUNCH(k_np_items, n_slots, n_slots, E.np_mask.p, E.np_off.p, E.items.p);
        // the survivors' count sizes every later kernel of the level
        int32_t n_items = 0;
        {
            const int32_t* src = E.np_off.p + n_words;
            RC(read_scalars(ctx, &src, 1, &n_items));
        }
        if (n_items > 0) {
            const int pf = prof_begin(ctx, PROF_NP, n_slots);
            LAUNCH(k_np, n_items, n_items, E.soup.p, d_pairs, E.pm.p, ctx->ntris.p, ctx->tris.p, ctx->eps.p,
                   ctx->inner_eps.p, ctx->geo_eps.p, E.search.p, E.res.p, res_eps.p, E.hit.p, E.entry_hits.p,
                   E.items.p, (const int32_t*)nullptr);
            prof_end(ctx, pf);
            LAUNCH(k_final_flags, n_items, n_items, E.items.p, E.soup.p, ctx->nodes.p, E.hit.p, E.flags.p);
        }
        // final contacts: compacted now, counted with the level-end read
        RC(E.flag_off.ensure(n_items + 1));
        RC(scan(ctx, E.flags.p, E.flag_off.p, n_items));
        RC(E.rec.ensure_keep(14 * (size_t)(n_rec + n_items + 1), 14 * (size_t)n_rec, s));
        RC(E.rec_pair.ensure_keep((size_t)(n_rec + n_items + 1), (size_t)n_rec, s));
        if (n_items > 0)
            LAUNCH(k_emit, n_items, n_items, E.flags.p, E.flag_off.p, E.items.p, 6, E.soup.p, (const int32_t*)nullptr,
                   0, d_pairs, E.res.p, res_eps.p, ctx->geo_eps.p, E.rec.p, E.rec_pair.p, n_rec);
        RC(E.cnt_a.ensure(n));
        RC(E.cnt_b.ensure(n));
        RC(E.off_a.ensure(n + 1));
        RC(E.off_b.ensure(n + 1));
        LAUNCH(k_expand_count, n, n, E.soup.p, E.entry_hits.p, ctx->nodes.p, 0, E.cnt_a.p,
                                                     E.cnt_b.p);
        RC(scan(ctx, E.cnt_a.p, E.off_a.p, n));
        D2G_CUDA(cudaMemsetAsync(E.off_b.p, 0, sizeof(int32_t) * (n + 1), s));
        int32_t vals[3];
        const int32_t* srcs[3] = {E.off_a.p + n, E.np_tri.p, E.flag_off.p + n_items};
        RC(read_scalars(ctx, srcs, 3, vals));
        const int32_t tot = vals[0];
        c_tri = vals[1];
        n_rec += vals[2];
        RC(E.soup_next.ensure(tot + 1));
        LAUNCH(k_expand_write, n, n, E.soup.p, E.entry_hits.p, ctx->nodes.p, 0, E.off_a.p,
                                                     E.off_b.p, E.soup_next.p, E.conn_next.p);
        std::swap(E.soup, E.soup_next);
        n = tot;
    }
    if (abandon) {
        n_rec = rec_start;
        c_tri = tri_start;
        ctx->h_pinned[0] = tri_start;  // stream-ordered before any later read into h_pinned
        D2G_CUDA(cudaMemcpyAsync(E.np_tri.p, ctx->h_pinned, sizeof(int32_t), cudaMemcpyHostToDevice, s));
        chunk = std::max(1, (p1 - p0) / 2);
        continue;
    }
    c_node += k_node;
    c_levels += k_levels;
    peak = std::max(peak, chunk_peak);
    p0 = p1;
    }
    if (n_pairs > 0) E.np_chunk = chunk >= n_pairs ? 0 : (peak < 1.0 / 3.0 ? 2 * chunk : chunk);
    RC(finish_records(ctx, n_pairs, n_rec));
    D2G_CUDA(cudaGetLastError());
    *n_out = n_rec;
    if (counters) {
        counters[0] = c_node;
        counters[1] = c_tri;
        counters[2] = c_leaf;
        counters[3] = c_levels;
    }
    return D2G_OK;
}

// findContactsBucketComparison (comparison_dist.h:205-240) as the reference's
// strategy interface issues it: one body pair, the node pairs of one level of
// compareTreesFull (full_tree_comparison.h:25).  The level runs as a level of
// run_narrowphase does (FP32 candidate bounds, then one FP64 triangle
// distance per surviving slot), except that every hit is emitted, in slot
// order, and the per-node-pair hit counts are summed into the reference's
// cumulative pair_used_out.
int run_bucket_comparison(d2g_ctx* ctx, const int32_t* d_pair, const int32_t* d_node_pairs, int n, int* n_hits) {
    Engine& E = ctx->eng;
    cudaStream_t s = ctx->stream;
    RC(E.pm.ensure(33));
    RC(E.search.ensure(2));
    RC(E.pm32.ensure(25));
    RC(E.roots.ensure(2));
    RC(E.np_tri.ensure(1));
    D2G_CUDA(cudaMemsetAsync(E.np_tri.p, 0, sizeof(int32_t), s));
    LAUNCH(k_np_prep, 1, 1, d_pair, ctx->fut.p, ctx->mesh.p, ctx->mesh_node_off.p, ctx->geo_eps.p, E.pm.p,
           E.search.p, E.roots.p, E.pm32.p);
    RC(E.soup.ensure(n + 1));
    RC(E.off_a.ensure(n + 1));
    RC(E.entry_hits.ensure(n + 1));
    D2G_CUDA(cudaMemsetAsync(E.entry_hits.p, 0, sizeof(int32_t) * (n + 1), s));
    *n_hits = 0;
    if (n == 0) {
        D2G_CUDA(cudaMemsetAsync(E.off_a.p, 0, sizeof(int32_t), s));
        return D2G_OK;
    }
    LAUNCH(k_bucket_entries, n, n, d_node_pairs, E.soup.p);
    const int n_slots = 64 * n;
    const int n_words = n_slots / 32;
    DBuf<double>& res_eps = E.pfut;  // as in run_narrowphase
    RC(E.res.ensure(n_slots));
    RC(res_eps.ensure(4 * (size_t)n_slots));
    RC(E.hit.ensure(n_slots));
    RC(E.np_mask.ensure(n_words + 1));
    RC(E.np_cnt.ensure(n_words + 1));
    RC(E.np_off.ensure(n_words + 1));
    RC(E.items.ensure(n_slots + 1));
    LAUNCH(k_np_mask, n_slots, n_slots, E.soup.p, E.pm32.p, ctx->ntris.p, ctx->tri_sph.p, ctx->tri32.p,
           ctx->eps_up.p, E.search.p, E.np_mask.p, E.np_cnt.p, E.np_tri.p, E.fp32_bounds ? 1 : 0);
    RC(scan(ctx, E.np_cnt.p, E.np_off.p, n_words));
    LAUNCH(k_np_items, n_slots, n_slots, E.np_mask.p, E.np_off.p, E.items.p);
    int32_t n_items = 0;
    {
        const int32_t* src = E.np_off.p + n_words;
        RC(read_scalars(ctx, &src, 1, &n_items));
    }
    if (n_items > 0) {
        const int pf = prof_begin(ctx, PROF_NP, n_slots);
        LAUNCH(k_np, n_items, n_items, E.soup.p, d_pair, E.pm.p, ctx->ntris.p, ctx->tris.p, ctx->eps.p,
               ctx->inner_eps.p, ctx->geo_eps.p, E.search.p, E.res.p, res_eps.p, E.hit.p, E.entry_hits.p, E.items.p,
               (const int32_t*)nullptr);
        prof_end(ctx, pf);
    }
    RC(E.flag_off.ensure(n_items + 1));
    RC(scan(ctx, E.hit.p, E.flag_off.p, n_items));
    RC(scan(ctx, E.entry_hits.p, E.off_a.p, n));
    int32_t tot = 0;
    {
        const int32_t* src = E.off_a.p + n;
        RC(read_scalars(ctx, &src, 1, &tot));
    }
    RC(E.rec.ensure(14 * (size_t)tot + 14));
    RC(E.rec_pair.ensure((size_t)tot + 1));
    if (tot > 0)
        LAUNCH(k_emit, n_items, n_items, E.hit.p, E.flag_off.p, E.items.p, 6, E.soup.p, (const int32_t*)nullptr, 0,
               d_pair, E.res.p, res_eps.p, ctx->geo_eps.p, E.rec.p, E.rec_pair.p, 0);
    D2G_CUDA(cudaGetLastError());
    *n_hits = tot;
    return D2G_OK;
}

}  // namespace d2g

// ============================================================================
// Allocation-free discrete narrow phase.
//
// For callers that may not allocate device memory while they run: a host that
// hands this library a fixed memory budget up front (game or robotics loops
// with real-time limits, where an allocation can stall or fail mid-frame), or
// an embedding runtime that owns every allocation itself.  Every intermediate
// buffer of the traversal is carved out of the file-scope array below, which
// each GPU that loads this library holds until the process exits.
//
// Limits (larger requests are rejected with D2G_ERR_INVALID and a message,
// before the traversal or at the level that would pass them):
//   body pairs per call          <= D2G_NOALLOC_MAX_PAIRS      (2048; each pair
//                                   puts its root node pair in the first level)
//   node pairs per tree level    <= D2G_NOALLOC_MAX_NODE_PAIRS (2048)
//   contacts found per call      <= D2G_NOALLOC_MAX_CONTACTS   (32768)
// All calls share the array and it keeps the previous call's contents: the
// counters that must start at zero are cleared on every call, and two calls
// whose work overlaps on the GPU (different streams, or different threads)
// race on it.  The call reads each level's sizes back to the host, so it
// synchronizes its stream once per tree level and once at the end.  The first
// call on a device looks up the array's device address (cudaGetSymbolAddress)
// and caches it; make that first call before any stream capture.
// ============================================================================
namespace d2g {
namespace {

constexpr size_t kNoAllocBytes = (size_t)24 << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[64] = {nullptr};

// Device address of the scratch array on the current device.
int noalloc_base(void** out) {
    int dev = 0;
    D2G_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("device index beyond the allocation-free path's table");
        return D2G_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_error(std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
            return D2G_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return D2G_OK;
}

// Bump carve-out of 256-byte aligned pieces.
struct Carve {
    unsigned char* base;
    size_t used, cap;
    template <class T>
    T* take(size_t n) {
        const size_t off = (used + 255) & ~(size_t)255;
        const size_t bytes = n * sizeof(T);
        if (off + bytes > cap) return nullptr;
        used = off + bytes;
        return (T*)(base + off);
    }
};

// Index checks of the caller's device inputs: pair body ids, their mesh ids,
// node links and bucket sizes.  Sets *err to 1 on any violation.
__global__ void k_noalloc_validate(int n_pairs, const int32_t* __restrict__ pairs, int n_bodies,
                                   const int32_t* __restrict__ mesh, int n_meshes,
                                   const int32_t* __restrict__ mesh_node_off, int n_nodes,
                                   const int4* __restrict__ nodes, const int32_t* __restrict__ ntris,
                                   int32_t* __restrict__ err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_meshes && (mesh_node_off[i] < 0 || mesh_node_off[i] >= n_nodes)) atomicExch(err, 1);
    if (i < n_pairs) {
        const int a = pairs[2 * i], b = pairs[2 * i + 1];
        if (a < 0 || a >= n_bodies || b < 0 || b >= n_bodies)
            atomicExch(err, 1);
        else if (mesh[a] < 0 || mesh[a] >= n_meshes || mesh[b] < 0 || mesh[b] >= n_meshes)
            atomicExch(err, 1);
    }
    if (i < n_nodes) {
        const int4 nd = nodes[i];
        if (ntris[i] < 0 || ntris[i] > 8 || nd.y < 0 || nd.y > 8 || (nd.z && (nd.x < 0 || nd.x + nd.y > n_nodes)))
            atomicExch(err, 1);
    }
}

int noalloc_read(cudaStream_t s, const int32_t* src, int32_t* dst) {
    D2G_CUDA(cudaMemcpyAsync(dst, src, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    D2G_CUDA(cudaStreamSynchronize(s));
    return D2G_OK;
}

int noalloc_scan(cudaStream_t s, void* tmp, size_t tmp_bytes, const int32_t* in, int32_t* out, int n) {
    D2G_CUDA(cudaMemsetAsync(out, 0, sizeof(int32_t), s));
    if (n == 0) return D2G_OK;
    size_t need = 0;
    D2G_CUDA(cub::DeviceScan::InclusiveSum(nullptr, need, in, out + 1, n, s));
    if (need > tmp_bytes) {
        set_error("allocation-free scratch: prefix-sum temporary storage too small");
        return D2G_ERR_INVALID;
    }
    size_t avail = tmp_bytes;
    D2G_CUDA(cub::DeviceScan::InclusiveSum(tmp, avail, in, out + 1, n, s));
    return D2G_OK;
}

#define NA_LAUNCH(kern, n, ...) kern<<<nblocks(n), kBlock, 0, s>>>(__VA_ARGS__)

}  // namespace
}  // namespace d2g

extern "C" int d2g_compare_trees_full_noalloc(const d2g_device_scene* sc, const int32_t* d_pairs, int32_t n_pairs,
                                              double* d_contacts, int32_t capacity, int32_t* d_offsets,
                                              int32_t* n_contacts, void* stream) {
    using namespace d2g;
    cudaStream_t s = (cudaStream_t)stream;
    if (!sc || !d_offsets || !n_contacts || n_pairs < 0 || (n_pairs > 0 && !d_pairs) || capacity < 0 ||
        (capacity > 0 && !d_contacts) || sc->n_meshes <= 0 || sc->n_bodies <= 0 || !sc->mesh_node_off ||
        !sc->nodes || !sc->ntris || !sc->tris || !sc->eps || !sc->inner_eps || !sc->mesh || !sc->fut ||
        !sc->geo_eps || sc->n_nodes <= 0) {
        set_error("invalid allocation-free narrow-phase arguments");
        return D2G_ERR_INVALID;
    }
    if (n_pairs > D2G_NOALLOC_MAX_PAIRS) {
        set_error("allocation-free narrow phase: " + std::to_string(n_pairs) + " pairs exceed the limit of " +
                  std::to_string(D2G_NOALLOC_MAX_PAIRS));
        return D2G_ERR_INVALID;
    }
    void* base = nullptr;
    if (int rc = noalloc_base(&base)) return rc;
    const int MP = D2G_NOALLOC_MAX_PAIRS, MN = D2G_NOALLOC_MAX_NODE_PAIRS, MR = D2G_NOALLOC_MAX_CONTACTS;
    static_assert(D2G_NOALLOC_MAX_PAIRS <= D2G_NOALLOC_MAX_NODE_PAIRS,
                  "the first tree level holds one root node pair per body pair");
    Carve cv{(unsigned char*)base, 0, kNoAllocBytes};
    double* pm = cv.take<double>(32 * (size_t)MP);
    float* search = cv.take<float>(MP);
    Entry* front = cv.take<Entry>(MN);
    Entry* next = cv.take<Entry>(MN);
    int32_t* entry_hits = cv.take<int32_t>(MN);
    int32_t* cnt_a = cv.take<int32_t>(MN);
    int32_t* cnt_b = cv.take<int32_t>(MN);
    int32_t* off_a = cv.take<int32_t>(MN + 1);
    int32_t* off_b = cv.take<int32_t>(MN + 1);
    PrimResult* res = cv.take<PrimResult>(64 * (size_t)MN);
    double* res_eps = cv.take<double>(4 * 64 * (size_t)MN);
    int32_t* hit = cv.take<int32_t>(64 * (size_t)MN);
    int32_t* flags = cv.take<int32_t>(64 * (size_t)MN);
    int32_t* flag_off = cv.take<int32_t>(64 * (size_t)MN + 1);
    double* rec = cv.take<double>(14 * (size_t)MR);
    int32_t* rec_pair = cv.take<int32_t>(MR);
    int32_t* rec_pair_sorted = cv.take<int32_t>(MR);
    int32_t* rec_idx = cv.take<int32_t>(MR);
    int32_t* rec_idx_sorted = cv.take<int32_t>(MR);
    int32_t* pair_cnt = cv.take<int32_t>(MP + 1);
    int32_t* err = cv.take<int32_t>(1);
    const size_t tmp_bytes = kNoAllocBytes - ((cv.used + 255) & ~(size_t)255) - 256;
    void* tmp = cv.take<unsigned char>(tmp_bytes);
    if (!tmp || !err) {
        set_error("allocation-free scratch layout does not fit");
        return D2G_ERR_INVALID;
    }
    const int4* nodes = (const int4*)sc->nodes;
    int32_t h_err = 0;
    D2G_CUDA(cudaMemsetAsync(err, 0, sizeof(int32_t), s));
    int nv = n_pairs > sc->n_nodes ? n_pairs : sc->n_nodes;
    nv = nv > sc->n_meshes ? nv : sc->n_meshes;
    NA_LAUNCH(k_noalloc_validate, nv, n_pairs, d_pairs, sc->n_bodies, sc->mesh, sc->n_meshes, sc->mesh_node_off,
              sc->n_nodes, nodes, sc->ntris, err);
    if (int rc = noalloc_read(s, err, &h_err)) return rc;
    if (h_err) {
        set_error("allocation-free narrow phase: a body, mesh or node index is out of range");
        return D2G_ERR_INVALID;
    }
    if (n_pairs > 0)
        NA_LAUNCH(k_np_prep, n_pairs, n_pairs, d_pairs, sc->fut, sc->mesh, sc->mesh_node_off, sc->geo_eps, pm, search,
                  front, nullptr);
    int n = n_pairs, n_rec = 0, level = 0;
    while (n > 0) {
        if (n > MN) {
            set_error("allocation-free narrow phase: " + std::to_string(n) + " node pairs at level " +
                      std::to_string(level) + " exceed the limit of " + std::to_string(MN));
            return D2G_ERR_INVALID;
        }
        const int n_slots = 64 * n;
        D2G_CUDA(cudaMemsetAsync(entry_hits, 0, sizeof(int32_t) * n, s));
        NA_LAUNCH(k_np, n_slots, n_slots, front, d_pairs, pm, sc->ntris, sc->tris, sc->eps, sc->inner_eps,
                  sc->geo_eps, search, res, res_eps, hit, entry_hits, nullptr, nullptr);
        NA_LAUNCH(k_final_flags, n_slots, n_slots, nullptr, front, nodes, hit, flags);
        if (int rc = noalloc_scan(s, tmp, tmp_bytes, flags, flag_off, n_slots)) return rc;
        int32_t tot = 0;
        if (int rc = noalloc_read(s, flag_off + n_slots, &tot)) return rc;
        if (n_rec + tot > MR) {
            set_error("allocation-free narrow phase: contacts exceed the limit of " + std::to_string(MR));
            return D2G_ERR_INVALID;
        }
        if (tot > 0)
            NA_LAUNCH(k_emit, n_slots, n_slots, flags, flag_off, nullptr, 6, front, nullptr, 0, d_pairs, res, res_eps,
                      sc->geo_eps, rec, rec_pair, n_rec);
        n_rec += tot;
        NA_LAUNCH(k_expand_count, n, n, front, entry_hits, nodes, 0, cnt_a, cnt_b);
        if (int rc = noalloc_scan(s, tmp, tmp_bytes, cnt_a, off_a, n)) return rc;
        D2G_CUDA(cudaMemsetAsync(off_b, 0, sizeof(int32_t) * (n + 1), s));
        int32_t nn = 0;
        if (int rc = noalloc_read(s, off_a + n, &nn)) return rc;
        if (nn > MN) {
            set_error("allocation-free narrow phase: " + std::to_string(nn) + " node pairs at level " +
                      std::to_string(level + 1) + " exceed the limit of " + std::to_string(MN));
            return D2G_ERR_INVALID;
        }
        NA_LAUNCH(k_expand_write, n, n, front, entry_hits, nodes, 0, off_a, off_b, next, next);
        Entry* t = front;
        front = next;
        next = t;
        n = nn;
        level++;
    }
    D2G_CUDA(cudaMemsetAsync(pair_cnt, 0, sizeof(int32_t) * (n_pairs + 1), s));
    if (n_rec > 0) {
        NA_LAUNCH(k_iota, n_rec, n_rec, rec_idx);
        int bits = 1;
        while ((1 << bits) < n_pairs + 1 && bits < 31) bits++;
        size_t need = 0;
        D2G_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, need, rec_pair, rec_pair_sorted, rec_idx, rec_idx_sorted,
                                                 n_rec, 0, bits, s));
        if (need > tmp_bytes) {
            set_error("allocation-free scratch: sort temporary storage too small");
            return D2G_ERR_INVALID;
        }
        size_t avail = tmp_bytes;
        D2G_CUDA(cub::DeviceRadixSort::SortPairs(tmp, avail, rec_pair, rec_pair_sorted, rec_idx, rec_idx_sorted,
                                                 n_rec, 0, bits, s));
        if (n_rec <= capacity) NA_LAUNCH(k_gather, n_rec, n_rec, rec_idx_sorted, rec, d_contacts);
        NA_LAUNCH(k_count_pairs, n_rec, n_rec, 0, n_pairs, rec_pair, pair_cnt);
    }
    if (int rc = noalloc_scan(s, tmp, tmp_bytes, pair_cnt, d_offsets, n_pairs)) return rc;
    D2G_CUDA(cudaGetLastError());
    D2G_CUDA(cudaStreamSynchronize(s));
    *n_contacts = n_rec;
    if (n_rec > capacity) {
        set_error("contact capacity " + std::to_string(capacity) + " < " + std::to_string(n_rec));
        return D2G_CAPACITY;
    }
    return D2G_OK;
}
