// Contact filtering and the per-cluster sequential-impulse solve.
//
// filterContacts (collision_detection/contact.h:44-69): one thread per body
// pair, stable insertion sort by (eps_a + eps_b, |A - B|) and the greedy
// de-duplication of contact midpoints.
//
// SequentialImpulses::solve (strategies/contact_force/sequential_impulses.cpp:
// 104-638): one block per cluster.  The reference's Gauss-Seidel sweep visits
// the contacts in sorted order and integrates both bodies after each one; a
// contact only reads and writes its own two bodies, so contacts are grouped
// into waves: a contact's wave is one past the last wave that touched either
// of its moving bodies.  Within a wave the bodies are disjoint and the
// contacts run in parallel; every body still sees its contacts in sorted
// order, so every floating-point operation happens in the reference's order
// (static bodies are never integrated; the impulse sum the convergence test
// reads for them is accumulated from per-contact deltas in sorted order).
#include <cub/cub.cuh>

#include <algorithm>
#include <vector>

#include "d2g_geom.cuh"
#include "d2g_internal.hpp"

namespace d2g {

namespace {

constexpr int kBlock = 128;
constexpr int kSolveBlock = 256;
constexpr int kGridMinContacts = 128;    // a cluster this large may take a cooperative grid
constexpr int kGridMaxClusters = 8;      // ... with more parts than D2G_TUNE_GRID_MIN_PARTS,
                                         // when at most this many clusters qualify
constexpr int kClusterMinContacts = 32;  // a cluster this large takes a thread-block cluster
inline int nblocks(long long n, int b = kBlock) { return (int)((n + b - 1) / b); }

// ------------------------------------------------------------ filtering ---
// Sort keys of compareContacts (contact.h:32-40): (eps_a + eps_b, |A - B|),
// both non-negative doubles, whose bit patterns order like the values.
__global__ void k_filter_keys(int n, const double* __restrict__ rec, unsigned long long* __restrict__ key_norm,
                              int32_t* __restrict__ idx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* c = rec + 14 * (size_t)i;
    key_norm[i] = (unsigned long long)__double_as_longlong(norm(mk(c[0] - c[3], c[1] - c[4], c[2] - c[5])));
    idx[i] = i;
}

__global__ void k_filter_eps_keys(int n, const double* __restrict__ rec, const int32_t* __restrict__ idx,
                                  unsigned long long* __restrict__ key_eps) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* c = rec + 14 * (size_t)idx[i];
    key_eps[i] = (unsigned long long)__double_as_longlong(c[6] + c[7]);
}

// The greedy pass of filterContacts (contact.h:49-66), one warp per body
// pair over its contacts in sorted order: a contact is kept unless its
// midpoint lies within eps_a + eps_b + margin (its own) of an already kept
// contact's midpoint.  Contacts are taken 32 at a time: each lane tests its
// contact against the pair's kept midpoints, then the chunk is resolved in
// order (the lowest surviving lane is kept and eliminates the later lanes
// near it).  kept_mid holds each pair's kept midpoints (from its first slot).
__global__ void k_filter_dedupe(int n_pairs, const int32_t* __restrict__ off, const int32_t* __restrict__ order,
                                const double* __restrict__ rec, double margin, int32_t* __restrict__ keep,
                                int32_t* __restrict__ kept_cnt, double* __restrict__ kept_mid) {
    const int warp = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (warp >= n_pairs) return;  // uniform per warp
    const int c0 = off[warp], c1 = off[warp + 1];
    int nk = 0;
    for (int base = c0; base < c1; base += 32) {
        const int j = base + lane;
        const bool in = j < c1;
        V3 mid = mk(0, 0, 0);
        double search = 0.0;
        if (in) {
            const double* ct = rec + 14 * (size_t)order[j];
            mid = mk((ct[0] + ct[3]) / 2, (ct[1] + ct[4]) / 2, (ct[2] + ct[5]) / 2);
            search = (ct[6] + ct[7]) + margin;
        }
        bool alive = in;
        for (int t = 0; t < nk && alive; t++) {
            const double* h = kept_mid + 3 * (size_t)(c0 + t);
            if (norm(mid - mk(h[0], h[1], h[2])) < search) alive = false;
        }
        unsigned kept = 0;
        unsigned live = __ballot_sync(0xffffffffu, alive);
        while (live) {
            const int src = __ffs(live) - 1;
            kept |= 1u << src;
            const V3 h = mk(__shfl_sync(0xffffffffu, mid.x, src), __shfl_sync(0xffffffffu, mid.y, src),
                            __shfl_sync(0xffffffffu, mid.z, src));
            if (alive && lane > src && norm(mid - h) < search) alive = false;
            live = __ballot_sync(0xffffffffu, alive) & ~((2u << src) - 1u);
        }
        const bool k = (kept >> lane) & 1u;
        if (in) keep[j] = k ? 1 : 0;
        if (k) {
            double* o = kept_mid + 3 * (size_t)(c0 + nk + __popc(kept & ((1u << lane) - 1u)));
            o[0] = mid.x;
            o[1] = mid.y;
            o[2] = mid.z;
        }
        nk += __popc(kept);
        __syncwarp();
    }
    if (lane == 0) kept_cnt[warp] = nk;
}

// Kept contacts, in sorted order per pair, to their scanned positions.
__global__ void k_filter_write(int n, const int32_t* __restrict__ order, const int32_t* __restrict__ keep,
                               const int32_t* __restrict__ pos, const double* __restrict__ rec,
                               double* __restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n || !keep[j]) return;
    const double* s = rec + 14 * (size_t)order[j];
    double* d = out + 14 * (size_t)pos[j];
    for (int k = 0; k < 14; k++) d[k] = s[k];
}

// flt_off[p] = pos[off[p]] for p in [0, n].
__global__ void k_filter_offsets(int n, const int32_t* __restrict__ off, const int32_t* __restrict__ pos,
                                 int32_t* __restrict__ out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p <= n) out[p] = pos[off[p]];
}

// ---------------------------------------------------------------- solve ---
// Per-body working state (indexed by global body id; moving bodies belong to
// one cluster only).
struct BodyWork {
    double FS[14], FSf[14];
    double T_FS[12], T_FSf[12], T_cur[12];
    double Iinv[9];  // R(fut.q) * ii * R(fut.q)^T, constant during a solve
    double imp[3], rimp[3], ioff[3], roff[3], last_imp[3];
    double rmass;  // 1 / mass, for m_div_recip
    int last_level;
};

// Per-contact working state (indexed by the contact's position in the call).
struct ConWork {
    double local_A[3], local_B[3], n[3];
    double start_dist, mass_eff, outer, impulse, impulse_offset;
    double slop, damp_m;  // per-solve constants of the normal loop: its slop and damp * mass_eff
    double rcnt;          // 1 / pair_cnt, for m_div_recip
    double last_fi[3], last_rot_A[3], last_rot_B[3], upd_total[3];
    int a, b, level, pair_cnt;
    int spos;  // position among the contacts touching a static body, -1 if none
};

__device__ __forceinline__ V3 ld3(const double* p) { return mk(p[0], p[1], p[2]); }
__device__ __forceinline__ void st3(double* p, V3 v) {
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}
__device__ __forceinline__ void rigid12(const State& s, double* T12) {
    double T[16];
    transformation(s.q, s.x, T);
    for (int k = 0; k < 12; k++) T12[k] = T[k];
}
__device__ __forceinline__ V3 calc_torque(V3 force, V3 point, V3 com) { return cross(-force, point - com); }

// sequential_impulses.cpp:46-70 updateState (variant 0, FS) or :72-96
// updateStateImmediate (variant 1, FSf) of one body, with R(fut.q) * ii *
// R(fut.q)^T precomputed (it only depends on fut).  Both forms are evaluated
// and the variant's selected, so lanes integrating different variants do
// not diverge.
__device__ void integrate_one(BodyWork& w, const double* fut, double mass, double t, int variant) {
    const State f = load_state(fut);
    const V3 imp = ld3(w.imp), ioff = ld3(w.ioff), rimp = ld3(w.rimp), roff = ld3(w.roff);
    State u = f;
    const V3 im = mk(m_div_recip(imp.x, mass, w.rmass), m_div_recip(imp.y, mass, w.rmass),
                     m_div_recip(imp.z, mass, w.rmass));
    u.v = f.v + im;
    const V3 xa = f.x + mk(m_div_recip(ioff.x, mass, w.rmass), m_div_recip(ioff.y, mass, w.rmass),
                           m_div_recip(ioff.z, mass, w.rmass)) * t;
    const V3 xb = xa + im * t;
    u.x = variant ? xb : xa;
    u.L = f.L + rimp;
    const V3 La = f.L + t * roff;
    const V3 Lb = La + t * rimp;
    const V3 omega = m3_vec(w.Iinv, variant ? Lb : La);
    u.q = qmul(qexp((0.5 * omega) * t), f.q);
    store_state(variant ? w.FSf : w.FS, u);
    rigid12(u, variant ? w.T_FSf : w.T_FS);
}

__device__ __forceinline__ double shfl_d(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ V3 shfl3(V3 v, int src) { return mk(shfl_d(v.x, src), shfl_d(v.y, src), shfl_d(v.z, src)); }

__device__ __forceinline__ V3 xf12(V3 p, const double* T) {
    return mk(((T[0] * p.x + T[1] * p.y) + T[2] * p.z) + T[3] * 1.0,
              ((T[4] * p.x + T[5] * p.y) + T[6] * p.z) + T[7] * 1.0,
              ((T[8] * p.x + T[9] * p.y) + T[10] * p.z) + T[11] * 1.0);
}

__device__ __forceinline__ bool block_any(bool v) { return __syncthreads_or(v ? 1 : 0) != 0; }

// Synchronisation of one cluster's solve: the threads of one block, the
// blocks of a thread-block cluster (the hardware cluster barrier), or every
// thread of a cooperative grid (all blocks resident) for a very large
// cluster.  The grid barrier is a 64-bit arrival counter in global memory:
// each block's thread 0 adds 1 with release semantics and waits, with
// acquire loads, until the count reaches the blocks times the barriers
// passed; the wait is bounded, and a barrier that gives up records the fact
// so the kernel can stop and report it.
enum SyncMode : int { kSyncBlock = 0, kSyncGrid = 1, kSyncCluster = 2 };

struct SolveSync {
    int mode;
    unsigned long long* count;  // grid barrier arrivals (monotonic within a launch)
    unsigned long long* passed;  // grid: the block's barriers passed so far (shared memory)
    int32_t* flags;       // [0] fail, [1] levels, [2] static contacts, [3], [4] "moved" by parity, [5] spin error
    unsigned int spin_limit;  // polls before a grid barrier wait gives up
};

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void red_add_release_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ int ld_relaxed_i32(const int32_t* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
// Every thread of the thread-block cluster; release / acquire at cluster
// scope order the blocks' global and shared memory accesses across it.
__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Grid barrier: after __syncthreads each block's thread 0 arrives with a
// release add (releasing its block's writes) and polls with acquire loads
// until every block has arrived as often as it has, then __syncthreads
// hands the acquired writes to the block.  The barriers passed so far are
// counted per block in shared memory (every block passes the same ones).
__device__ bool solve_sync(const SolveSync& S) {
    if (S.mode == kSyncBlock) {
        __syncthreads();
        return true;
    }
    if (S.mode == kSyncCluster) {
        cluster_barrier();
        return true;
    }
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        red_add_release_u64(S.count, 1ull);
        const unsigned long long target = (unsigned long long)gridDim.x * ++*S.passed;
        unsigned int spins = 0;
        while (ld_acquire_u64(S.count) < target) {
            if (++spins > S.spin_limit) {  // seconds at the default: the other blocks are gone
                atomicExch(S.flags + 5, 1);
                ok = 0;
                break;
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// true when any thread of the cluster's solve passes v; slot 3 or 4 by the
// iteration's parity (the other slot is cleared for the next iteration by
// the first block, gb = 0).
__device__ bool solve_any(const SolveSync& S, bool v, int parity, int gb, bool* ok) {
    if (S.mode == kSyncBlock) return block_any(v);
    const bool blk = __syncthreads_or(v ? 1 : 0) != 0;
    if (threadIdx.x == 0 && blk) atomicOr(S.flags + 3 + parity, 1);
    *ok = solve_sync(S) && *ok;
    const bool r = ld_relaxed_i32(S.flags + 3 + parity) != 0;
    if (gb == 0 && threadIdx.x == 0) S.flags[3 + (parity ^ 1)] = 0;
    return r;
}

// Arguments of a cluster solve.
struct SolveArgs {
    const int32_t *cl_part_off, *cl_parts, *cl_con_off, *order;
    const double* rec;
    const int32_t* pair_cnt;
    const double *warm, *cl_step;
    const uint8_t* is_static;
    const double *mass, *ii, *mu, *cur;
    double* fut;
    double gravity_z;
    BodyWork* bw;
    ConWork* cw;
    int32_t *wave_idx, *wave_off, *wave_cursor, *scon;
    double* sdelta;  // per contact touching a static body: its impulse delta on that body
    double* static_imp;
    int32_t *status, *iters;
    double* out_impulse;
    int32_t* out_ab;
    const int32_t* con_pair;
    double* pair_warm;
    int lanes;  // normal-loop lanes per contact: 0 = by wave width, 4 or 16
};

// This lane's contact (index within its cluster) and body in the warp's
// first task of a sixteen-lane wave [n0, n1), or (-1, -1) when the warp has
// no task in it.  Loaded before the barrier that precedes the wave (the
// schedule does not change during the loop), so the wave starts with one
// round of loads instead of three dependent ones.
__device__ __forceinline__ int2 wave16_first(int n0, int n1, const int32_t* __restrict__ widx, int c0, int G,
                                             int gb, const SolveArgs& a) {
    const int lane = threadIdx.x & 31, side = lane & 1;
    const int wslot = (int)(threadIdx.x >> 5) * G + gb;
    if (wslot >= (n1 - n0 + 1) >> 1) return make_int2(-1, -1);
    const int q = n0 + 2 * wslot + (lane >> 4);
    const int ci = widx[q < n1 ? q : n0];
    return make_int2(ci, side ? a.cw[c0 + ci].b : a.cw[c0 + ci].a);
}

// One wave of the normal loop (sequential_impulses.cpp:239-378: per contact
// the normal and offset impulses, then updateState :46-70 and
// updateStateImmediate :72-96 of both bodies) with sixteen lanes per
// contact: lane bit 0 picks the body side (A, B) and bit 1 the integrated
// state (FS, FSf) as in the four-lane form, bits 2-3 a component (x, y, z
// of the vectors and rows of the matrices; the fourth lane carries the
// quaternions' w).  Every value
// is the four-lane form's, operation for operation: vector and matrix work
// is spread over the component lanes and gathered with shuffles, the
// d1 / v1 dot products run on the FS / FSf lanes and sin / cos of the
// quaternion exponential on even / odd component lanes, which halves the
// FP64 instructions of a contact's dependent chain.  Each warp takes two
// contacts; warps are dealt to SMs first, then to the SMs' sub-partitions,
// as in the four-lane form.
__device__ __forceinline__ void normal_wave16(int n0, int n1, const int32_t* __restrict__ widx, int c0, int G,
                                              int gb, double t, double rt, int2 pre, const SolveArgs& a) {
    const int lane = threadIdx.x & 31;
    const int side = lane & 1, variant = (lane >> 1) & 1, c = (lane >> 2) & 3;
    const int cc = c < 3 ? c : 0;   // the w lane repeats component x in vector work
    const int grp = lane & ~12;     // component 0 of this lane's (side, state)
    const int s1 = grp | ((cc == 2 ? 0 : cc + 1) << 2), s2 = grp | ((cc == 0 ? 2 : cc - 1) << 2);
    const int tasks = (n1 - n0 + 1) >> 1;
    const int wslot = (int)(threadIdx.x >> 5) * G + gb, nwarps = (int)(blockDim.x >> 5) * G;
    for (int task = wslot; task < tasks; task += nwarps) {
        const int q = n0 + 2 * task + (lane >> 4);
        const bool act = q < n1;
        int ci, g;
        if (task == wslot && pre.x >= 0) {  // loaded before the barrier
            ci = pre.x;
            g = pre.y;
        } else {
            ci = widx[act ? q : n0];
            g = side ? a.cw[c0 + ci].b : a.cw[c0 + ci].a;
        }
        ConWork& C = a.cw[c0 + ci];
        BodyWork& W = a.bw[g];
        const bool st = a.is_static[g];
        // this side's contact point p1 = T_FS local and its velocity
        // v1 = v + (ii L) x (p1 - x) (State::pointVelocity), component cc
        // (p1 on the FS lanes and ii L on the FSf lanes in one instruction
        // stream, each with its own operations in its order, then swapped)
        const double* lp = side ? C.local_B : C.local_A;
        const double* Tr = W.T_FS + 4 * cc;
        const double* Ir = a.ii + 9 * (size_t)g + 3 * cc;
        const double* X = variant ? Ir : Tr;
        const double* Y = variant ? W.FS + 5 : lp;
        const double dot3 = (X[0] * Y[0] + X[1] * Y[1]) + X[2] * Y[2];
        const double mine = variant ? dot3 : dot3 + Tr[3] * 1.0;
        const double other = shfl_d(mine, lane ^ 2);
        const double p1 = variant ? other : mine;
        const double wv = variant ? mine : other;
        const double r = p1 - W.FS[8 + cc];
        const double w1 = shfl_d(wv, s1), w2 = shfl_d(wv, s2), r1 = shfl_d(r, s1), r2 = shfl_d(r, s2);
        const double v1s = W.FS[11 + cc] + (w1 * r2 - w2 * r1);
        const double pA = shfl_d(p1, lane & ~1), pB = shfl_d(p1, lane | 1);
        const double vA = shfl_d(v1s, lane & ~1), vB = shfl_d(v1s, lane | 1);
        // d1 = n.p1B - n.p1A on the FS lanes, v1 = n.v1A - n.v1B on the FSf lanes
        const double ncc = C.n[cc];
        const double PX = (variant ? vA : pB) * ncc, PY = (variant ? vB : pA) * ncc;
        const double dd = ((shfl_d(PX, grp) + shfl_d(PX, grp | 4)) + shfl_d(PX, grp | 8)) -
                          ((shfl_d(PY, grp) + shfl_d(PY, grp | 4)) + shfl_d(PY, grp | 8));
        const double d1 = shfl_d(dd, lane & ~2), v1 = shfl_d(dd, lane | 2);
        const double outer = C.outer, m = C.mass_eff, damp = 0.1;
        const double imp0 = C.impulse, off0 = C.impulse_offset;
        const double dimp = d1 < outer ? (v1 * m) * damp : -imp0;
        const double imp1 = dmax(imp0 + dimp, 0.0);
        const double u = (-ncc) * (imp1 - imp0);
        const double pen = outer - d1;
        const double doff = d1 < outer ? m_div_recip(C.damp_m * dmax(0.0, pen - C.slop), t, rt) : -off0;
        const double off1 = dmax(off0 + doff, 0.0);
        const double uo = (-ncc) * (off1 - off0);
        // this side's impulse sums after the contact: imp + us,
        // rimp + (-us) x (p1 - x), ioff + uso (us, uso: u, uo or their negatives)
        const double us = side ? -u : u;
        const double nus = -us;
        const double imp = W.imp[cc] + us;
        const double rimp = W.rimp[cc] + (shfl_d(nus, s1) * r2 - shfl_d(nus, s2) * r1);
        const double ioff = W.ioff[cc] + (side ? -uo : uo);
        // integrate_one on these sums, component cc
        const double* F = a.fut + 14 * (size_t)g;
        const double ms = a.mass[g];
        // imp / ms on the FS lanes, ioff / ms on the FSf lanes, then swapped
        const double qm = m_div_recip(variant ? ioff : imp, ms, W.rmass);
        const double qm2 = shfl_d(qm, lane ^ 2);
        const double im = variant ? qm2 : qm, iom = variant ? qm : qm2;
        const double vnew = F[11 + cc] + im;
        const double xa = F[8 + cc] + iom * t;
        const double xb = xa + im * t;
        const double xnew = variant ? xb : xa;
        const double Lnew = F[5 + cc] + rimp;
        const double La = F[5 + cc] + t * W.roff[cc];
        const double Lb = La + t * rimp;
        const double Ls = variant ? Lb : La;
        const double* Ii = W.Iinv + 3 * cc;
        const double om = (Ii[0] * shfl_d(Ls, grp) + Ii[1] * shfl_d(Ls, grp | 4)) + Ii[2] * shfl_d(Ls, grp | 8);
        const double d = (0.5 * om) * t;
        // qexp(d) = (cos |d|, (d / |d|) sin |d|), the identity for |d| = 0
        const double dq = d * d;
        const double nrm = sqrt((shfl_d(dq, grp) + shfl_d(dq, grp | 4)) + shfl_d(dq, grp | 8));
        const bool finite_arg = (nrm < 0.0 ? -nrm : nrm) < 1e9;
        double rr;
        int qd;
        m_reduce(finite_arg ? nrm : 0.0, rr, qd);
        const double kk = m_kernel_sincos(rr, (c & 1) != 0);
        const double ks = shfl_d(kk, grp), kc = shfl_d(kk, grp | 4);
        double sn = qd == 0 ? ks : (qd == 1 ? kc : (qd == 2 ? -ks : -kc));  // m_sin
        double cs = qd == 0 ? kc : (qd == 1 ? -ks : (qd == 2 ? -kc : ks));  // m_cos
        if (!finite_arg) sn = cs = nrm - nrm;
        const bool ident = nrm == 0.0;
        const double ew = ident ? 1.0 : cs;
        const double ev = ident ? 0.0 : (d / nrm) * sn;
        // u.q = qmul(e, f.q), component c (w on the fourth lane):
        // w = ((ew bw - ex bx) - ey by) - ez bz, x = ((ew bx + ex bw) + ey bz) - ez by, ...
        const double ex = shfl_d(ev, grp), ey = shfl_d(ev, grp | 4), ez = shfl_d(ev, grp | 8);
        const double fw = F[1], fx = F[2], fy = F[3], fz = F[4];
        const bool wl = c == 3;
        const double b1 = wl ? fw : (c == 0 ? fx : (c == 1 ? fy : fz));
        const double a2 = wl ? ex : (c == 0 ? ex : (c == 1 ? ey : ez));
        const double b2 = wl ? fx : fw;
        const double a3 = wl ? ey : (c == 0 ? ey : (c == 1 ? ez : ex));
        const double b3 = wl ? fy : (c == 0 ? fz : (c == 1 ? fx : fy));
        const double a4 = wl ? ez : (c == 0 ? ez : (c == 1 ? ex : ey));
        const double b4 = wl ? fz : (c == 0 ? fy : (c == 1 ? fz : fx));
        const double P1 = ew * b1, P2 = a2 * b2, P3 = a3 * b3, P4 = a4 * b4;
        const double qn = ((P1 + (wl ? -P2 : P2)) + (wl ? -P3 : P3)) - P4;
        // rigid12 of the new state: row cc of R(q) (qmat), then x
        const double qw = shfl_d(qn, grp | 12), qx = shfl_d(qn, grp), qy = shfl_d(qn, grp | 4),
                     qz = shfl_d(qn, grp | 8);
        const double tc = 2.0 * qn;
        const double tx = shfl_d(tc, grp), ty = shfl_d(tc, grp | 4), tz = shfl_d(tc, grp | 8);
        // row 0: 1 - (tyy + tzz), txy - twz, txz + twy
        // row 1: txy + twz, 1 - (txx + tzz), tyz - twx
        // row 2: txz - twy, tyz + twx, 1 - (txx + tyy)
        const double Pd = (cc == 0 ? ty : tx) * (cc == 0 ? qy : qx);
        const double Qd = (cc == 2 ? ty : tz) * (cc == 2 ? qy : qz);
        const double A1 = (cc == 2 ? tz : ty) * qx;
        const double B1 = (cc == 2 ? ty : tz) * qw;
        const double A2 = tz * (cc == 0 ? qx : qy);
        const double B2 = (cc == 0 ? ty : tx) * qw;
        const double diag = 1.0 - (Pd + Qd);
        const double o1 = A1 + (cc == 1 ? B1 : -B1);
        const double o2 = A2 + (cc == 1 ? -B2 : B2);
        __syncwarp();
        if (act && variant == 0 && c < 3) {
            if (!st) {
                W.imp[c] = imp;
                W.rimp[c] = rimp;
                W.ioff[c] = ioff;
            }
            if (side == 0) {
                if (C.spos >= 0) a.sdelta[3 * (size_t)(c0 + C.spos) + c] = a.is_static[C.a] ? u : -u;
                if (c == 0) {
                    C.impulse = imp1;
                    C.impulse_offset = off1;
                }
            }
        }
        if (act && !st) {
            double* S = variant ? W.FSf : W.FS;
            double* T = (variant ? W.T_FSf : W.T_FS) + 4 * cc;
            if (wl) {
                S[1] = qn;
            } else {
                if (c == 0) S[0] = F[0];
                S[2 + c] = qn;
                S[5 + c] = Lnew;
                S[8 + c] = xnew;
                S[11 + c] = vnew;
                T[c] = diag;
                T[c == 0 ? 1 : 0] = o1;
                T[c == 2 ? 1 : 2] = o2;
                T[3] = xnew;
            }
        }
    }
}

#define SYNC()                           \
    do {                                 \
        if (!solve_sync(S)) {            \
            if (tid == 0) status[k] = 3; \
            return;                      \
        }                                \
    } while (0)

// One chunk of a wave of the friction loop's ordered accumulation
// (sequential_impulses.cpp:560-607) with four lanes per contact: lane bits
// 0-1 pick the component (x, y, z; the fourth lane repeats x and writes
// nothing), eight contacts per warp.  Each lane evaluates its component of
// the reference's vector expressions operation for operation; the cross
// products and norms gather the other components with shuffles.
// Returns whether a contact of this lane's quad changed an impulse by more
// than 1e-4 (the loop's convergence test).
__device__ __forceinline__ bool friction_accumulate4(int base, int end4, const int32_t* __restrict__ widx,
                                                     int w0, int c0, const SolveArgs& a) {
    const int lane = threadIdx.x & 31, quad = lane & ~3, c = lane & 3;
    const int cc = c < 3 ? c : 0;
    const int c1 = cc == 2 ? 0 : cc + 1, c2 = cc == 0 ? 2 : cc - 1;  // cross: a[c1] b[c2] - a[c2] b[c1]
    const int qq = base + lane;
    const bool act = qq < end4;
    ConWork& C = a.cw[c0 + widx[act ? (qq >> 2) : w0]];
    BodyWork &A = a.bw[C.a], &B = a.bw[C.b];
    const bool sa = a.is_static[C.a], sb = a.is_static[C.b];
    const double cnt = (double)C.pair_cnt;
    const double* TA = A.T_FS + 4 * cc;
    const double* TB = B.T_FS + 4 * cc;
    const double p1A = ((TA[0] * C.local_A[0] + TA[1] * C.local_A[1]) + TA[2] * C.local_A[2]) + TA[3] * 1.0;
    const double p1B = ((TB[0] * C.local_B[0] + TB[1] * C.local_B[1]) + TB[2] * C.local_B[2]) + TB[3] * 1.0;
    const double lf = C.upd_total[cc];
    const double u = m_div_recip(lf - C.last_fi[cc], cnt, C.rcnt);
    const double ux = shfl_d(u, quad), uy = shfl_d(u, quad | 1), uz = shfl_d(u, quad | 2);
    const double nu = sqrt((ux * ux + uy * uy) + uz * uz);
    // rfA = (-lf) x (p1A - xA), rfB = lf x (p1B - xB) (calc_torque with -lf)
    const double rA = p1A - A.FS[8 + cc], rB = p1B - B.FS[8 + cc];
    const double nlf = -lf;
    const double rA1 = shfl_d(rA, quad | c1), rA2 = shfl_d(rA, quad | c2);
    const double rB1 = shfl_d(rB, quad | c1), rB2 = shfl_d(rB, quad | c2);
    const double nlf1 = shfl_d(nlf, quad | c1), nlf2 = shfl_d(nlf, quad | c2);
    const double lf1 = shfl_d(lf, quad | c1), lf2 = shfl_d(lf, quad | c2);
    const double rfA = nlf1 * rA2 - nlf2 * rA1;
    const double rfB = lf1 * rB2 - lf2 * rB1;
    const double uo = m_div_recip(0.0 - 0.0, cnt, C.rcnt);
    const double uox = shfl_d(uo, quad), uoy = shfl_d(uo, quad | 1), uoz = shfl_d(uo, quad | 2);
    const double nuo = sqrt((uox * uox + uoy * uoy) + uoz * uoz);
    // roff: (-uo) x (p1A - xA) for A, uo x (p1B - xB) for B (calc_torque with uo, -uo)
    const double nuo_ = -uo;
    const double nuo1 = shfl_d(nuo_, quad | c1), nuo2 = shfl_d(nuo_, quad | c2);
    const double uo1 = shfl_d(uo, quad | c1), uo2 = shfl_d(uo, quad | c2);
    const double roA = nuo1 * rA2 - nuo2 * rA1;
    const double roB = uo1 * rB2 - uo2 * rB1;
    __syncwarp();
    if (act && c < 3) {
        C.last_fi[c] = lf;
        double sd = 0.0;
        if (!sa)
            A.imp[c] = A.imp[c] + u;
        else
            sd = u;
        if (!sb)
            B.imp[c] = B.imp[c] - u;
        else
            sd = -u;
        if (C.spos >= 0) a.sdelta[3 * (size_t)(c0 + C.spos) + c] = sd;
        if (!sa) A.rimp[c] = (A.rimp[c] - C.last_rot_A[c]) + rfA;
        if (!sb) B.rimp[c] = (B.rimp[c] - C.last_rot_B[c]) + rfB;
        C.last_rot_A[c] = rfA;
        C.last_rot_B[c] = rfB;
        if (!sa) A.ioff[c] = A.ioff[c] + uo;
        if (!sb) B.ioff[c] = B.ioff[c] - uo;
        if (!sa) A.roff[c] = A.roff[c] + roA;
        if (!sb) B.roff[c] = B.roff[c] + roB;
    }
    return act && (nu > 1e-4 || nuo > 1e-4);
}

// SequentialImpulses::solve of cluster k.  tid / nt: this thread's index
// among the cluster's threads and their count; G blocks cooperate (G = 1 for
// one block), gb is this block's index among them.  In a grid the indices
// interleave the blocks, so consecutive bodies, contacts and warps of a wave
// land on different SMs.  shv: three ints shared by those threads.
__device__ void solve_body(int k, int tid, int nt, int gb, int G, int* shv, const SolveSync& S,
                           const SolveArgs& a) {
    const int32_t *cl_part_off = a.cl_part_off, *cl_parts = a.cl_parts, *cl_con_off = a.cl_con_off,
                  *order = a.order, *pair_cnt = a.pair_cnt, *con_pair = a.con_pair;
    const double *rec = a.rec, *warm = a.warm, *cl_step = a.cl_step, *mass = a.mass, *ii = a.ii, *mu = a.mu,
                 *cur = a.cur;
    const uint8_t* is_static = a.is_static;
    double* fut = a.fut;
    const double gravity_z = a.gravity_z;
    BodyWork* bw = a.bw;
    ConWork* cw = a.cw;
    int32_t *wave_idx = a.wave_idx, *wave_off = a.wave_off, *wave_cursor = a.wave_cursor, *scon = a.scon;
    double* sdelta = a.sdelta;
    double* static_imp = a.static_imp;
    int32_t *status = a.status, *iters = a.iters, *out_ab = a.out_ab;
    double *out_impulse = a.out_impulse, *pair_warm = a.pair_warm;
    const int p0 = cl_part_off[k], p1 = cl_part_off[k + 1];
    const int c0 = cl_con_off[k], c1 = cl_con_off[k + 1];
    const int nc = c1 - c0;
    const double t = cl_step[k];
    const double rt = 1.0 / t;  // for m_div_recip
    bool ok = true;

    // ---- contacts in sorted order: local frames, normal mass, failure test (:109-168)
    if (tid == 0) shv[0] = 0;
    SYNC();
    for (int i = tid; i < nc; i += nt) {
        ConWork& C = cw[c0 + i];
        const double* h = rec + 14 * (size_t)order[c0 + i];
        const V3 A = ld3(h), B = ld3(h + 3);
        C.a = (int)h[11];
        C.b = (int)h[12];
        C.pair_cnt = pair_cnt[order[c0 + i]];
        C.rcnt = 1.0 / (double)C.pair_cnt;
        C.start_dist = norm(A - B);
        if (C.start_dist < 1e-6 && t > 1e-4) atomicExch(&shv[0], 1);
        double T[16], Ti[16];
        const State fa = load_state(fut + 14 * (size_t)C.a), fb = load_state(fut + 14 * (size_t)C.b);
        transformation(fa.q, fa.x, T);
        mat_inverse(T, Ti);
        st3(C.local_A, xform_general(A, Ti));
        transformation(fb.q, fb.x, T);
        mat_inverse(T, Ti);
        st3(C.local_B, xform_general(B, Ti));
        const V3 gn = (B - A) / 2.0;
        st3(C.n, normalized(gn));
        const V3 rnA = cross(A - fa.x, gn), rnB = cross(B - fb.x, gn);
        double kn = 0.0;
        if (!is_static[C.a]) kn += 1.0 / mass[C.a] + quad_form(rnA, ii + 9 * (size_t)C.a);
        if (!is_static[C.b]) kn += 1.0 / mass[C.b] + quad_form(rnB, ii + 9 * (size_t)C.b);
        C.mass_eff = kn < 1e-6 ? 0.0 : 1.0 / kn;
        C.outer = (h[6] + h[7]) * 0.25;
        // the normal loop's slop and damp * m (sequential_impulses.cpp:
        // 260-287) depend on the contact alone
        C.slop = lerp1(dmax(C.outer * 0.2, C.outer - C.start_dist), C.outer * 0.2, 0.3);
        C.damp_m = 0.1 * C.mass_eff;
        C.impulse = warm[order[c0 + i]] == warm[order[c0 + i]] ? warm[order[c0 + i]] * 0.75 : 0.0;
        C.impulse_offset = 0.0;
        for (int q = 0; q < 3; q++) C.last_fi[q] = C.last_rot_A[q] = C.last_rot_B[q] = 0.0;
    }
    SYNC();
    if (((volatile int*)shv)[0]) {
        if (tid == 0) status[k] = 1;
        return;
    }
    // ---- bodies: gravity impulse, states (:178-188)
    for (int i = p0 + tid; i < p1; i += nt) {
        const int g = cl_parts[i];
        BodyWork& W = bw[g];
        const double m = mass[g];
        W.rmass = 1.0 / m;
        const V3 f = mk(m * 0.0, m * 0.0, m * gravity_z);
        st3(W.imp, f * t);
        for (int q = 0; q < 3; q++) W.rimp[q] = W.ioff[q] = W.roff[q] = 0.0;
        for (int q = 0; q < 14; q++) W.FS[q] = W.FSf[q] = fut[14 * (size_t)g + q];
        const State fs = load_state(fut + 14 * (size_t)g);
        rigid12(fs, W.T_FS);
        rigid12(fs, W.T_FSf);
        rigid12(load_state(cur + 14 * (size_t)g), W.T_cur);
        world_inv_inertia(fs.q, ii + 9 * (size_t)g, W.Iinv);
        W.last_level = -1;
        if (is_static[g]) st3(static_imp + 3 * (size_t)i, f * t);
    }
    SYNC();
    // ---- wave schedule (sequential, integer work only)
    if (tid == 0) {
        int levels = 0;
        for (int i = 0; i < nc; i++) {
            ConWork& C = cw[c0 + i];
            int lv = 0;
            if (!is_static[C.a]) lv = max(lv, bw[C.a].last_level + 1);
            if (!is_static[C.b]) lv = max(lv, bw[C.b].last_level + 1);
            C.level = lv;
            if (!is_static[C.a]) bw[C.a].last_level = lv;
            if (!is_static[C.b]) bw[C.b].last_level = lv;
            levels = max(levels, lv + 1);
        }
        for (int l = 0; l <= levels; l++) wave_off[c0 + k + l] = 0;
        for (int i = 0; i < nc; i++) wave_off[c0 + k + cw[c0 + i].level + 1]++;
        for (int l = 0; l < levels; l++) wave_off[c0 + k + l + 1] += wave_off[c0 + k + l];
        // stable scatter: contacts of each wave in sorted order
        int32_t* cursor = wave_cursor + c0 + k;
        for (int l = 0; l < levels; l++) cursor[l] = wave_off[c0 + k + l];
        for (int i = 0; i < nc; i++) wave_idx[c0 + cursor[cw[c0 + i].level]++] = i;
        // the contacts touching a static body, in sorted order, for its impulse
        // sums: each writes its delta at its position, scon holds the body
        int ns = 0;
        for (int i = 0; i < nc; i++) {
            ConWork& C = cw[c0 + i];
            const bool sa = is_static[C.a], sb = is_static[C.b];
            C.spos = (sa || sb) ? ns : -1;
            if (sa || sb) scon[c0 + ns++] = sa ? C.a : C.b;
        }
        shv[1] = levels;
        shv[2] = ns;
    }
    SYNC();
    const int levels = ((volatile int*)shv)[1];
    const int n_scon = ((volatile int*)shv)[2];
    const int* woff = wave_off + c0 + k;
    const int* widx = wave_idx + c0;

    // Static impulse sums: add the contacts' deltas in sorted order.
    auto static_sum = [&]() {
        for (int i = p0 + tid; i < p1; i += nt) {
            const int g = cl_parts[i];
            if (!is_static[g]) continue;
            V3 s = ld3(static_imp + 3 * (size_t)i);
            for (int q = 0; q < n_scon; q++)
                if (scon[c0 + q] == g) s = s + ld3(sdelta + 3 * (size_t)(c0 + q));
            st3(static_imp + 3 * (size_t)i, s);
        }
    };

    // ---- warm-start impulses (:193-215), in waves
    for (int l = 0; l < levels; l++) {
        for (int q = woff[l] + tid; q < woff[l + 1]; q += nt) {
            ConWork& C = cw[c0 + widx[q]];
            BodyWork &A = bw[C.a], &B = bw[C.b];
            const V3 n = ld3(C.n);
            const V3 p1A = xf12(ld3(C.local_A), A.T_FS), p1B = xf12(ld3(C.local_B), B.T_FS);
            const V3 u = (-n) * C.impulse;
            V3 sd = mk(0, 0, 0);
            if (!is_static[C.a]) {
                st3(A.imp, ld3(A.imp) + u);
                st3(A.rimp, ld3(A.rimp) + calc_torque(u, p1A, ld3(A.FS + 8)));
            } else {
                sd = u;
            }
            if (!is_static[C.b]) {
                st3(B.imp, ld3(B.imp) - u);
                st3(B.rimp, ld3(B.rimp) + calc_torque(-u, p1B, ld3(B.FS + 8)));
            } else {
                sd = -u;
            }
            if (C.spos >= 0) st3(sdelta + 3 * (size_t)(c0 + C.spos), sd);
        }
        SYNC();
    }
    static_sum();
    SYNC();
    for (int k2 = tid; k2 < 2 * (p1 - p0); k2 += nt) {  // two lanes per body: FS, FSf
        const int g = cl_parts[p0 + (k2 >> 1)];
        if (!is_static[g]) integrate_one(bw[g], fut + 14 * (size_t)g, mass[g], t, k2 & 1);
    }
    SYNC();

    int it_n = 0, it_f = 0;
    if (nc > 0) {
        // ---- normal loop (:230-395)
        bool converged = false;
        // every iteration compares the moving bodies' impulses with their values
        // at its start (kept in last_imp, refreshed by the convergence test);
        // static bodies keep their running sums in static_imp
        for (int i = p0 + tid; i < p1; i += nt) {
            const int g = cl_parts[i];
            if (!is_static[g])
                for (int q = 0; q < 3; q++) bw[g].last_imp[q] = bw[g].imp[q];
        }
        SYNC();
        // Narrow waves (a warp of two contacts per SM sub-partition) take
        // sixteen lanes per contact, wider ones four.  The next wave's bounds
        // and first sixteen-lane task are loaded before each barrier.
        auto lanes16 = [&](int w0, int w1) { return a.lanes == 16 || (a.lanes == 0 && (w1 - w0 + 1) / 2 <= 4 * G); };
        int n0 = woff[0], n1 = woff[1];
        int2 pre = lanes16(n0, n1) ? wave16_first(n0, n1, widx, c0, G, gb, a) : make_int2(-1, -1);
        while (!converged && it_n < 1000) {
            for (int l = 0; l < levels; l++) {
                const int w0 = n0, w1 = n1;
                const int ln = l + 1 < levels ? l + 1 : 0;
                n0 = woff[ln];
                n1 = woff[ln + 1];
                if (lanes16(w0, w1)) {
                    // the next wave's first task, loaded while this wave computes
                    const int2 pre_next =
                        lanes16(n0, n1) ? wave16_first(n0, n1, widx, c0, G, gb, a) : make_int2(-1, -1);
                    normal_wave16(w0, w1, widx, c0, G, gb, t, rt, pre, a);
                    pre = pre_next;
                    SYNC();
                    continue;
                }
                // Four lanes per contact, one warp instruction stream: lane bit 0
                // picks the body side (A, B), bit 1 the integrated state (FS,
                // FSf).  FP64 latency, not lane count, bounds a wave, so the
                // sides and the four integrations run side by side.
                const int end4 = 4 * w1;
                const int wslot = (int)(threadIdx.x >> 5) * G + gb, nwarps = (int)(blockDim.x >> 5) * G;
                for (int base = 4 * w0 + 32 * wslot; base < end4; base += 32 * nwarps) {
                    const int lane = threadIdx.x & 31, quad = lane & ~3, side = lane & 1, variant = (lane >> 1) & 1;
                    const int qq = base + lane;
                    const bool act = qq < end4;
                    ConWork& C = cw[c0 + widx[act ? (qq >> 2) : w0]];
                    const int g = side ? C.b : C.a;
                    BodyWork& W = bw[g];
                    const bool st = is_static[g];
                    // this side's contact point and its velocity (State::pointVelocity)
                    const V3 p1 = xf12(ld3(side ? C.local_B : C.local_A), W.T_FS);
                    const V3 x = ld3(W.FS + 8);
                    const V3 v1s = ld3(W.FS + 11) + cross(m3_vec(ii + 9 * (size_t)g, ld3(W.FS + 5)), p1 - x);
                    const V3 p1A = shfl3(p1, quad), p1B = shfl3(p1, quad + 1);
                    const V3 v1A = shfl3(v1s, quad), v1B = shfl3(v1s, quad + 1);
                    const bool sa = is_static[C.a];
                    const V3 n = ld3(C.n);
                    const double outer = C.outer;
                    const double d1 = dot(p1B, n) - dot(p1A, n);
                    const double v1 = dot(v1A, n) - dot(v1B, n);
                    const double m = C.mass_eff;
                    const double damp = 0.1;
                    const double imp0 = C.impulse, off0 = C.impulse_offset;
                    const double dimp = d1 < outer ? (v1 * m) * damp : -imp0;
                    const double imp1 = dmax(imp0 + dimp, 0.0);
                    const V3 u = (-n) * (imp1 - imp0);
                    const double pen = outer - d1;
                    const double doff = d1 < outer ? m_div_recip(C.damp_m * dmax(0.0, pen - C.slop), t, rt) : -off0;
                    const double off1 = dmax(off0 + doff, 0.0);
                    const V3 uo = (-n) * (off1 - off0);
                    __syncwarp();
                    if (act && variant == 0) {
                        if (!st) {  // imp[b] - u is imp[b] + (-u) in IEEE arithmetic
                            const V3 us = side ? -u : u;
                            st3(W.imp, ld3(W.imp) + us);
                            st3(W.rimp, ld3(W.rimp) + calc_torque(us, p1, x));
                            st3(W.ioff, ld3(W.ioff) + (side ? -uo : uo));
                        }
                        if (side == 0) {
                            C.impulse = imp1;
                            C.impulse_offset = off1;
                            if (C.spos >= 0) st3(sdelta + 3 * (size_t)(c0 + C.spos), sa ? u : -u);
                        }
                    }
                    __syncwarp();
                    if (act && !st) integrate_one(W, fut + 14 * (size_t)g, mass[g], t, variant);
                }
                pre = lanes16(n0, n1) ? wave16_first(n0, n1, widx, c0, G, gb, a) : make_int2(-1, -1);
                SYNC();
            }
            // convergence over every particle of the cluster (:380-387)
            bool moved = false;
            for (int i = p0 + tid; i < p1; i += nt) {
                const int g = cl_parts[i];
                if (is_static[g]) {
                    const V3 before = ld3(static_imp + 3 * (size_t)i);
                    V3 s = before;
                    for (int q = 0; q < n_scon; q++)
                        if (scon[c0 + q] == g) s = s + ld3(sdelta + 3 * (size_t)(c0 + q));
                    st3(static_imp + 3 * (size_t)i, s);
                    if (norm(s - before) > 1e-6) moved = true;
                } else {
                    const V3 now = ld3(bw[g].imp);
                    if (norm(now - ld3(bw[g].last_imp)) > 1e-6) moved = true;
                    st3(bw[g].last_imp, now);
                }
            }
            converged = !solve_any(S, moved, it_n & 1, gb, &ok);
            if (!ok) {
                if (tid == 0) status[k] = 3;
                return;
            }
            it_n++;
        }
        // ---- friction loop (:397-607)
        converged = false;
        while (!converged && it_f < 100) {
            for (int i = tid; i < nc; i += nt) {  // pass 1: every contact reads, none writes bodies
                ConWork& C = cw[c0 + i];
                const BodyWork &A = bw[C.a], &B = bw[C.b];
                const bool sa = is_static[C.a], sb = is_static[C.b];
                const double* h = rec + 14 * (size_t)order[c0 + i];
                const V3 n = ld3(C.n);
                const V3 p1A = xf12(ld3(C.local_A), A.T_FS), p1B = xf12(ld3(C.local_B), B.T_FS);
                const V3 v1A = sa ? mk(0, 0, 0)
                                  : ld3(A.FS + 11) + cross(m3_vec(ii + 9 * (size_t)C.a, ld3(A.FS + 5)), p1A - ld3(A.FS + 8));
                const V3 v1B = sb ? mk(0, 0, 0)
                                  : ld3(B.FS + 11) + cross(m3_vec(ii + 9 * (size_t)C.b, ld3(B.FS + 5)), p1B - ld3(B.FS + 8));
                const V3 lpA = xf12(ld3(C.local_A), A.T_cur), fpA = xf12(ld3(C.local_A), A.T_FSf);
                const V3 vdA = (fpA - lpA) / t;
                const V3 lpB = xf12(ld3(C.local_B), B.T_cur), fpB = xf12(ld3(C.local_B), B.T_FSf);
                const V3 vdB = (fpB - lpB) / t;
                const V3 vAB = v1A - v1B;
                const V3 vABd = vdA - vdB;
                const V3 vt = vAB - dot(vAB, n) * n;
                (void)vABd;
                const double mu_ = dmin(mu[C.a], mu[C.b]);
                const double max_force = (C.impulse * mu_) * 10;
                const V3 rA = ld3(h) - ld3(fut + 14 * (size_t)C.a + 8);
                const V3 rB = ld3(h + 3) - ld3(fut + 14 * (size_t)C.b + 8);
                const V3 tan = normalized(vt);
                double kt = 0.0;
                if (!sa) kt += A.rmass + quad_form(cross(rA, tan), ii + 9 * (size_t)C.a);  // 1.0 / mass
                if (!sb) kt += B.rmass + quad_form(cross(rB, tan), ii + 9 * (size_t)C.b);
                const double mit = kt < 1e-6 ? 0.0 : 1.0 / kt;
                const V3 dfi = ((-vt) * mit) * 0.9;
                V3 total = ld3(C.last_fi) + dfi;
                total = normalized(total) * dclamp(norm(total), 0.0, max_force);
                st3(C.upd_total, total);
            }
            SYNC();
            bool big = false;
            for (int l = 0; l < levels; l++) {  // pass 2: ordered accumulation, wave by wave
                const int end4 = 4 * woff[l + 1];
                const int wslot = (int)(threadIdx.x >> 5) * G + gb, nwarps = (int)(blockDim.x >> 5) * G;
                for (int base = 4 * woff[l] + 32 * wslot; base < end4; base += 32 * nwarps)
                    big = friction_accumulate4(base, end4, widx, woff[l], c0, a) || big;
                SYNC();
            }
            // (the static bodies' impulse sums are read only by the normal loop's test)
            for (int k2 = tid; k2 < 2 * (p1 - p0); k2 += nt) {  // two lanes per body: FS, FSf
                const int g = cl_parts[p0 + (k2 >> 1)];
                if (!is_static[g]) integrate_one(bw[g], fut + 14 * (size_t)g, mass[g], t, k2 & 1);
            }
            converged = !solve_any(S, big, (it_n + it_f) & 1, gb, &ok);
            if (!ok) {
                if (tid == 0) status[k] = 3;
                return;
            }
            it_f++;
        }
    }
    SYNC();
    // ---- write back (:622-624) and the contacts' impulses for the warm start
    for (int i = p0 + tid; i < p1; i += nt) {
        const int g = cl_parts[i];
        if (!is_static[g])
            for (int q = 0; q < 14; q++) fut[14 * (size_t)g + q] = bw[g].FS[q];
    }
    for (int i = tid; i < nc; i += nt) {
        out_impulse[c0 + i] = cw[c0 + i].impulse;
        out_ab[2 * (c0 + i)] = cw[c0 + i].a;
        out_ab[2 * (c0 + i) + 1] = cw[c0 + i].b;
    }
    if (tid == 0) {
        status[k] = 0;
        iters[2 * k] = it_n;
        iters[2 * k + 1] = it_f;
        // Warm-start store (sequential_impulses_warm_start.cpp:28-54): each
        // body pair keeps the impulse of its last contact in sorted order;
        // a pair's first contact enters as 0.0 + impulse.
        if (pair_warm)
            for (int i = 0; i < nc; i++) {
                const int oi = order[c0 + i];
                pair_warm[con_pair[oi]] = pair_cnt[oi] == 1 ? 0.0 + cw[c0 + i].impulse : cw[c0 + i].impulse;
            }
    }
}

#undef SYNC

// One block per cluster (clusters cl_list[b], or b when cl_list is null).
__global__ void __launch_bounds__(kSolveBlock) k_solve(int n_list, const int32_t* __restrict__ cl_list, SolveArgs a) {
    if ((int)blockIdx.x >= n_list) return;
    __shared__ int s_local[3];
    const SolveSync S{kSyncBlock, nullptr, nullptr, nullptr, 0u};
    solve_body(cl_list ? cl_list[blockIdx.x] : (int)blockIdx.x, threadIdx.x, blockDim.x, 0, 1, s_local, S, a);
}

// Every block of a cooperative grid on cluster k (all blocks resident).
__global__ void __launch_bounds__(kSolveBlock) k_solve_grid(int k, SolveSync S, SolveArgs a) {
    __shared__ unsigned long long s_passed;
    if (threadIdx.x == 0) s_passed = 0;
    __syncthreads();
    S.passed = &s_passed;
    solve_body(k, threadIdx.x * gridDim.x + blockIdx.x, gridDim.x * blockDim.x, blockIdx.x, gridDim.x, S.flags, S,
               a);
}

// The blocks of thread-block cluster c solve cluster cl_list[c] together
// (every block of a hardware cluster is resident at once); flags: 16 ints
// per hardware cluster, zeroed before the launch.
__global__ void __launch_bounds__(kSolveBlock) k_solve_cl(const int32_t* __restrict__ cl_list,
                                                          int32_t* __restrict__ flags, SolveArgs a) {
    unsigned int rank, nrank, cid;
    asm("mov.u32 %0, %%cluster_ctarank;" : "=r"(rank));
    asm("mov.u32 %0, %%cluster_nctarank;" : "=r"(nrank));
    asm("mov.u32 %0, %%clusterid.x;" : "=r"(cid));
    int32_t* f = flags + 16 * (size_t)cid;
    const SolveSync S{kSyncCluster, nullptr, nullptr, f, 0u};
    solve_body(cl_list[cid], threadIdx.x * nrank + rank, (int)(nrank * blockDim.x), (int)rank, (int)nrank, f, S, a);
}

// Sort key of Contact::operator< (contact.h:17-21) as orderable bits
// (proportions are >= +0).
__global__ void k_prop_keys(int n, const double* __restrict__ rec, unsigned long long* __restrict__ keys,
                            int32_t* __restrict__ vals) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* h = rec + 14 * (size_t)i;
    const double prop = norm(mk(h[0] - h[3], h[1] - h[4], h[2] - h[5])) / (h[6] + h[7]);
    keys[i] = (unsigned long long)__double_as_longlong(prop);
    vals[i] = i;
}

#define VLAUNCH(kern, n, ...)                                        \
    do {                                                             \
        kern<<<nblocks(n), kBlock, 0, ctx->stream>>>(__VA_ARGS__);   \
        ctx->eng.launches++;                                         \
    } while (0)
#define RC(x)                          \
    do {                               \
        if (int rc_ = (x)) return rc_; \
    } while (0)

}  // namespace

// Per-pair filterContacts of contact records grouped by pair (d_rec /
// d_off over n_pairs), into flt (records) / flt_off / flt_cnt (kept per pair).
int run_filter(d2g_ctx* ctx, const int32_t* d_off, const double* d_rec, int n_pairs, int n_rec, double margin,
               int* n_out) {
    Engine& E = ctx->eng;
    cudaStream_t s = ctx->stream;
    const size_t n = (size_t)n_rec;
    RC(E.flt_keys.ensure(n + 1));
    RC(E.flt_keys_s.ensure(n + 1));
    RC(E.flt_idx.ensure(n + 1));
    RC(E.flt_order.ensure(n + 1));
    RC(E.flt_keep.ensure(n + 1));
    RC(E.flt_pos.ensure(n + 1));
    RC(E.flt_mid.ensure(3 * n + 3));
    RC(E.flt_cnt.ensure(n_pairs + 1));
    RC(E.flt_off.ensure(n_pairs + 1));
    if (n_rec > 0 && n_pairs > 0) {
        // stable sort by |A - B|, then stable by eps_a + eps_b: lexicographic, ties in input order
        VLAUNCH(k_filter_keys, n_rec, n_rec, d_rec, E.flt_keys.p, E.flt_idx.p);
        size_t bytes = 0;
        D2G_CUDA(cub::DeviceSegmentedSort::StableSortPairs(nullptr, bytes, E.flt_keys.p, E.flt_keys_s.p, E.flt_idx.p,
                                                          E.flt_order.p, n_rec, n_pairs, d_off, d_off + 1, s));
        RC(E.cub_tmp.ensure(bytes + 16));
        D2G_CUDA(cub::DeviceSegmentedSort::StableSortPairs(E.cub_tmp.p, bytes, E.flt_keys.p, E.flt_keys_s.p,
                                                          E.flt_idx.p, E.flt_order.p, n_rec, n_pairs, d_off,
                                                          d_off + 1, s));
        VLAUNCH(k_filter_eps_keys, n_rec, n_rec, d_rec, E.flt_order.p, E.flt_keys.p);
        bytes = 0;
        D2G_CUDA(cub::DeviceSegmentedSort::StableSortPairs(nullptr, bytes, E.flt_keys.p, E.flt_keys_s.p,
                                                          E.flt_order.p, E.flt_idx.p, n_rec, n_pairs, d_off,
                                                          d_off + 1, s));
        RC(E.cub_tmp.ensure(bytes + 16));
        D2G_CUDA(cub::DeviceSegmentedSort::StableSortPairs(E.cub_tmp.p, bytes, E.flt_keys.p, E.flt_keys_s.p,
                                                          E.flt_order.p, E.flt_idx.p, n_rec, n_pairs, d_off,
                                                          d_off + 1, s));
        // E.flt_idx now holds the sorted order
        k_filter_dedupe<<<nblocks(32LL * n_pairs), kBlock, 0, s>>>(n_pairs, d_off, E.flt_idx.p, d_rec, margin,
                                                                    E.flt_keep.p, E.flt_cnt.p, E.flt_mid.p);
        ctx->eng.launches++;
    } else if (n_pairs > 0) {
        D2G_CUDA(cudaMemsetAsync(E.flt_cnt.p, 0, sizeof(int32_t) * n_pairs, s));
    }
    RC(E.flt_keep.ensure(n + 1));
    if (n_rec > 0) {
        size_t bytes = 0;
        D2G_CUDA(cudaMemsetAsync(E.flt_pos.p, 0, sizeof(int32_t), s));
        D2G_CUDA(cub::DeviceScan::InclusiveSum(nullptr, bytes, E.flt_keep.p, E.flt_pos.p + 1, n_rec, s));
        RC(E.cub_tmp.ensure(bytes + 16));
        D2G_CUDA(cub::DeviceScan::InclusiveSum(E.cub_tmp.p, bytes, E.flt_keep.p, E.flt_pos.p + 1, n_rec, s));
        VLAUNCH(k_filter_offsets, n_pairs + 1, n_pairs, d_off, E.flt_pos.p, E.flt_off.p);
    } else {
        D2G_CUDA(cudaMemsetAsync(E.flt_off.p, 0, sizeof(int32_t) * (n_pairs + 1), s));
    }
    D2G_CUDA(cudaMemcpyAsync(ctx->h_pinned, E.flt_off.p + n_pairs, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    D2G_CUDA(cudaStreamSynchronize(s));
    prof_mark_collect(ctx);
    const int kept = ctx->h_pinned[0];
    RC(E.flt.ensure(14 * (size_t)kept + 14));
    if (n_rec > 0) VLAUNCH(k_filter_write, n_rec, n_rec, E.flt_idx.p, E.flt_keep.p, E.flt_pos.p, d_rec, E.flt.p);
    *n_out = kept;
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

// Thread-block clusters of `cs` solve blocks that can be resident at once
// (cached per context).
int max_solve_clusters(d2g_ctx* ctx, int cs, int* out) {
    Engine& E = ctx->eng;
    const int slot = cs == 16 ? 0 : cs == 8 ? 1 : cs == 4 ? 2 : 3;
    if (E.sv_cl_fit[slot] < 0) {
        if (cs > 8)
            D2G_CUDA(cudaFuncSetAttribute((const void*)k_solve_cl, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cs);
        cfg.blockDim = dim3(kSolveBlock);
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = cs;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, (const void*)k_solve_cl, &cfg) != cudaSuccess) {
            (void)cudaGetLastError();  // this size is not available: never chosen
            n = 0;
        }
        E.sv_cl_fit[slot] = n;
    }
    *out = E.sv_cl_fit[slot];
    return D2G_OK;
}

// k_solve_cl over n clusters (list d_list), cs blocks each.
int launch_solve_cl(d2g_ctx* ctx, int cs, int n, const int32_t* d_list, int32_t* d_flags, const SolveArgs& a,
                    cudaStream_t st) {
    if (cs > 8)
        D2G_CUDA(cudaFuncSetAttribute((const void*)k_solve_cl, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(n * cs));
    cfg.blockDim = dim3(kSolveBlock);
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    D2G_CUDA(cudaLaunchKernelEx(&cfg, k_solve_cl, d_list, d_flags, a));
    ctx->eng.launches++;
    return D2G_OK;
}

// Solve clusters.  Contacts (14-double records in the reference's hit order,
// clusters contiguous per d_con_off) with per-contact pair counts and warm
// values (NaN = none).  Outputs: status / iteration counts per cluster, the
// final impulse and body pair of each contact in sorted order.
int run_solve(d2g_ctx* ctx, int n_clusters, const int32_t* d_part_off, const int32_t* d_parts, int n_parts,
              const int32_t* d_con_off, int n_con, const double* d_rec, const int32_t* d_pair_cnt,
              const double* d_warm, const double* d_step, double gravity_z, int32_t* d_status, int32_t* d_iters,
              double* d_out_impulse, int32_t* d_out_ab, const int32_t* d_con_pair, double* d_pair_warm,
              const int32_t* h_con_off, const int32_t* h_part_off) {
    Engine& E = ctx->eng;
    cudaStream_t s = ctx->stream;
    RC(E.sv_scon.ensure(n_con + 1));
    RC(E.sv_sdelta.ensure(3 * (size_t)n_con + 3));
    RC(E.sv_keys.ensure(n_con + 1));
    RC(E.sv_keys_out.ensure(n_con + 1));
    RC(E.sv_vals.ensure(n_con + 1));
    RC(E.sv_order.ensure(n_con + 1));
    RC(E.sv_bw_raw.ensure(sizeof(BodyWork) * ((size_t)ctx->n_bodies + 1)));
    RC(E.sv_cw_raw.ensure(sizeof(ConWork) * ((size_t)n_con + 1)));
    BodyWork* bw = (BodyWork*)E.sv_bw_raw.p;
    ConWork* cw = (ConWork*)E.sv_cw_raw.p;
    RC(E.sv_wave_idx.ensure(n_con + 1));
    RC(E.sv_wave_off.ensure(n_con + n_clusters + 2));
    RC(E.sv_wave_cursor.ensure(n_con + n_clusters + 2));
    RC(E.sv_static_imp.ensure(3 * (size_t)n_parts + 3));
    if (n_con > 0) {
        VLAUNCH(k_prop_keys, n_con, n_con, d_rec, E.sv_keys.p, E.sv_vals.p);
        size_t bytes = 0;
        D2G_CUDA(cub::DeviceSegmentedRadixSort::SortPairs(nullptr, bytes, E.sv_keys.p, E.sv_keys_out.p, E.sv_vals.p,
                                                          E.sv_order.p, n_con, n_clusters, d_con_off, d_con_off + 1,
                                                          0, 64, s));
        RC(E.cub_tmp.ensure(bytes + 16));
        D2G_CUDA(cub::DeviceSegmentedRadixSort::SortPairs(E.cub_tmp.p, bytes, E.sv_keys.p, E.sv_keys_out.p,
                                                          E.sv_vals.p, E.sv_order.p, n_con, n_clusters, d_con_off,
                                                          d_con_off + 1, 0, 64, s));
    }
    if (n_clusters > 0) {
        SolveArgs a;
        a.cl_part_off = d_part_off;
        a.cl_parts = d_parts;
        a.cl_con_off = d_con_off;
        a.order = E.sv_order.p;
        a.rec = d_rec;
        a.pair_cnt = d_pair_cnt;
        a.warm = d_warm;
        a.cl_step = d_step;
        a.is_static = ctx->is_static.p;
        a.mass = ctx->mass.p;
        a.ii = ctx->inv_inertia.p;
        a.mu = ctx->mu.p;
        a.cur = ctx->cur.p;
        a.fut = ctx->fut.p;
        a.gravity_z = gravity_z;
        a.bw = bw;
        a.cw = cw;
        a.wave_idx = E.sv_wave_idx.p;
        a.wave_off = E.sv_wave_off.p;
        a.wave_cursor = E.sv_wave_cursor.p;
        a.scon = E.sv_scon.p;
        a.sdelta = E.sv_sdelta.p;
        a.static_imp = E.sv_static_imp.p;
        a.status = d_status;
        a.iters = d_iters;
        a.out_impulse = d_out_impulse;
        a.out_ab = d_out_ab;
        a.con_pair = d_con_pair;
        a.pair_warm = d_pair_warm;
        a.lanes = E.tune[D2G_TUNE_SOLVE_LANES];
        // Where each cluster is solved.  A wave holds at most one contact per
        // moving body and lasts about one contact's dependent FP64 chain when
        // its warps each have an SM sub-partition to themselves: a block runs
        // waves of up to eight contacts that way, a thread-block cluster of
        // 16 blocks up to 128 (with a hardware barrier, ~0.2 us, between
        // waves), a cooperative grid over all SMs any width (~1.5 us per
        // grid barrier).  So a cluster with at least 128 contacts and more
        // than D2G_TUNE_GRID_MIN_PARTS parts takes a grid when at most 8
        // clusters of the call qualify (grids run one after another); any
        // other cluster of at least 32 contacts takes a thread-block cluster
        // (D2G_TUNE_SOLVE_CLUSTER blocks, or the most that lets every such
        // cluster be resident at once); the rest one block each.  Blocks and
        // thread-block clusters run side by side on two streams, the grids
        // after them.
        const int cl_setting = E.tune[D2G_TUNE_SOLVE_CLUSTER];
        std::vector<int32_t> small, mid, big;
        if (h_con_off && h_part_off)
            for (int c = 0; c < n_clusters; c++)
                if (h_con_off[c + 1] - h_con_off[c] >= kGridMinContacts &&
                    h_part_off[c + 1] - h_part_off[c] > E.tune[D2G_TUNE_GRID_MIN_PARTS])
                    big.push_back(c);
        if ((int)big.size() > kGridMaxClusters) big.clear();
        for (int c = 0, b = 0; c < n_clusters; c++) {
            if (b < (int)big.size() && big[b] == c) {
                b++;
                continue;
            }
            const int nck = h_con_off ? h_con_off[c + 1] - h_con_off[c] : 0;
            if (h_con_off && cl_setting != 1 && nck >= kClusterMinContacts)
                mid.push_back(c);
            else
                small.push_back(c);
        }
        int cs = 1;  // blocks per thread-block cluster
        if (!mid.empty()) {
            if (cl_setting > 1) {
                cs = cl_setting;
            } else {
                for (int cand : {16, 8, 4, 2}) {
                    int fit = 0;
                    RC(max_solve_clusters(ctx, cand, &fit));
                    if (fit >= (int)mid.size()) {
                        cs = cand;
                        break;
                    }
                }
            }
            if (cs == 1) {  // too many to be resident at once: one block each
                small.insert(small.end(), mid.begin(), mid.end());
                std::sort(small.begin(), small.end());
                mid.clear();
            }
        }
        const bool all_small = mid.empty() && big.empty();
        E.sv_layout[0] = (int)small.size();
        E.sv_layout[1] = (int)mid.size();
        E.sv_layout[2] = (int)big.size();
        E.sv_layout[3] = mid.empty() ? 0 : cs;
        const int pf = prof_mark_begin(ctx, PROF_SOLVE, n_con);
        RC(E.sv_list.ensure(small.size() + mid.size() + 2));
        if (!small.empty()) {
            const int32_t* d_list = nullptr;
            if (!all_small) {
                D2G_CUDA(cudaMemcpyAsync(E.sv_list.p, small.data(), small.size() * sizeof(int32_t),
                                         cudaMemcpyHostToDevice, s));
                d_list = E.sv_list.p;
            }
            k_solve<<<(int)small.size(), kSolveBlock, 0, s>>>((int)small.size(), d_list, a);
            ctx->eng.launches++;
        }
        if (!mid.empty()) {
            // on the second stream, beside the blocks
            int32_t* d_mid = E.sv_list.p + small.size() + 1;
            RC(E.sv_cl_flags.ensure(16 * mid.size() + 16));
            D2G_CUDA(cudaMemcpyAsync(d_mid, mid.data(), mid.size() * sizeof(int32_t), cudaMemcpyHostToDevice, s));
            D2G_CUDA(cudaMemsetAsync(E.sv_cl_flags.p, 0, (16 * mid.size() + 16) * sizeof(int32_t), s));
            D2G_CUDA(cudaEventRecord(ctx->ev_fork, s));
            D2G_CUDA(cudaStreamWaitEvent(ctx->stream2, ctx->ev_fork, 0));
            RC(launch_solve_cl(ctx, cs, (int)mid.size(), d_mid, E.sv_cl_flags.p, a, ctx->stream2));
            D2G_CUDA(cudaEventRecord(ctx->ev_join, ctx->stream2));
            D2G_CUDA(cudaStreamWaitEvent(s, ctx->ev_join, 0));
        }
        if (!big.empty()) {
            int dev_sms = 0, per_sm = 0;
            D2G_CUDA(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device));
            D2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_solve_grid, kSolveBlock, 0));
            const int G_max = std::max(1, std::min(dev_sms, dev_sms * per_sm));
            RC(E.sv_grid.ensure(16 * big.size() + 16));
            D2G_CUDA(cudaMemsetAsync(E.sv_grid.p, 0, (16 * big.size() + 16) * sizeof(int32_t), s));
            for (size_t b = 0; b < big.size(); b++) {
                SolveSync S;
                S.mode = kSyncGrid;
                S.count = (unsigned long long*)(E.sv_grid.p + 16 * b);  // 8-byte aligned: 16 ints per cluster
                S.passed = nullptr;
                S.flags = E.sv_grid.p + 16 * b + 4;
                S.spin_limit = (unsigned int)E.tune[D2G_TUNE_SPIN_LIMIT];
                int k = big[b];
                // about one warp of contacts per SM and wave: fewer blocks for
                // smaller clusters keep the grid barriers cheap
                const int nck = h_con_off[k + 1] - h_con_off[k];
                const int G = std::max(1, std::min(G_max, std::max(8, nck / E.tune[D2G_TUNE_GRID_CONTACTS])));
                void* args[] = {&k, &S, &a};
                D2G_CUDA(cudaLaunchCooperativeKernel((const void*)k_solve_grid, dim3(G), dim3(kSolveBlock), args, 0,
                                                     s));
                ctx->eng.launches++;
            }
        }
        prof_mark_end(ctx, pf);
    }
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

}  // namespace d2g
