// CCD-driven time-step selection for many clusters at once.
//
// Restates fineCollisionClustersWithTimeStepSelection
// (collision_detection/separate_clusters.cpp:462-599) and the clamp of
// TimeStepSelectionDynamicContinuous::selectTimeStep
// (strategies/time_step_size/time_step_selection_dynamic_continuous.cpp:17-21):
//   1. one CCD query per interaction (all clusters' interactions in one
//      engine call, max_time = min(last_dt_a, last_dt_b));
//   2. one thread per interaction: the step scale each of its contacts asks
//      for, and their minimum (order-independent: NaN never wins a min);
//   3. one thread per cluster: the reference's order-dependent propagation
//      step[a] = step[b] = min(new_dt, step[a], step[b]) over the cluster's
//      interactions in order, then the cluster step and its clamp.
#include "d2g_geom.cuh"
#include "d2g_internal.hpp"

namespace d2g {

namespace {

constexpr int kBlock = 128;
inline int nblocks(long long n, int b = kBlock) { return (int)((n + b - 1) / b); }

// separate_clusters.cpp:497-554: the scale one continuous contact asks for
// (Ia, Ib: the future world inverse inertias, Particle::futurePointVelocity).
__device__ double contact_step_scale(const double* c, const State& fa, const double* Ia, const State& fb,
                                     const double* Ib, double max_dt) {
    double scale = 1.0;
    const V3 A = mk(c[0], c[1], c[2]), B = mk(c[3], c[4], c[5]);
    const double toc = c[10];
    const V3 hit_normal = A - B;
    const double interaction_dist = c[6] + c[7];
    const V3 a_vel = fa.v + cross(m3_vec(Ia, fa.L), A - fa.x);
    const V3 b_vel = fb.v + cross(m3_vec(Ib, fb.L), B - fb.x);
    const V3 rel = a_vel - b_vel;
    if (dot(normalized(hit_normal), normalized(rel)) <= 0.0 || norm(hit_normal) < 1e-4) {
        if (norm(hit_normal) < 1e-4) {
            if (toc == 0.0) return 1.0;
            const double toc_start = dmax(0.0, toc - (norm(rel) * max_dt) / interaction_dist);
            scale = dmin(scale, lerp1(toc_start, toc, 0.75));
        } else if (toc < 1.0) {
            const double proj_vel = -(dot(normalized(hit_normal), rel));
            const double depth = interaction_dist - norm(hit_normal);
            const double proj_dist = (proj_vel * toc) * max_dt;
            if (proj_dist > 1e-6) {
                if (depth < proj_dist) {
                    scale = dmin(scale, lerp1(toc * (1.0 - depth / proj_dist), toc, 0.5));
                } else {
                    const double future_point = toc + ((1.0 - toc) * interaction_dist) / (proj_vel * max_dt);
                    scale = dmin(scale, lerp1(toc, dmin(future_point, 1.0), 0.8));
                }
            }
        }
    }
    return scale;
}

// min(b, a) as (b < a) ? b : a, through an integer compare when both are
// finite and non-negative (their bit patterns order like the values, and
// equal values have equal bits); the FP64 compare otherwise.
__device__ __forceinline__ double dmin_fast(double a, double b) {
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    if ((ia | ib) >= 0 && ia < 0x7ff0000000000000LL && ib < 0x7ff0000000000000LL) return ib < ia ? b : a;
    return b < a ? b : a;
}

// One warp per interaction (separate_clusters.cpp:494-562): every contact's
// scale in parallel, then the reference's running minimum from 1.0, which
// keeps the first of equal values and never takes a NaN, as a leftmost-
// minimum reduction over (value, contact index).
__global__ void k_pair_new_dt(int n_pairs, const int32_t* __restrict__ pairs, const double* __restrict__ max_time,
                              const int32_t* __restrict__ off, const double* __restrict__ rec,
                              const double* __restrict__ pfut, const double* __restrict__ ii,
                              double* __restrict__ new_dt, int32_t* __restrict__ has) {
    const int p = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (p >= n_pairs) return;  // uniform per warp
    const int a = pairs[2 * p], b = pairs[2 * p + 1];
    const int c0 = off[p], c1 = off[p + 1];
    if (c1 <= c0) {
        if (lane == 0) {
            has[p] = 0;
            new_dt[p] = 0.0;
        }
        return;
    }
    const State fa = load_state(pfut + 28 * (size_t)p), fb = load_state(pfut + 28 * (size_t)p + 14);
    const double mt = max_time[p];
    double Ia[9], Ib[9];
    world_inv_inertia(fa.q, ii + 9 * (size_t)a, Ia);
    world_inv_inertia(fb.q, ii + 9 * (size_t)b, Ib);
    double best = 1.0;
    int best_i = -1;  // the running minimum's start value comes first
    for (int c = c0 + lane; c < c1; c += 32) {
        const double sc = contact_step_scale(rec + 14 * (size_t)c, fa, Ia, fb, Ib, mt);
        if (sc < best) {
            best = sc;
            best_i = c;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_down_sync(0xffffffffu, best, o);
        const int oi = __shfl_down_sync(0xffffffffu, best_i, o);
        if (ob < best || (ob == best && oi < best_i)) {
            best = ob;
            best_i = oi;
        }
    }
    if (lane == 0) {
        has[p] = 1;
        new_dt[p] = mt * best;
    }
}

// Leftmost minimum of (value, index) over a block (all threads call it; the
// result is returned to every thread).  red holds 2 * 32 words.
__device__ void block_lmin(double& v, int& i, double* red_v, int* red_i) {
    for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_down_sync(0xffffffffu, v, o);
        const int oi = __shfl_down_sync(0xffffffffu, i, o);
        if (ov < v || (ov == v && oi < i)) {
            v = ov;
            i = oi;
        }
    }
    const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
        red_v[w] = v;
        red_i[w] = i;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < nw; k++)
            if (red_v[k] < v || (red_v[k] == v && red_i[k] < i)) {
                v = red_v[k];
                i = red_i[k];
            }
        red_v[0] = v;
        red_i[0] = i;
    }
    __syncthreads();
    v = red_v[0];
    i = red_i[0];
}

constexpr int kStepsBlock = 256;
constexpr int kStepsChunk = 1024;  // interactions staged per pass

// The reference's order-dependent propagation over a cluster's interactions
// (separate_clusters.cpp:555-598), one block per cluster.  The moving bodies'
// steps live in shared memory (loc maps a moving body to its slot).  Each
// chunk of interactions is first staged by all threads as (slot a, slot b,
// new step, step of the static side), then thread 0 walks the chunk in order
// touching shared memory only.  The final running minimum is a leftmost-
// minimum reduction when every value is non-negative (the fold is then
// associative); otherwise thread 0 repeats the reference's fold.
__global__ void __launch_bounds__(kStepsBlock)
    k_cluster_steps(int n_clusters, const int32_t* __restrict__ cl_pair_off, const int32_t* __restrict__ cl_part_off,
                    const int32_t* __restrict__ cl_parts, const int32_t* __restrict__ pairs,
                    const double* __restrict__ new_dt, const int32_t* __restrict__ has,
                    const uint8_t* __restrict__ is_static, const double* __restrict__ last_dt,
                    int32_t* __restrict__ loc, double opt_dt, double* __restrict__ out, double* __restrict__ gstep,
                    int n_step_slots, int chunk) {
    extern __shared__ __align__(16) double s_dyn[];
    __shared__ double red_v[32];
    __shared__ int red_i[32];
    const int c = blockIdx.x;
    if (c >= n_clusters) return;
    const int p0 = cl_part_off[c], p1 = cl_part_off[c + 1];
    double* s_step = gstep ? gstep + p0 : s_dyn;  // global scratch for clusters too large for shared memory
    double2* r_val = reinterpret_cast<double2*>(s_dyn + n_step_slots);
    int2* r_slot = reinterpret_cast<int2*>(r_val + chunk);
    for (int i = p0 + threadIdx.x; i < p1; i += blockDim.x) {
        const int g = cl_parts[i];
        s_step[i - p0] = last_dt[g];
        if (!is_static[g]) loc[g] = i - p0;
    }
    __syncthreads();
    const int q0 = cl_pair_off[c], q1 = cl_pair_off[c + 1];
    for (int base = q0; base < q1; base += chunk) {
        const int n = min(chunk, q1 - base);
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            const int i = base + j;
            int sa = -1, sb = -1;
            double nd = 0.0, sv = 0.0;
            if (has[i]) {
                const int a = pairs[2 * i], b = pairs[2 * i + 1];
                const bool as = is_static[a], bs = is_static[b];
                if (!(as && bs)) {  // two static sides write nothing
                    sa = as ? -1 : loc[a];
                    sb = bs ? -1 : loc[b];
                    nd = new_dt[i];
                    sv = as ? last_dt[a] : (bs ? last_dt[b] : 0.0);
                }
            }
            r_slot[j] = make_int2(sa, sb);
            r_val[j] = make_double2(nd, sv);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int j = 0; j < n; j++) {
                const int2 sl = r_slot[j];
                if ((sl.x & sl.y) < 0) continue;  // no contact, or both sides static
                const double2 v = r_val[j];
                const double va = sl.x >= 0 ? s_step[sl.x] : v.y;
                const double vb = sl.y >= 0 ? s_step[sl.y] : v.y;
                const double use = dmin_fast(v.x, dmin_fast(va, vb));
                if (sl.x >= 0) s_step[sl.x] = use;
                if (sl.y >= 0) s_step[sl.y] = use;
            }
        }
        __syncthreads();
    }
    auto step_of = [&](int g) { return is_static[g] ? last_dt[g] : s_step[loc[g]]; };
    // the first interaction with a moving side contributes the step of its
    // first body, every later one the step of its moving (or first) body
    double fv = 0.0;
    int first = 0x7fffffff;
    for (int i = q0 + threadIdx.x; i < q1; i += blockDim.x)
        if (!(is_static[pairs[2 * i]] && is_static[pairs[2 * i + 1]])) {
            first = i;
            break;
        }
    block_lmin(fv, first, red_v, red_i);
    double best = __longlong_as_double(0x7ff0000000000000LL);
    int bi = 0x7fffffff;
    bool irregular = false;
    for (int i = q0 + threadIdx.x; i < q1; i += blockDim.x) {
        const int a = pairs[2 * i], b = pairs[2 * i + 1];
        const bool as = is_static[a], bs = is_static[b];
        if (as && bs) continue;
        const double v = step_of(i == first || !as ? a : b);
        if (!(v >= 0.0)) irregular = true;
        if (v < best) {
            best = v;
            bi = i;
        }
    }
    irregular = __syncthreads_or(irregular);
    block_lmin(best, bi, red_v, red_i);
    if (threadIdx.x != 0) return;
    double cs = -1.0;
    if (first == 0x7fffffff) {
        cs = last_dt[cl_parts[p0]];
    } else if (!irregular) {
        cs = best;
    } else {
        for (int i = q0; i < q1; i++) {
            const int a = pairs[2 * i], b = pairs[2 * i + 1];
            int id;
            if (!is_static[a] && !is_static[b])
                id = a;
            else if (is_static[a] && is_static[b])
                continue;
            else if (is_static[a])
                id = b;
            else
                id = a;
            cs = cs < 0.0 ? step_of(a) : dmin_fast(cs, step_of(id));
        }
        if (cs < 0.0) cs = last_dt[cl_parts[p0]];
    }
    out[c] = dmax(1e-3, dmin(cs, opt_dt));
}

__global__ void k_max_time(int n, const int32_t* __restrict__ pairs, const double* __restrict__ last_dt,
                           double* __restrict__ mt) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) mt[p] = dmin(last_dt[pairs[2 * p]], last_dt[pairs[2 * p + 1]]);
}


#define SLAUNCH(kern, n, ...)                                          \
    do {                                                               \
        kern<<<nblocks(n), kBlock, 0, ctx->stream>>>(__VA_ARGS__);     \
        ctx->eng.launches++;                                           \
    } while (0)

#define RC(x)                          \
    do {                               \
        if (int rc_ = (x)) return rc_; \
    } while (0)

// Outer step start (broad_phase_embree_cluster.cpp:126-132): every body's
// last_dt doubles (capped at the option step) and its future is projected.
__global__ void k_outer_project(int n, double opt_dt, const double* __restrict__ cur, const double* __restrict__ ii,
                                double* __restrict__ last_dt, double* __restrict__ fut) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double l = last_dt[i] * 2.0;
    l = dmin(l, opt_dt);
    last_dt[i] = l;
    store_state(fut + 14 * (size_t)i, extrapolate(load_state(cur + 14 * (size_t)i), l, ii + 9 * (size_t)i));
}

// PDEExplicit::step preamble (PDE_explicit.cpp:49-63) for the moving bodies of
// each cluster: last_dt = step, roll back to the cluster's minimum current
// time, project the future.  err[k] = 1 where the reference would throw.
__global__ void k_pde_prepare(int n_clusters, const int32_t* __restrict__ part_off, const int32_t* __restrict__ parts,
                              const double* __restrict__ step, const double* __restrict__ t_min,
                              const uint8_t* __restrict__ is_static, const double* __restrict__ ii,
                              const double* __restrict__ last, double* __restrict__ cur, double* __restrict__ fut,
                              double* __restrict__ last_dt, int32_t* __restrict__ err) {
    const int k = blockIdx.x;
    if (k >= n_clusters) return;
    for (int i = part_off[k] + threadIdx.x; i < part_off[k + 1]; i += blockDim.x) {
        const int g = parts[i];
        if (is_static[g]) continue;
        last_dt[g] = step[k];
        State r;
        if (!interpolate(load_state(cur + 14 * (size_t)g), load_state(last + 14 * (size_t)g), t_min[k], r)) {
            err[k] = 1;
            continue;
        }
        store_state(cur + 14 * (size_t)g, r);
        store_state(fut + 14 * (size_t)g, extrapolate(r, step[k], ii + 9 * (size_t)g));
    }
}

// PDEExplicit::step after a successful solve (PDE_explicit.cpp:109-139):
// sleep bookkeeping and the state shift.  One block per cluster; the sleep
// counters are per body, the cluster's will_sleep is an AND over them.
__global__ void k_pde_finish(int n_clusters, const int32_t* __restrict__ part_off, const int32_t* __restrict__ parts,
                             const double* __restrict__ step, const int32_t* __restrict__ status,
                             const uint8_t* __restrict__ is_static, const double* __restrict__ ii,
                             double* __restrict__ last, double* __restrict__ cur, double* __restrict__ fut,
                             int32_t* __restrict__ sleep_steps, uint8_t* __restrict__ sleeping,
                             int32_t* __restrict__ will_sleep_out) {
    const int k = blockIdx.x;
    if (k >= n_clusters || status[k] != 0) return;
    bool awake = false;
    for (int i = part_off[k] + threadIdx.x; i < part_off[k + 1]; i += blockDim.x) {
        const int g = parts[i];
        if (is_static[g]) continue;
        const State L = load_state(last + 14 * (size_t)g), Cu = load_state(cur + 14 * (size_t)g),
                    F = load_state(fut + 14 * (size_t)g);
        auto stationary = [](const State& s) { return norm(s.v) < 1e-4 && norm(s.L) < 1e-4; };
        bool can = stationary(L) && stationary(Cu) && stationary(F);
        can = can && L.time < Cu.time && Cu.time < F.time;
        const int ss = can ? sleep_steps[g] + 1 : 0;
        sleep_steps[g] = ss;
        if (ss < 20) awake = true;
        store_state(last + 14 * (size_t)g, Cu);
        store_state(cur + 14 * (size_t)g, F);
        store_state(fut + 14 * (size_t)g, extrapolate(F, step[k], ii + 9 * (size_t)g));
    }
    const bool will_sleep = __syncthreads_or(awake ? 1 : 0) == 0;
    for (int i = part_off[k] + threadIdx.x; i < part_off[k + 1]; i += blockDim.x)
        if (!is_static[parts[i]]) sleeping[parts[i]] = will_sleep ? 1 : 0;
    if (threadIdx.x == 0) will_sleep_out[k] = will_sleep ? 1 : 0;
}

// separateCollisionClusters' rollback (separate_clusters.cpp:445-456): every
// moving body's current state is interpolated back to its cluster's minimum
// current time (t_body[g] < 0 leaves the body alone).
__global__ void k_rollback(int n, const double* __restrict__ t_body, const uint8_t* __restrict__ is_static,
                           const double* __restrict__ last, double* __restrict__ cur, int32_t* __restrict__ err) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n || is_static[g] || !(t_body[g] >= 0.0)) return;
    State r;
    if (!interpolate(load_state(cur + 14 * (size_t)g), load_state(last + 14 * (size_t)g), t_body[g], r)) {
        atomicExch(err, 1);
        return;
    }
    store_state(cur + 14 * (size_t)g, r);
}

// PDEStrategy::stepSleeping with apply (PDE_strategy.cpp:11-15) for the
// moving bodies of sleeping clusters: the clock advances, the future is the
// current state.
__global__ void k_sleep_apply(int n_clusters, const int32_t* __restrict__ part_off, const int32_t* __restrict__ parts,
                              const double* __restrict__ step, const uint8_t* __restrict__ is_static,
                              double* __restrict__ cur, double* __restrict__ fut) {
    const int k = blockIdx.x;
    if (k >= n_clusters) return;
    for (int i = part_off[k] + threadIdx.x; i < part_off[k + 1]; i += blockDim.x) {
        const int g = parts[i];
        if (is_static[g]) continue;
        cur[14 * (size_t)g] = cur[14 * (size_t)g] + step[k];
        for (int q = 0; q < 14; q++) fut[14 * (size_t)g + q] = cur[14 * (size_t)g + q];
    }
}

// The bookkeeping of stepRecursive (broad_phase_embree_cluster.cpp:16-123)
// between its PDE steps, as per-cluster op lists run in order by one block
// per cluster.  frame_start[f] holds a frame's start_step; stash + f's offset
// the moving bodies' current states saved after the frame's first half.
__global__ void k_cluster_ops(int n_clusters, const int32_t* __restrict__ cl_idx, const int32_t* __restrict__ op_off,
                              const int4* __restrict__ ops, const int32_t* __restrict__ part_off,
                              const int32_t* __restrict__ parts, const uint8_t* __restrict__ is_static,
                              const double* __restrict__ ii, double* __restrict__ cl_step,
                              double* __restrict__ cl_tmin, double* __restrict__ frame_start,
                              double* __restrict__ stash, double* __restrict__ last, double* __restrict__ cur,
                              double* __restrict__ fut, double* __restrict__ last_dt, int32_t* __restrict__ err) {
    const int b = blockIdx.x;
    if (b >= n_clusters) return;
    const int k = cl_idx[b];
    const int p0 = part_off[k], p1 = part_off[k + 1];
    const int tid = threadIdx.x, nt = blockDim.x;
    __shared__ double s_val;
    for (int o = op_off[b]; o < op_off[b + 1]; o++) {
        const int4 op = ops[o];  // (code, frame slot, stash offset in states, -)
        double* st = stash + 14 * (size_t)op.z;
        switch (op.x) {
            case D2G_OP_ENTER:
                if (tid == 0) frame_start[op.y] = cl_step[k];
                break;
            case D2G_OP_SPLIT:  // :42-65 after a failed step: roll back to the midpoint
                if (tid == 0) {
                    double new_min = 0.0;
                    for (int i = p0; i < p1; i++) {
                        const int g = parts[i];
                        if (is_static[g]) continue;
                        new_min = dmax(new_min, (last[14 * (size_t)g] + cur[14 * (size_t)g]) / 2.0);
                    }
                    s_val = new_min;
                    cl_tmin[k] = new_min;
                }
                __syncthreads();
                for (int i = p0 + tid; i < p1; i += nt) {
                    const int g = parts[i];
                    if (is_static[g]) continue;
                    const State c = load_state(cur + 14 * (size_t)g);
                    store_state(fut + 14 * (size_t)g, c);
                    State r;
                    if (!interpolate(c, load_state(last + 14 * (size_t)g), s_val, r)) {
                        atomicExch(err, 1);
                        continue;
                    }
                    store_state(cur + 14 * (size_t)g, r);
                }
                __syncthreads();
                if (tid == 0) {
                    double step_size = 0.0;
                    for (int i = p0; i < p1; i++)
                        if (!is_static[parts[i]]) step_size = fut[14 * (size_t)parts[i]] - s_val;
                    cl_step[k] = step_size;
                }
                break;
            case D2G_OP_SAVE: {  // :67-83 keep the first half's end, start the second half
                const double half = frame_start[op.y] / 2.0;
                int j = 0;
                for (int i = p0; i < p1; i++) {
                    const int g = parts[i];
                    if (is_static[g]) continue;
                    if ((j % nt) == tid)
                        for (int q = 0; q < 14; q++) st[14 * (size_t)j + q] = cur[14 * (size_t)g + q];
                    j++;
                }
                for (int i = p0 + tid; i < p1; i += nt) {
                    const int g = parts[i];
                    if (is_static[g]) continue;
                    store_state(fut + 14 * (size_t)g, extrapolate(load_state(cur + 14 * (size_t)g), half,
                                                                   ii + 9 * (size_t)g));
                }
                if (tid == 0) {
                    cl_step[k] = half;
                    for (int i = p0; i < p1; i++)
                        if (!is_static[parts[i]]) cl_tmin[k] = cur[14 * (size_t)parts[i]];
                }
                break;
            }
            case D2G_OP_MID:  // :87-91
                if (tid == 0)
                    for (int i = p0; i < p1; i++)
                        if (!is_static[parts[i]]) cl_tmin[k] = cur[14 * (size_t)parts[i]];
                break;
            case D2G_OP_RESTORE: {  // :95-107
                const double half = frame_start[op.y] / 2.0;
                int j = 0;
                for (int i = p0; i < p1; i++) {
                    const int g = parts[i];
                    if (is_static[g]) continue;
                    if ((j % nt) == tid) {
                        for (int q = 0; q < 14; q++) last[14 * (size_t)g + q] = st[14 * (size_t)j + q];
                        last_dt[g] = dmin(last_dt[g], half);
                    }
                    j++;
                }
                break;
            }
            case D2G_OP_EXIT:  // :122
                if (tid == 0) cl_step[k] = frame_start[op.y];
                break;
            default:
                break;
        }
        __syncthreads();
    }
}

// Per-contact warm value, body-pair contact count and pair index from the
// per-pair arrays of the filtered contacts.
__global__ void k_expand_contacts(int n_pairs, const int32_t* __restrict__ off, const double* __restrict__ pwarm,
                                  const int32_t* __restrict__ pcnt, double* __restrict__ warm,
                                  int32_t* __restrict__ cnt, int32_t* __restrict__ pair) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_pairs) return;
    for (int c = off[p]; c < off[p + 1]; c++) {
        warm[c] = pwarm[p];
        cnt[c] = pcnt[p];
        pair[c] = p;
    }
}

__global__ void k_gather_f64(int n, const int32_t* __restrict__ idx, const double* __restrict__ src,
                             double* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[idx[i]];
}

// con_off[b] = flt_off[pair_off[b]] for b in [0, n].
__global__ void k_con_off(int n, const int32_t* __restrict__ pair_off, const int32_t* __restrict__ flt_off,
                          int32_t* __restrict__ con_off) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i <= n) con_off[i] = flt_off[pair_off[i]];
}

// The static bodies' current states, last_dt and sleeping flags, compacted.
__global__ void k_gather_static(int n, const int32_t* __restrict__ idx, const double* __restrict__ cur,
                                const double* __restrict__ last_dt, const uint8_t* __restrict__ sleeping,
                                double* __restrict__ rec, uint8_t* __restrict__ sl) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int g = idx[k];
    for (int q = 0; q < 14; q++) rec[15 * (size_t)k + q] = cur[14 * (size_t)g + q];
    rec[15 * (size_t)k + 14] = last_dt[g];
    sl[k] = sleeping[g];
}

}  // namespace

int run_gather_static(d2g_ctx* ctx, int n, const int32_t* d_idx, double* d_rec, uint8_t* d_sleep) {
    if (n > 0) SLAUNCH(k_gather_static, n, n, d_idx, ctx->cur.p, ctx->last_dt.p, ctx->sleeping.p, d_rec, d_sleep);
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

int run_outer_project(d2g_ctx* ctx, double opt_dt) {
    SLAUNCH(k_outer_project, ctx->n_bodies, ctx->n_bodies, opt_dt, ctx->cur.p, ctx->inv_inertia.p, ctx->last_dt.p,
            ctx->fut.p);
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

int run_pde_prepare(d2g_ctx* ctx, int n_clusters, const int32_t* d_part_off, const int32_t* d_parts,
                    const double* d_step, const double* d_tmin, int32_t* d_err) {
    if (n_clusters > 0) {
        k_pde_prepare<<<n_clusters, 64, 0, ctx->stream>>>(n_clusters, d_part_off, d_parts, d_step, d_tmin,
                                                           ctx->is_static.p, ctx->inv_inertia.p, ctx->last.p,
                                                           ctx->cur.p, ctx->fut.p, ctx->last_dt.p, d_err);
        ctx->eng.launches++;
    }
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

int run_pde_finish(d2g_ctx* ctx, int n_clusters, const int32_t* d_part_off, const int32_t* d_parts,
                   const double* d_step, const int32_t* d_status, int32_t* d_will_sleep) {
    if (n_clusters > 0) {
        k_pde_finish<<<n_clusters, 64, 0, ctx->stream>>>(n_clusters, d_part_off, d_parts, d_step, d_status,
                                                          ctx->is_static.p, ctx->inv_inertia.p, ctx->last.p,
                                                          ctx->cur.p, ctx->fut.p, ctx->sleep_steps.p,
                                                          ctx->sleeping.p, d_will_sleep);
        ctx->eng.launches++;
    }
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

int run_rollback(d2g_ctx* ctx, const double* d_t_body, int32_t* d_err) {
    if (ctx->n_bodies > 0)
        SLAUNCH(k_rollback, ctx->n_bodies, ctx->n_bodies, d_t_body, ctx->is_static.p, ctx->last.p, ctx->cur.p, d_err);
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

int run_sleep_apply(d2g_ctx* ctx, int n_clusters, const int32_t* d_part_off, const int32_t* d_parts,
                    const double* d_step) {
    if (n_clusters > 0) {
        k_sleep_apply<<<n_clusters, 64, 0, ctx->stream>>>(n_clusters, d_part_off, d_parts, d_step, ctx->is_static.p,
                                                           ctx->cur.p, ctx->fut.p);
        ctx->eng.launches++;
    }
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

int run_cluster_ops(d2g_ctx* ctx, int n_active, const int32_t* d_cl_idx, const int32_t* d_op_off, const int4* d_ops,
                    const int32_t* d_part_off, const int32_t* d_parts, double* d_cl_step, double* d_cl_tmin,
                    double* d_frame_start, double* d_stash, int32_t* d_err) {
    if (n_active > 0) {
        k_cluster_ops<<<n_active, 64, 0, ctx->stream>>>(n_active, d_cl_idx, d_op_off, d_ops, d_part_off, d_parts,
                                                         ctx->is_static.p, ctx->inv_inertia.p, d_cl_step, d_cl_tmin,
                                                         d_frame_start, d_stash, ctx->last.p, ctx->cur.p, ctx->fut.p,
                                                         ctx->last_dt.p, d_err);
        ctx->eng.launches++;
    }
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

int run_expand_contacts(d2g_ctx* ctx, int n_pairs, const int32_t* d_off, const double* d_pwarm,
                        const int32_t* d_pcnt, double* d_warm, int32_t* d_cnt, int32_t* d_pair) {
    if (n_pairs > 0) SLAUNCH(k_expand_contacts, n_pairs, n_pairs, d_off, d_pwarm, d_pcnt, d_warm, d_cnt, d_pair);
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

int run_gather_f64(d2g_ctx* ctx, int n, const int32_t* d_idx, const double* d_src, double* d_dst) {
    if (n > 0) SLAUNCH(k_gather_f64, n, n, d_idx, d_src, d_dst);
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

int run_con_off(d2g_ctx* ctx, int n, const int32_t* d_pair_off, const int32_t* d_flt_off, int32_t* d_con_off) {
    SLAUNCH(k_con_off, n + 1, n, d_pair_off, d_flt_off, d_con_off);
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

// Device-side driver: pairs/cluster arrays already in HBM.
int run_select_steps(d2g_ctx* ctx, const int32_t* d_pairs, int n_pairs, const int32_t* d_cl_pair_off,
                     const int32_t* d_cl_part_off, const int32_t* d_cl_parts, int n_clusters, int n_parts,
                     int max_cluster_parts, double opt_dt, double* d_out, int64_t* counters, int* n_ccd_contacts) {
    Engine& E = ctx->eng;
    RC(E.st_mt.ensure(n_pairs + 1));
    RC(E.st_new_dt.ensure(n_pairs + 1));
    RC(E.st_has.ensure(n_pairs + 1));
    if (n_pairs > 0) SLAUNCH(k_max_time, n_pairs, n_pairs, d_pairs, ctx->last_dt.p, E.st_mt.p);
    // The CCD's records only feed each pair's new step: they are consumed
    // chunk by chunk (sorted per chunk) and dropped.
    struct Use {
        const int32_t* pairs;
    } use{d_pairs};
    CcdSink sink;
    sink.user = &use;
    sink.consume = [](d2g_ctx* c, void* u, int p0, int p1) -> int {
        Engine& En = c->eng;
        const int32_t* pr = static_cast<Use*>(u)->pairs;
        const int np = p1 - p0;
        if (np > 0) {
            k_pair_new_dt<<<nblocks(32LL * np), kBlock, 0, c->stream>>>(
                np, pr + 2 * (size_t)p0, En.st_mt.p + p0, En.out_off.p, En.rec_sorted.p, En.pfut.p + 28 * (size_t)p0,
                c->inv_inertia.p, En.st_new_dt.p + p0, En.st_has.p + p0);
            En.launches++;
        }
        D2G_CUDA(cudaGetLastError());
        return D2G_OK;
    };
    int n_rec = 0;
    RC(run_ccd(ctx, d_pairs, E.st_mt.p, n_pairs, &n_rec, counters, &sink));
    if (n_ccd_contacts) *n_ccd_contacts = n_rec;
    if (n_clusters > 0) {
        RC(E.st_loc.ensure(ctx->n_bodies + 1));
        constexpr int kMaxSmemParts = 24 * 1024;  // 192 KB of steps
        // staged interactions per pass: enough for a cluster's interactions
        // (about twice its members), at most kStepsChunk
        int chunk = 32;
        while (chunk < kStepsChunk && chunk < 2 * max_cluster_parts) chunk *= 2;
        double* gstep = nullptr;
        int n_slots = (max_cluster_parts + 1) & ~1;  // keeps the double2 records 16-byte aligned
        if (max_cluster_parts > kMaxSmemParts) {
            RC(E.st_step.ensure((size_t)n_parts + 1));
            gstep = E.st_step.p;
            n_slots = 0;
        }
        const size_t smem = (size_t)n_slots * sizeof(double) + (size_t)chunk * (sizeof(double2) + sizeof(int2));
        if (smem > 48 * 1024)
            D2G_CUDA(cudaFuncSetAttribute(k_cluster_steps, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_cluster_steps<<<n_clusters, kStepsBlock, smem, ctx->stream>>>(
            n_clusters, d_cl_pair_off, d_cl_part_off, d_cl_parts, d_pairs, E.st_new_dt.p, E.st_has.p,
            ctx->is_static.p, ctx->last_dt.p, E.st_loc.p, opt_dt, d_out, gstep, n_slots, chunk);
        ctx->eng.launches++;
    }
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

}  // namespace d2g
