// The adaptive cluster stepper with every cluster's work batched on the GPU.
//
// Restates BroadPhaseEmbreeCluster::step and stepRecursive
// (strategies/broad_phase/broad_phase_embree_cluster.cpp:16-257),
// separateCollisionClusters (collision_detection/separate_clusters.cpp:
// 355-459), PDEExplicit::step (strategies/PDE/PDE_explicit.cpp:30-142) and
// PDEStrategy::stepSleeping (PDE_strategy.cpp:11-15).
//
// The reference steps clusters one after another.  Clusters share no moving
// body, and the warm-start store is keyed by body pair, so their steps are
// independent; here every cluster advances in the same launches:
//   * the host runs the broad phase over the states copied back once per
//     outer step, labels the clusters and schedules;
//   * one CCD launch sequence selects every cluster's step
//     (d2g_step.cu run_select_steps);
//   * stepRecursive runs as one state machine per cluster on the host; each
//     round batches the PDE steps of all clusters that need one (narrow
//     phase, contact filter, sequential-impulse solve, state shift) and the
//     bookkeeping between steps runs as per-cluster op lists on the device.
// Static bodies are the one state clusters share.  The reference's
// sequential order decides three of their fields, reproduced here on the
// host: last_dt and sleeping come from the last PDE step (in cluster order)
// of a cluster holding the body, and the current time advances once per
// sleeping cluster holding it, in cluster order.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <utility>
#include <vector>

#include "d2g_geom.cuh"
#include "d2g_internal.hpp"

namespace d2g {

int run_gather_static(d2g_ctx* ctx, int n, const int32_t* d_idx, double* d_rec, uint8_t* d_sleep);
int run_gather_f64(d2g_ctx* ctx, int n, const int32_t* d_idx, const double* d_src, double* d_dst);
int run_con_off(d2g_ctx* ctx, int n, const int32_t* d_pair_off, const int32_t* d_flt_off, int32_t* d_con_off);
int run_expand_contacts(d2g_ctx* ctx, int n_pairs, const int32_t* d_off, const double* d_pwarm,
                        const int32_t* d_pcnt, double* d_warm, int32_t* d_cnt, int32_t* d_pair);

namespace {

#define RC(x)                          \
    do {                               \
        if (int rc_ = (x)) return rc_; \
    } while (0)

constexpr int kMaxDepth = 60;  // stepRecursive's depth guard (the reference has none)

template <class T>
struct Pinned {
    T* p = nullptr;
    size_t cap = 0;
    int ensure(size_t n) {
        if (n <= cap) return D2G_OK;
        if (p) cudaFreeHost(p);
        p = nullptr;
        const size_t c = n + n / 2 + 64;
        cudaError_t e = cudaMallocHost((void**)&p, c * sizeof(T));
        if (e != cudaSuccess) {
            cap = 0;
            set_error(std::string("cudaMallocHost: ") + cudaGetErrorString(e));
            return D2G_ERR_CUDA;
        }
        cap = c;
        return D2G_OK;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
};

// Packs host arrays into one pinned staging area and one device buffer with
// a single copy.  The staging area is rewritten only after the stream has
// been synchronised past the previous copy (the callers sync once per round).
template <class T>
struct Packer {
    Pinned<T> stage;
    DBuf<T> dev;
    std::vector<T> host;
    std::vector<size_t> offs;
    void clear() {
        host.clear();
        offs.clear();
    }
    int add(const T* v, size_t n) {
        offs.push_back(host.size());
        host.insert(host.end(), v, v + n);
        // keep each array 16-byte aligned on the device
        while ((host.size() * sizeof(T)) % 16) host.push_back(T());
        return (int)offs.size() - 1;
    }
    int add(const std::vector<T>& v) { return add(v.data(), v.size()); }
    int upload(cudaStream_t s) {
        const size_t n = host.size() + 1;
        RC(stage.ensure(n));
        RC(dev.ensure(n));
        if (!host.empty()) memcpy(stage.p, host.data(), host.size() * sizeof(T));
        D2G_CUDA(cudaMemcpyAsync(dev.p, stage.p, host.size() * sizeof(T), cudaMemcpyHostToDevice, s));
        return D2G_OK;
    }
    T* ptr(int id) { return dev.p + offs[id]; }
    void release() {
        stage.release();
        dev.release();
    }
};

struct HostCluster {
    std::vector<int32_t> parts;  // component members ascending, then static bodies by first interaction
    std::vector<int32_t> pairs;  // interactions (a, b), broad-phase order
    double mct = 0.0, step = 0.0;
    bool sleeping = true;
    int n_dyn = 0;
    int scene = 0;
};

struct Frame {
    int depth = 0, phase = 0;
};

struct Machine {
    std::vector<Frame> stack;
    std::vector<int4> ops;
    bool need_pde = false;
    double last_step = 0.0;  // step of its latest PDE step
    int last_sleep = 0;      // will_sleep of its latest successful PDE step
};

}  // namespace

struct WorldState {
    std::vector<float> local_aabb;
    float opt_dt = 0.01f;
    double gravity_z = -9.8;
    std::map<std::pair<int, int>, double> warm;
    int64_t stats[13] = {0};
    // static bodies: indices, slot of a body in that list, their records
    std::vector<int32_t> static_ids, slot_of;
    int n_dyn_total = 0;
    DBuf<float> d_aabb;
    DBuf<int32_t> d_static;
    DBuf<double> d_st_rec;
    DBuf<uint8_t> d_st_sleep;
    Pinned<int32_t> h_cl;   // cluster CSR and flags copied back each step
    Pinned<double> h_cld;   // cluster times, steps and the static records
    Pinned<uint8_t> h_sleeping;  // static bodies' sleeping flags being written
    Pinned<double> h_rd;
    Pinned<int32_t> h_ri;
    Packer<int32_t> pk_round, pk_batch, pk_cl;
    Packer<double> pk_round_d, pk_warm;
    Packer<int4> pk_ops;
    DBuf<double> cl_step, cl_tmin, frame_start, stash, step_a, tmin_a, con_warm, pair_warm, con_imp, sel_out;
    DBuf<int32_t> err, status, iters, will_sleep, con_cnt, con_pair, con_off, con_ab;
    size_t stash_used = 0;
    // host wall time per phase (instrumentation): see d2g_world_timing
    double phase_ms[D2G_WORLD_PHASES] = {0};
    std::chrono::steady_clock::time_point t_mark;
    void mark(int phase) {
        const auto now = std::chrono::steady_clock::now();
        if (phase >= 0) phase_ms[phase] += std::chrono::duration<double, std::milli>(now - t_mark).count();
        t_mark = now;
    }
};

void world_free(WorldState* w) {
    if (!w) return;
    w->h_cl.release();
    w->h_cld.release();
    w->h_sleeping.release();
    w->d_aabb.release();
    w->d_static.release();
    w->d_st_rec.release();
    w->d_st_sleep.release();
    w->h_rd.release();
    w->h_ri.release();
    w->pk_round.release();
    w->pk_batch.release();
    w->pk_cl.release();
    w->pk_round_d.release();
    w->pk_warm.release();
    w->pk_ops.release();
    for (DBuf<double>* b : {&w->cl_step, &w->cl_tmin, &w->frame_start, &w->stash, &w->step_a, &w->tmin_a,
                            &w->con_warm, &w->pair_warm, &w->con_imp, &w->sel_out})
        b->release();
    for (DBuf<int32_t>* b : {&w->err, &w->status, &w->iters, &w->will_sleep, &w->con_cnt, &w->con_pair,
                             &w->con_off, &w->con_ab})
        b->release();
    delete w;
}

namespace {

// Reads the device error flag (after the stream has been synchronised).
int check_err(d2g_ctx* c, WorldState& W, const char* where) {
    D2G_CUDA(cudaMemcpyAsync(W.h_ri.p, W.err.p, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
    D2G_CUDA(cudaStreamSynchronize(c->stream));
    prof_mark_collect(c);
    if (W.h_ri.p[0]) {
        set_error(std::string("invalid state interpolation in ") + where + " (the reference throws here)");
        return D2G_ERR_STATE;
    }
    return D2G_OK;
}

// One batched PDEExplicit::step over the clusters R[a] for a in `act`.
int pde_round(d2g_ctx* c, WorldState& W, const std::vector<HostCluster>& cls, const std::vector<int>& R,
              const std::vector<int>& act, std::vector<Machine>& M, std::vector<int>& ok_out) {
    cudaStream_t s = c->stream;
    Engine& E = c->eng;
    const int nA = (int)act.size();
    std::vector<int32_t> a_idx(nA), part_off(nA + 1, 0), parts, pairs, pair_off(nA + 1, 0);
    for (int b = 0; b < nA; b++) {
        const HostCluster& h = cls[R[act[b]]];
        a_idx[b] = act[b];
        parts.insert(parts.end(), h.parts.begin(), h.parts.end());
        pairs.insert(pairs.end(), h.pairs.begin(), h.pairs.end());
        part_off[b + 1] = (int32_t)parts.size();
        pair_off[b + 1] = (int32_t)(pairs.size() / 2);
    }
    const int n_pairs = (int)(pairs.size() / 2);
    W.pk_batch.clear();
    const int i_idx = W.pk_batch.add(a_idx), i_poff = W.pk_batch.add(part_off), i_parts = W.pk_batch.add(parts),
              i_pairs = W.pk_batch.add(pairs), i_pairoff = W.pk_batch.add(pair_off);
    RC(W.pk_batch.upload(s));
    RC(W.step_a.ensure(nA + 1));
    RC(W.tmin_a.ensure(nA + 1));
    RC(run_gather_f64(c, nA, W.pk_batch.ptr(i_idx), W.cl_step.p, W.step_a.p));
    RC(run_gather_f64(c, nA, W.pk_batch.ptr(i_idx), W.cl_tmin.p, W.tmin_a.p));
    RC(run_pde_prepare(c, nA, W.pk_batch.ptr(i_poff), W.pk_batch.ptr(i_parts), W.step_a.p, W.tmin_a.p, W.err.p));
    int n_rec = 0;
    int64_t cnt[4] = {0, 0, 0, 0};
    RC(run_narrowphase(c, W.pk_batch.ptr(i_pairs), n_pairs, &n_rec, cnt));
    W.mark(5);
    int n_kept = 0;
    RC(run_filter(c, E.out_off.p, E.rec_sorted.p, n_pairs, n_rec, 0.0, &n_kept));
    // warm-start values per interaction (sequential_impulses_warm_start.cpp:11-26)
    std::vector<double> pwarm(n_pairs + 1, std::numeric_limits<double>::quiet_NaN());
    for (int p = 0; p < n_pairs; p++) {
        auto f = W.warm.find(std::make_pair(pairs[2 * p], pairs[2 * p + 1]));
        if (f != W.warm.end()) pwarm[p] = f->second;
    }
    W.pk_warm.clear();
    const int i_w = W.pk_warm.add(pwarm);
    RC(W.pk_warm.upload(s));
    RC(W.con_warm.ensure(n_kept + 1));
    RC(W.con_cnt.ensure(n_kept + 1));
    RC(W.con_pair.ensure(n_kept + 1));
    RC(W.con_off.ensure(nA + 1));
    RC(W.con_imp.ensure(n_kept + 1));
    RC(W.con_ab.ensure(2 * (size_t)n_kept + 2));
    RC(W.pair_warm.ensure(n_pairs + 1));
    RC(W.status.ensure(nA + 1));
    RC(W.iters.ensure(2 * (size_t)nA + 2));
    RC(W.will_sleep.ensure(nA + 1));
    RC(run_expand_contacts(c, n_pairs, E.flt_off.p, W.pk_warm.ptr(i_w), E.flt_cnt.p, W.con_warm.p, W.con_cnt.p,
                           W.con_pair.p));
    W.mark(6);
    RC(run_con_off(c, nA, W.pk_batch.ptr(i_pairoff), E.flt_off.p, W.con_off.p));
    // the contact count of every cluster decides how it is solved (one block, or a grid)
    const size_t ni = (size_t)nA * 4 + n_pairs + 1;
    RC(W.h_ri.ensure(ni + nA + 8));
    int32_t* h_con_off = W.h_ri.p + ni + 4;
    D2G_CUDA(cudaMemcpyAsync(h_con_off, W.con_off.p, (nA + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    D2G_CUDA(cudaStreamSynchronize(s));
    RC(run_solve(c, nA, W.pk_batch.ptr(i_poff), W.pk_batch.ptr(i_parts), (int)parts.size(), W.con_off.p, n_kept,
                 E.flt.p, W.con_cnt.p, W.con_warm.p, W.step_a.p, W.gravity_z, W.status.p, W.iters.p, W.con_imp.p,
                 W.con_ab.p, W.con_pair.p, W.pair_warm.p, h_con_off, part_off.data()));
    RC(run_pde_finish(c, nA, W.pk_batch.ptr(i_poff), W.pk_batch.ptr(i_parts), W.step_a.p, W.status.p,
                      W.will_sleep.p));
    // results back: status, iterations, will_sleep, kept counts (int); step, pair warm (double)

    RC(W.h_rd.ensure((size_t)nA + n_pairs + 1));
    int32_t* hi = W.h_ri.p + 1;
    D2G_CUDA(cudaMemcpyAsync(hi, W.status.p, nA * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    D2G_CUDA(cudaMemcpyAsync(hi + nA, W.iters.p, 2 * nA * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    D2G_CUDA(cudaMemcpyAsync(hi + 3 * nA, W.will_sleep.p, nA * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    if (n_pairs > 0)
        D2G_CUDA(cudaMemcpyAsync(hi + 4 * nA, E.flt_cnt.p, n_pairs * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    D2G_CUDA(cudaMemcpyAsync(W.h_rd.p, W.step_a.p, nA * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (n_pairs > 0)
        D2G_CUDA(cudaMemcpyAsync(W.h_rd.p + nA, W.pair_warm.p, n_pairs * sizeof(double), cudaMemcpyDeviceToHost, s));
    RC(check_err(c, W, "PDEExplicit::step"));
    hi = W.h_ri.p + 1;
    // statistics (PDE_explicit.cpp:77-101)
    W.stats[2] += n_pairs;
    W.stats[3] += n_kept;
    W.stats[4] += nA;
    W.stats[11] += cnt[0];
    W.stats[12] += cnt[1];
    ok_out.assign(nA, 0);
    for (int b = 0; b < nA; b++)
        if (hi[b] == 3) {
            set_error("a grid barrier of the sequential-impulse solve gave up waiting");
            return D2G_SPIN_LIMIT;
        }
    for (int b = 0; b < nA; b++) {
        Machine& m = M[act[b]];
        m.last_step = W.h_rd.p[b];
        const bool ok = hi[b] == 0;
        ok_out[b] = ok ? 1 : 0;
        if (!ok) {
            W.stats[5]++;
            continue;
        }
        W.stats[6] += hi[nA + 2 * b];
        W.stats[7] += hi[nA + 2 * b + 1];
        m.last_sleep = hi[3 * nA + b];
        for (int p = pair_off[b]; p < pair_off[b + 1]; p++)
            if (hi[4 * nA + p] > 0) W.warm[std::make_pair(pairs[2 * p], pairs[2 * p + 1])] = W.h_rd.p[nA + p];
    }
    W.mark(7);
    return D2G_OK;
}

// stepRecursive as a state machine.  Frame slots: frame_start[depth * nR + r];
// stash of a frame: depth * total_dyn + dyn_base[r] (in states).
struct Recursion {
    int nR = 0, total_dyn = 0;
    std::vector<int> dyn_base;
    int slot(int r, int depth) const { return depth * nR + r; }
    int stash_off(int r, int depth) const { return depth * total_dyn + dyn_base[r]; }
};

int enter_frame(Machine& m, const Recursion& Rc, int r, int depth) {
    if (depth > kMaxDepth) {
        set_error("stepRecursive exceeded depth " + std::to_string(kMaxDepth));
        return D2G_ERR_STATE;
    }
    Frame f;
    f.depth = depth;
    f.phase = 0;
    m.stack.push_back(f);
    m.ops.push_back(make_int4(D2G_OP_ENTER, Rc.slot(r, depth), 0, 0));
    m.need_pde = true;
    return D2G_OK;
}

int ensure_stash(d2g_ctx* c, WorldState& W, const Recursion& Rc, int depth) {
    const size_t need = 14 * (size_t)(depth + 1) * Rc.total_dyn;
    if (need > W.stash_used) {
        RC(W.stash.ensure_keep(need, W.stash_used, c->stream));
        W.stash_used = need;
    }
    return D2G_OK;
}

// Advances cluster r after its PDE step (ok) until it needs another or ends.
int advance(d2g_ctx* c, WorldState& W, const Recursion& Rc, Machine& m, int r, bool ok) {
    m.need_pde = false;
    if (!ok) {  // :42-65 roll back to the midpoint and recurse
        const int d = m.stack.back().depth;
        m.ops.push_back(make_int4(D2G_OP_SPLIT, 0, 0, 0));
        return enter_frame(m, Rc, r, d + 1);
    }
    for (;;) {  // the frame on top has finished
        const Frame f = m.stack.back();
        m.ops.push_back(make_int4(D2G_OP_EXIT, Rc.slot(r, f.depth), 0, 0));
        m.stack.pop_back();
        if (m.stack.empty()) return D2G_OK;
        Frame& p = m.stack.back();
        p.phase++;
        if (p.phase == 1) {  // :67-85 second half, first part
            RC(ensure_stash(c, W, Rc, p.depth));
            m.ops.push_back(make_int4(D2G_OP_SAVE, Rc.slot(r, p.depth), Rc.stash_off(r, p.depth), 0));
            return enter_frame(m, Rc, r, p.depth + 1);
        }
        if (p.phase == 2) {  // :87-93 second half, second part
            m.ops.push_back(make_int4(D2G_OP_MID, Rc.slot(r, p.depth), 0, 0));
            return enter_frame(m, Rc, r, p.depth + 1);
        }
        // :95-107 restore the first half's end as the last state
        m.ops.push_back(make_int4(D2G_OP_RESTORE, Rc.slot(r, p.depth), Rc.stash_off(r, p.depth), 0));
    }
}

int flush_ops(d2g_ctx* c, WorldState& W, std::vector<Machine>& M, const int32_t* d_part_off,
              const int32_t* d_parts) {
    std::vector<int32_t> idx, off(1, 0);
    std::vector<int4> ops;
    for (int r = 0; r < (int)M.size(); r++) {
        if (M[r].ops.empty()) continue;
        idx.push_back(r);
        ops.insert(ops.end(), M[r].ops.begin(), M[r].ops.end());
        off.push_back((int32_t)ops.size());
        M[r].ops.clear();
    }
    if (idx.empty()) return D2G_OK;
    W.pk_cl.clear();
    const int i_idx = W.pk_cl.add(idx), i_off = W.pk_cl.add(off);
    RC(W.pk_cl.upload(c->stream));
    W.pk_ops.clear();
    const int i_ops = W.pk_ops.add(ops);
    RC(W.pk_ops.upload(c->stream));
    return run_cluster_ops(c, (int)idx.size(), W.pk_cl.ptr(i_idx), W.pk_cl.ptr(i_off), W.pk_ops.ptr(i_ops), d_part_off,
                           d_parts, W.cl_step.p, W.cl_tmin.p, W.frame_start.p, W.stash.p, W.err.p);
}

int world_step_once(d2g_ctx* c, WorldState& W) {
    const int n = c->n_bodies;
    cudaStream_t s = c->stream;
    const double opt_dt = (double)W.opt_dt;
    W.mark(-1);
    D2G_CUDA(cudaMemsetAsync(W.err.p, 0, sizeof(int32_t), s));
    // :126-132 every body: last_dt doubles (capped), future projected
    RC(run_outer_project(c, opt_dt));
    W.mark(0);
    // :134 broad phase and :136 cluster separation (with its rollback), on the device
    Engine& E = c->eng;
    int nb = 0;
    RC(run_broad_phase(c, W.d_aabb.p, &nb, W.err.p));
    W.mark(1);
    int nc = 0, n_parts = 0;
    RC(run_clusters(c, E.bp_pairs.p, nb, W.n_dyn_total, &nc, &n_parts, W.err.p));
    RC(run_cluster_rollback(c, W.err.p));
    // the clusters and the static bodies' records come back for the host schedule
    const int n_st = (int)W.static_ids.size();
    RC(W.h_cl.ensure(3 * (size_t)nc + n_parts + 2 * (size_t)nb + 8));
    RC(W.h_cld.ensure(2 * (size_t)nc + 15 * (size_t)n_st + 8));
    int32_t* h_part_off = W.h_cl.p;
    int32_t* h_pair_off = h_part_off + nc + 1;
    int32_t* h_ndyn = h_pair_off + nc + 1;
    int32_t* h_sleep = h_ndyn + nc;
    int32_t* h_parts = h_sleep + nc;
    int32_t* h_pairs = h_parts + n_parts;
    double* h_mct = W.h_cld.p;
    double* h_step = h_mct + nc;
    double* h_st = h_step + nc;  // static records: 14 (cur) + last_dt per static body
    D2G_CUDA(cudaMemcpyAsync(h_part_off, E.cl_part_off.p, (nc + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    D2G_CUDA(cudaMemcpyAsync(h_pair_off, E.cl_pair_off.p, (nc + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    if (nc > 0) {
        D2G_CUDA(cudaMemcpyAsync(h_ndyn, E.cl_n_dyn.p, nc * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        D2G_CUDA(cudaMemcpyAsync(h_sleep, E.cl_sleep.p, nc * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        D2G_CUDA(cudaMemcpyAsync(h_mct, E.cl_mct.p, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
        D2G_CUDA(cudaMemcpyAsync(h_step, E.cl_step.p, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
        D2G_CUDA(cudaMemcpyAsync(h_parts, E.cl_parts.p, n_parts * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    }
    if (nb > 0)
        D2G_CUDA(cudaMemcpyAsync(h_pairs, E.cl_pairs.p, 2 * (size_t)nb * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    if (n_st > 0) {
        RC(W.d_st_rec.ensure(15 * (size_t)n_st));
        RC(run_gather_static(c, n_st, W.d_static.p, W.d_st_rec.p, W.d_st_sleep.p));
        D2G_CUDA(cudaMemcpyAsync(h_st, W.d_st_rec.p, 15 * (size_t)n_st * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    RC(check_err(c, W, "the broad phase or separateCollisionClusters"));
    std::vector<HostCluster> cls(nc);
    for (int k = 0; k < nc; k++) {
        HostCluster& h = cls[k];
        h.parts.assign(h_parts + h_part_off[k], h_parts + h_part_off[k + 1]);
        h.pairs.assign(h_pairs + 2 * (size_t)h_pair_off[k], h_pairs + 2 * (size_t)h_pair_off[k + 1]);
        h.n_dyn = h_ndyn[k];
        h.mct = h_mct[k];
        h.step = h_step[k];
        h.sleeping = h_sleep[k] != 0;
    }
    W.mark(2);
    // :139-147 the earliest end of any cluster's step
    // (per scene: every scene is scheduled as its own world)
    const double inf = std::numeric_limits<double>::infinity();
    std::vector<double> min_final_s(c->n_scenes, inf), fine_s(c->n_scenes, inf);
    for (HostCluster& h : cls) h.scene = c->h_scene[h.parts[0]];
    for (const HostCluster& h : cls) min_final_s[h.scene] = dmin(min_final_s[h.scene], h.mct + h.step);
    // :149-170 time-step selection for the awake clusters that start in time
    std::vector<int> sel;
    for (int k = 0; k < nc; k++)
        if (!(cls[k].mct > min_final_s[cls[k].scene]) && !cls[k].sleeping) sel.push_back(k);
    if (!sel.empty()) {
        std::vector<int32_t> pairs, pair_off(1, 0), part_off(1, 0), parts;
        for (int k : sel) {
            pairs.insert(pairs.end(), cls[k].pairs.begin(), cls[k].pairs.end());
            parts.insert(parts.end(), cls[k].parts.begin(), cls[k].parts.end());
            pair_off.push_back((int32_t)(pairs.size() / 2));
            part_off.push_back((int32_t)parts.size());
        }
        W.pk_round.clear();
        const int i_pairs = W.pk_round.add(pairs), i_pairoff = W.pk_round.add(pair_off),
                  i_partoff = W.pk_round.add(part_off), i_parts = W.pk_round.add(parts);
        RC(W.pk_round.upload(s));
        RC(W.sel_out.ensure(sel.size() + 1));
        int64_t cnt[4] = {0, 0, 0, 0};
        int n_ccd = 0;
        int max_parts = 0;
        for (int k : sel) max_parts = std::max(max_parts, (int)cls[k].parts.size());
        RC(run_select_steps(c, W.pk_round.ptr(i_pairs), (int)(pairs.size() / 2), W.pk_round.ptr(i_pairoff),
                            W.pk_round.ptr(i_partoff), W.pk_round.ptr(i_parts), (int)sel.size(), (int)parts.size(),
                            max_parts, opt_dt, W.sel_out.p, cnt, &n_ccd));
        RC(W.h_rd.ensure(sel.size() + 1));
        D2G_CUDA(cudaMemcpyAsync(W.h_rd.p, W.sel_out.p, sel.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
        D2G_CUDA(cudaStreamSynchronize(s));
        for (size_t q = 0; q < sel.size(); q++) cls[sel[q]].step = W.h_rd.p[q];
        W.stats[0] += (int64_t)(pairs.size() / 2);
        W.stats[1] += n_ccd;
        W.stats[8] += cnt[0];
        W.stats[9] += cnt[1];
        W.stats[10] += cnt[2];
    }
    W.mark(3);
    for (int k = 0; k < nc; k++) {
        const int sc = cls[k].scene;
        if (cls[k].mct > min_final_s[sc]) continue;
        fine_s[sc] = dmin(fine_s[sc], cls[k].mct + (cls[k].sleeping ? opt_dt : cls[k].step));
    }
    // :172-255 the clusters that start before the earliest end step
    std::vector<int> sleepers, R;
    for (int k = 0; k < nc; k++) {
        if (cls[k].mct > fine_s[cls[k].scene]) continue;
        (cls[k].sleeping ? sleepers : R).push_back(k);
    }
    std::vector<double> static_time(n, 0.0);
    std::vector<uint8_t> static_touched(n, 0);
    if (!sleepers.empty()) {
        std::vector<int32_t> part_off(1, 0), parts;
        std::vector<double> steps;
        for (int k : sleepers) {
            parts.insert(parts.end(), cls[k].parts.begin(), cls[k].parts.end());
            part_off.push_back((int32_t)parts.size());
            steps.push_back(cls[k].step);
            for (size_t q = cls[k].n_dyn; q < cls[k].parts.size(); q++) {
                const int st = cls[k].parts[q];
                if (!static_touched[st]) static_time[st] = h_st[15 * (size_t)W.slot_of[st]];
                static_touched[st] = 1;
                static_time[st] = static_time[st] + cls[k].step;
            }
        }
        W.pk_round.clear();
        const int i_off = W.pk_round.add(part_off), i_parts = W.pk_round.add(parts);
        RC(W.pk_round.upload(s));
        W.pk_round_d.clear();
        const int i_st = W.pk_round_d.add(steps);
        RC(W.pk_round_d.upload(s));
        RC(run_sleep_apply(c, (int)sleepers.size(), W.pk_round.ptr(i_off), W.pk_round.ptr(i_parts),
                           W.pk_round_d.ptr(i_st)));
        D2G_CUDA(cudaStreamSynchronize(s));
    }
    W.mark(4);
    if (!R.empty()) {
        const int nR = (int)R.size();
        Recursion Rc;
        Rc.nR = nR;
        Rc.dyn_base.resize(nR);
        std::vector<int32_t> part_off(1, 0), parts;
        std::vector<double> step0(nR), tmin0(nR);
        for (int r = 0; r < nR; r++) {
            const HostCluster& h = cls[R[r]];
            Rc.dyn_base[r] = Rc.total_dyn;
            Rc.total_dyn += h.n_dyn;
            parts.insert(parts.end(), h.parts.begin(), h.parts.end());
            part_off.push_back((int32_t)parts.size());
            step0[r] = h.step;
            tmin0[r] = h.mct;
        }
        W.pk_round.clear();
        const int i_off = W.pk_round.add(part_off), i_parts = W.pk_round.add(parts);
        RC(W.pk_round.upload(s));
        RC(W.cl_step.ensure(nR + 1));
        RC(W.cl_tmin.ensure(nR + 1));
        RC(W.frame_start.ensure((size_t)(kMaxDepth + 2) * nR + 1));
        D2G_CUDA(cudaMemcpyAsync(W.cl_step.p, step0.data(), nR * sizeof(double), cudaMemcpyHostToDevice, s));
        D2G_CUDA(cudaMemcpyAsync(W.cl_tmin.p, tmin0.data(), nR * sizeof(double), cudaMemcpyHostToDevice, s));
        W.stash_used = 0;
        std::vector<Machine> M(nR);
        for (int r = 0; r < nR; r++) RC(enter_frame(M[r], Rc, r, 0));
        std::vector<int> act, ok;
        for (;;) {
            act.clear();
            for (int r = 0; r < nR; r++)
                if (M[r].need_pde) act.push_back(r);
            if (act.empty()) break;
            W.mark(8);
            RC(flush_ops(c, W, M, W.pk_round.ptr(i_off), W.pk_round.ptr(i_parts)));
            RC(pde_round(c, W, cls, R, act, M, ok));
            for (size_t q = 0; q < act.size(); q++) RC(advance(c, W, Rc, M[act[q]], act[q], ok[q] != 0));
        }
        RC(flush_ops(c, W, M, W.pk_round.ptr(i_off), W.pk_round.ptr(i_parts)));
        RC(check_err(c, W, "stepRecursive"));
        // static bodies: last_dt and sleeping of the last stepped cluster holding them
        std::vector<int> last_r(n, -1);
        for (int r = 0; r < nR; r++) {
            const HostCluster& h = cls[R[r]];
            for (size_t q = h.n_dyn; q < h.parts.size(); q++) last_r[h.parts[q]] = r;
        }
        for (int g = 0; g < n; g++) {
            if (last_r[g] < 0) continue;
            double* ldt = h_st + 15 * (size_t)W.slot_of[g] + 14;
            uint8_t* sl = W.h_sleeping.p + W.slot_of[g];
            *ldt = M[last_r[g]].last_step;
            *sl = (uint8_t)(M[last_r[g]].last_sleep ? 1 : 0);
            D2G_CUDA(cudaMemcpyAsync(c->last_dt.p + g, ldt, sizeof(double), cudaMemcpyHostToDevice, s));
            D2G_CUDA(cudaMemcpyAsync(c->sleeping.p + g, sl, 1, cudaMemcpyHostToDevice, s));
        }
    }
    // static bodies of sleeping clusters: the clock advanced, future = current
    for (int g = 0; g < n; g++) {
        if (!static_touched[g]) continue;
        double* cur = h_st + 15 * (size_t)W.slot_of[g];
        cur[0] = static_time[g];
        D2G_CUDA(cudaMemcpyAsync(c->cur.p + 14 * (size_t)g, cur, 14 * sizeof(double), cudaMemcpyHostToDevice, s));
        D2G_CUDA(cudaMemcpyAsync(c->fut.p + 14 * (size_t)g, cur, 14 * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    D2G_CUDA(cudaStreamSynchronize(s));
    W.mark(8);
    return D2G_OK;
}

}  // namespace
}  // namespace d2g

using namespace d2g;

extern "C" int d2g_world_configure(d2g_ctx* c, const float* local_aabb, float opt_dt, double gravity_z) {
    if (!c || !local_aabb || !(opt_dt > 0.0f)) {
        set_error("invalid world configuration");
        return D2G_ERR_INVALID;
    }
    if (c->n_bodies <= 0 || c->n_meshes <= 0) {
        set_error("set trees and bodies before configuring the world");
        return D2G_ERR_STATE;
    }
    if ((int)c->h_bounding_radius.size() != c->n_bodies) {
        set_error("the world stepper needs the bodies' bounding radii");
        return D2G_ERR_INVALID;
    }
    D2G_CUDA(cudaSetDevice(c->device));
    if (!c->world) c->world = new WorldState();
    WorldState& W = *c->world;
    const int n = c->n_bodies;
    W.local_aabb.assign(local_aabb, local_aabb + 6 * (size_t)n);
    W.opt_dt = opt_dt;
    W.gravity_z = gravity_z;
    W.warm.clear();
    for (int64_t& v : W.stats) v = 0;
    for (double& v : W.phase_ms) v = 0.0;
    W.static_ids.clear();
    W.slot_of.assign(n, -1);
    W.n_dyn_total = 0;
    for (int g = 0; g < n; g++) {
        if (c->h_is_static[g]) {
            W.slot_of[g] = (int)W.static_ids.size();
            W.static_ids.push_back(g);
        } else {
            W.n_dyn_total++;
        }
    }
    RC(W.d_aabb.ensure(6 * (size_t)n));
    D2G_CUDA(cudaMemcpy(W.d_aabb.p, local_aabb, 6 * (size_t)n * sizeof(float), cudaMemcpyHostToDevice));
    RC(W.d_static.ensure(W.static_ids.size() + 1));
    RC(W.d_st_sleep.ensure(W.static_ids.size() + 1));
    if (!W.static_ids.empty())
        D2G_CUDA(cudaMemcpy(W.d_static.p, W.static_ids.data(), W.static_ids.size() * sizeof(int32_t),
                            cudaMemcpyHostToDevice));
    RC(W.h_sleeping.ensure(W.static_ids.size() + 1));
    RC(W.h_ri.ensure(64));
    RC(W.h_rd.ensure(64));
    RC(W.err.ensure(4));
    return D2G_OK;
}

extern "C" int d2g_world_step(d2g_ctx* c, int32_t n_steps) {
    if (!c || n_steps < 0) {
        set_error("invalid arguments");
        return D2G_ERR_INVALID;
    }
    if (!c->world || (int)(c->world->local_aabb.size() / 6) != c->n_bodies) {
        set_error("configure the world (d2g_world_configure) after setting the bodies");
        return D2G_ERR_STATE;
    }
    D2G_CUDA(cudaSetDevice(c->device));
    for (int i = 0; i < n_steps; i++) RC(world_step_once(c, *c->world));
    return D2G_OK;
}

extern "C" int d2g_world_stats(d2g_ctx* c, int64_t* out13) {
    if (!c || !out13 || !c->world) {
        set_error("no world configured");
        return D2G_ERR_STATE;
    }
    for (int i = 0; i < 13; i++) out13[i] = c->world->stats[i];
    return D2G_OK;
}

extern "C" int d2g_world_timing(d2g_ctx* c, double* ms, int32_t n) {
    if (!c || !ms || !c->world || n < 0) {
        set_error("no world configured");
        return D2G_ERR_STATE;
    }
    for (int i = 0; i < n && i < D2G_WORLD_PHASES; i++) ms[i] = c->world->phase_ms[i];
    return D2G_OK;
}

extern "C" int d2g_world_warm(d2g_ctx* c, int32_t* keys, double* vals, int32_t capacity, int32_t* n) {
    if (!c || !n || !c->world) {
        set_error("no world configured");
        return D2G_ERR_STATE;
    }
    const auto& m = c->world->warm;
    *n = (int32_t)m.size();
    int i = 0;
    if (keys && vals)
        for (const auto& kv : m) {
            if (i >= capacity) break;
            keys[2 * i] = kv.first.first;
            keys[2 * i + 1] = kv.first.second;
            vals[i] = kv.second;
            i++;
        }
    if (keys && vals && (int)m.size() > capacity) {
        set_error("warm-start capacity too small");
        return D2G_CAPACITY;
    }
    return D2G_OK;
}
