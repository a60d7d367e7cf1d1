// Internal context of the C ABI: device-resident trees and bodies, the
// growable work buffers of the traversal engine, and error reporting.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/d2g.h"

namespace d2g {

struct WorldState;
void world_free(WorldState* w);

// Kernels timed in profiling mode (d2g_ctx_profile kinds).
enum { PROF_SOUP_FILTER = 0, PROF_SOUP_CCD = 1, PROF_CONN = 2, PROF_NP = 3, PROF_SOLVE = 4, D2G_PROF_KINDS = 8 };

void set_error(const std::string& msg);

#define D2G_CUDA(call)                                                                              \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) {                                                                    \
            ::d2g::set_error(std::string(#call) + ": " + cudaGetErrorString(e_));                   \
            return D2G_ERR_CUDA;                                                                    \
        }                                                                                           \
    } while (0)

// The failed allocation's size and the device memory then free, in the error text.
inline void alloc_error(cudaError_t e, size_t bytes) {
    cudaGetLastError();  // clear the (non-sticky) allocation error
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    set_error(std::string("cudaMalloc of ") + std::to_string(bytes) + " bytes (" + std::to_string(free_b) +
              " of " + std::to_string(total_b) + " free): " + cudaGetErrorString(e));
}

// Device buffer that grows geometrically (capacity in elements); owns its
// memory (freed on destruction, movable, not copyable).
template <class T>
struct DBuf {
    T* p = nullptr;
    size_t cap = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : p(o.p), cap(o.cap) {
        o.p = nullptr;
        o.cap = 0;
    }
    DBuf& operator=(DBuf&& o) noexcept {
        if (this != &o) {
            release();
            p = o.p;
            cap = o.cap;
            o.p = nullptr;
            o.cap = 0;
        }
        return *this;
    }
    ~DBuf() { release(); }
    int ensure(size_t n) {
        if (n <= cap) return D2G_OK;
        if (p) {
            cudaDeviceSynchronize();  // no launch still reads the old buffer
            cudaFree(p);
        }
        p = nullptr;
        size_t c = n + n / 2 + 64;
        cudaError_t e = cudaMalloc((void**)&p, c * sizeof(T));
        if (e != cudaSuccess) {
            cap = 0;
            p = nullptr;
            alloc_error(e, c * sizeof(T));
            return D2G_ERR_CUDA;
        }
        cap = c;
        return D2G_OK;
    }
    // Grow to n elements keeping the first `used` ones (accumulating buffers).
    int ensure_keep(size_t n, size_t used, cudaStream_t stream) {
        if (n <= cap) return D2G_OK;
        size_t c = n + n / 2 + 64;
        T* q = nullptr;
        cudaError_t e = cudaMalloc((void**)&q, c * sizeof(T));
        if (e != cudaSuccess) {
            alloc_error(e, c * sizeof(T));
            return D2G_ERR_CUDA;
        }
        if (p) {
            if (used) {
                e = cudaMemcpyAsync(q, p, used * sizeof(T), cudaMemcpyDeviceToDevice, stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
                if (e != cudaSuccess) {
                    cudaFree(q);
                    set_error(std::string("buffer growth: ") + cudaGetErrorString(e));
                    return D2G_ERR_CUDA;
                }
            }
            cudaDeviceSynchronize();
            cudaFree(p);
        }
        p = q;
        cap = c;
        return D2G_OK;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

// One separation witness (d2g_engine.cu): the key of (body a, body b, node
// of a, node of b) and a separating axis in a's frame.
struct WitnessSlot {
    unsigned long long key;  // 0: empty
    float ax, ay, az;
    int32_t unused;
};

// One frontier entry: body pair index and the two node ids.
struct Entry {
    int32_t pair, na, nb;
};

// Result of one primitive test (tri-tri CCD, point-triangle, edge-edge or
// discrete tri-tri): distance, the two points, time of contact.
struct PrimResult {
    double dist, P[3], Q[3], toc;
};

struct Engine {
    // frontiers
    DBuf<Entry> soup, conn, soup_next, conn_next;
    // per-entry counters / offsets
    DBuf<int32_t> entry_hits, cnt_a, cnt_b, off_a, off_b;
    // items of a stage
    DBuf<int32_t> flags, flag_off, items;
    DBuf<PrimResult> res;
    DBuf<int32_t> hit;
    // flattened primitive tests of a CCD level: soup sub-test results, leaf-pair
    // results, their hit flags and offsets
    DBuf<PrimResult> sub, cres;
    DBuf<int32_t> chit, cflag_off, nn_cnt, nn_off, citem_off;
    // time-step selection
    DBuf<double> st_mt, st_new_dt, st_step, st_out;
    DBuf<int32_t> st_has, st_cl_pair_off, st_cl_part_off, st_cl_parts, st_loc;
    // contact filtering
    DBuf<int32_t> flt_idx, flt_order, flt_keep, flt_pos, flt_cnt, flt_off, np_tri;
    DBuf<unsigned long long> flt_keys, flt_keys_s;
    DBuf<double> flt_mid;
    // CCD candidates: FP32 poses (8 per pair), survivor counts and lists
    DBuf<float> pm32c;
    DBuf<int32_t> ccd_cnt, ccd_list;  // CCD survivors: counts (point-triangle, edge-edge) and lists
    // discrete narrow-phase candidates: FP32 poses, survivor masks and offsets
    DBuf<float> pm32;
    DBuf<uint32_t> np_mask;
    DBuf<int32_t> np_cnt, np_off;
    DBuf<double> flt;
    // sequential-impulse solve
    DBuf<unsigned long long> sv_keys, sv_keys_out;
    DBuf<int32_t> sv_vals, sv_order, sv_wave_idx, sv_wave_off, sv_wave_cursor;
    DBuf<double> sv_static_imp, sv_sdelta;
    DBuf<int32_t> sv_scon, sv_list, sv_grid, sv_cl_flags;
    int sv_cl_fit[4] = {-1, -1, -1, -1};  // resident thread-block clusters of 16, 8, 4, 2 solve blocks
    int sv_layout[4] = {0, 0, 0, 0};  // the last solve call's layout (d2g_ctx_solve_layout)
    DBuf<unsigned char> sv_bw_raw, sv_cw_raw;
    // GPU broad phase (d2g_broadphase.cu)
    DBuf<float> bp_box;
    DBuf<unsigned long long> bp_key, bp_key_s;
    DBuf<int32_t> bp_idx, bp_order, bp_count, bp_pairs;
    DBuf<long long> bp_range, bp_roff;
    DBuf<unsigned long long> bp_pkey, bp_pkey2;
    // GPU cluster separation (d2g_broadphase.cu)
    DBuf<int32_t> uf_parent, uf_root, uf_roff, cl_cid, cl_uidx, cl_member, cl_pair_cid, cl_piota, cl_porder,
        cl_pairs, cl_st_pos, cl_st_pos_s, cl_st_flag, cl_st_off, cl_st_body, cl_st_body3, cl_st_body4, cl_n_dyn,
        cl_n_stat, cl_n_all, cl_dyn_off, cl_stat_off, cl_part_off, cl_pair_cnt, cl_pair_off, cl_sleep, cl_parts;
    DBuf<uint32_t> cl_ukey, cl_ukey_s, cl_pkey_s;
    DBuf<unsigned long long> cl_st_key, cl_st_key_s, cl_st_key2, cl_st_key3, cl_st_key4;
    DBuf<double> cl_mct, cl_step;
    // inputs / outputs of the host filter and solve entry points
    DBuf<double> up_rec, up_warm, up_step, up_imp;
    DBuf<float> up_aabb;
    DBuf<int32_t> up_err;
    DBuf<int32_t> up_off, up_part_off, up_parts, up_con_off, up_cnt, up_status, up_iters, up_ab;
    // per pair
    DBuf<double> pm;    // [pairs][128] pose matrices
    DBuf<double> pfut;  // [pairs][28] projected futures of a and b
    DBuf<float> search;
    DBuf<int32_t> last_pair;
    // results (processing order) and the sorted output
    DBuf<double> rec, rec_sorted;
    DBuf<int32_t> rec_pair, rec_pair_sorted, rec_idx, rec_idx_sorted, out_off, pair_cnt;
    DBuf<int32_t> d_pairs, bucket_nodes;
    // mesh sets of d2g_mass_properties
    DBuf<double> ms_V, ms_out;
    DBuf<int32_t> ms_F, ms_voff, ms_foff;
    DBuf<uint8_t> ms_surface;
    DBuf<double> d_max_time;
    DBuf<uint8_t> cub_tmp, cub_tmp2;
    // phased edge-edge CCD (d2g_engine.cu)
    DBuf<double> ee_rec;
    DBuf<int32_t> ee_work;
    int ee_grid = 0;  // k_ee_rest4 grid (every block resident)
    // traversal chunking: root entries of the call's pairs; a byte budget for
    // a level's buffers (0: a third of the device memory)
    DBuf<Entry> roots;
    long long level_budget = 0;
    size_t device_bytes = 0;
    int ccd_chunk = 0, np_chunk = 0;  // pair-chunk sizes that fitted the budget last time (0: whole calls)
    // launch-shape settings (d2g_ctx_set_tuning): speed only, results identical
    int tune[D2G_TUNE_KEYS] = {2, 512, 0, 1 << 25, 16, 0};
  // cub_tmp2: scans on the context's second stream
    DBuf<int32_t> scratch_i32;  // small device scalars
    // instrumentation: kernel launches issued, and optional per-kernel event timing
    long long launches = 0;
    bool profiling = false;
    bool fp32_bounds = true;  // FP32 candidate bounds before the FP64 tests (results identical either way)
    bool certificates = true;  // conservative-advancement cut-off of edge-edge CCD tests (results identical)
    // learned proposal (d2g_ctx_set_ccd_proposal): the network consulted by
    // CCD calls, the hit logit below which a pair is predicted contact-free,
    // per-pair features, predictions and skip flags
    // separation witnesses (d2g_ctx_set_ccd_witnesses): the table of
    // separating axes, its size, the witnesses written since it was cleared,
    // per-entry skip flags of the current level
    bool witnesses = false;
    DBuf<WitnessSlot> wt_table;
    int wt_log2cap = 20;
    long long wt_inserts = 0;
    DBuf<uint8_t> wt_flag;
    d2g_mlp* proposal = nullptr;
    float proposal_logit = 0.0f;
    DBuf<float> pp_feat;
    DBuf<uint8_t> pp_skip;
    // CCD counters since the last read-and-reset: [0] edge-edge tests cut by
    // conservative advancement, [1] Newton iterations they did not run
    DBuf<unsigned long long> ccd_stats;
    struct Pending {
        int kind;
        cudaEvent_t e0, e1;
        long long items;
    };
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> event_pool;
    double prof_ms[D2G_PROF_KINDS] = {0};
    long long prof_launches[D2G_PROF_KINDS] = {0};
    long long prof_items[D2G_PROF_KINDS] = {0};
};

}  // namespace d2g

struct d2g_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    // a second stream for independent work within a call (forked from and
    // joined back into `stream` by the two events)
    cudaStream_t stream2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // trees
    int n_meshes = 0, n_nodes = 0;
    d2g::DBuf<int32_t> mesh_node_off, ntris;
    d2g::DBuf<int4> nodes;
    d2g::DBuf<double> tris, eps, inner_eps;
    d2g::DBuf<float4> tri_sph;  // per tree triangle: centroid, bounding radius (rounded up), FP32
    d2g::DBuf<float> eps_up;    // eps rounded up to FP32
    d2g::DBuf<float> tri32;     // bucket triangles in FP32 ([N][8][9])
    // bodies
    int n_bodies = 0;
    d2g::DBuf<int32_t> mesh, sleep_steps;
    d2g::DBuf<uint8_t> is_static, sleeping;
    d2g::DBuf<double> geo_eps, mu, mass, inv_inertia, last, cur, fut, last_dt, bounding_radius;
    // independent scenes batched in one context: scene of every body
    d2g::DBuf<int32_t> scene;
    std::vector<int32_t> h_scene;
    int n_scenes = 1;
    // host copies of the constant body data the host-side stepper reads
    std::vector<uint8_t> h_is_static;
    std::vector<double> h_geo_eps, h_bounding_radius;
    d2g::Engine eng;
    d2g::WorldState* world = nullptr;  // adaptive cluster stepper (d2g_world.cpp)
    int32_t* h_pinned = nullptr;  // small pinned scratch for counts
    std::vector<d2g_mlp*> nets;   // networks created on this context (orphaned when it is destroyed)
};

namespace d2g {
// Profiling-mode event marks around a kernel (d2g_engine.cu); collect after a
// stream synchronisation.
int prof_mark_begin(d2g_ctx* ctx, int kind, long long items);
void prof_mark_end(d2g_ctx* ctx, int idx);
void prof_mark_collect(d2g_ctx* ctx);
// Engine entry points (d2g_engine.cu).
// Consumer of a CCD call's records chunk by chunk (pairs [p0, p1)): when run_ccd
// is given one, each chunk's records are sorted into rec_sorted with offsets
// out_off[0 .. p1 - p0], handed over, and dropped, so the call never holds
// every record at once.
struct CcdSink {
    void* user;
    int (*consume)(d2g_ctx* ctx, void* user, int p0, int p1);
};
int run_ccd(d2g_ctx* ctx, const int32_t* d_pairs, const double* d_max_time, int n_pairs, int* n_out,
            int64_t* counters, const CcdSink* sink = nullptr);
int run_narrowphase(d2g_ctx* ctx, const int32_t* d_pairs, int n_pairs, int* n_out, int64_t* counters);
// The learned proposal's network (d2g_mlp.cu): forward pass over device
// feature rows, and the context the network belongs to.
int mlp_forward_device(d2g_mlp* m, const float* d_feat, int n, const float** d_out);
d2g_ctx* mlp_context(d2g_mlp* m);
// Detach every network of a context that is being destroyed: each keeps its
// device memory until d2g_mlp_destroy, and its other calls report the lost
// context.
void mlp_orphan_all(d2g_ctx* ctx);
int run_ccd_features(d2g_ctx* ctx, const int32_t* d_pairs, const double* d_max_time, int n);
// D2G_ERR_INVALID (with a message) unless every body index of the device pair
// list lies inside the context's bodies; one stream synchronisation.
int check_device_pairs(d2g_ctx* ctx, const int32_t* d_pairs, int n);
// Mass properties of many meshes (d2g_mesh.cu): out [n][22].
int run_mass_properties(d2g_ctx* ctx, const double* d_V, const int32_t* d_F, const int32_t* d_voff,
                        const int32_t* d_foff, const uint8_t* d_surface, int n_meshes, double thickness,
                        double* d_out);
// CCD counters (D2G_CCD_STATS entries, see d2g_ctx_ccd_stats), read on the host.
constexpr int kCcdStats = 8;
int read_ccd_stats(d2g_ctx* ctx, int64_t* out, int n, bool reset);
// One level of one body pair's discrete traversal over the caller's node
// pairs (d_pair: the pair's two bodies; d_node_pairs [n][2] global node ids):
// every hit as a contact record in E.rec, the cumulative hit count after each
// node pair in E.off_a[1 .. n].
int run_bucket_comparison(d2g_ctx* ctx, const int32_t* d_pair, const int32_t* d_node_pairs, int n, int* n_hits);
// Time-step selection (d2g_step.cu).
// n_parts: particles of all clusters; max_cluster_parts: of the largest.
int run_select_steps(d2g_ctx* ctx, const int32_t* d_pairs, int n_pairs, const int32_t* d_cl_pair_off,
                     const int32_t* d_cl_part_off, const int32_t* d_cl_parts, int n_clusters, int n_parts,
                     int max_cluster_parts, double opt_dt, double* d_out, int64_t* counters,
                     int* n_ccd_contacts = nullptr);
int run_outer_project(d2g_ctx* ctx, double opt_dt);
int run_pde_prepare(d2g_ctx* ctx, int n_clusters, const int32_t* d_part_off, const int32_t* d_parts,
                    const double* d_step, const double* d_tmin, int32_t* d_err);
int run_pde_finish(d2g_ctx* ctx, int n_clusters, const int32_t* d_part_off, const int32_t* d_parts,
                   const double* d_step, const int32_t* d_status, int32_t* d_will_sleep);
int run_rollback(d2g_ctx* ctx, const double* d_t_body, int32_t* d_err);
int run_sleep_apply(d2g_ctx* ctx, int n_clusters, const int32_t* d_part_off, const int32_t* d_parts,
                    const double* d_step);
// stepRecursive bookkeeping ops (k_cluster_ops): int4 (code, frame slot, stash offset, 0).
enum { D2G_OP_ENTER = 1, D2G_OP_SPLIT = 2, D2G_OP_SAVE = 3, D2G_OP_MID = 4, D2G_OP_RESTORE = 5, D2G_OP_EXIT = 6 };
int run_cluster_ops(d2g_ctx* ctx, int n_active, const int32_t* d_cl_idx, const int32_t* d_op_off, const int4* d_ops,
                    const int32_t* d_part_off, const int32_t* d_parts, double* d_cl_step, double* d_cl_tmin,
                    double* d_frame_start, double* d_stash, int32_t* d_err);
// Broad phase and cluster separation over the device bodies (d2g_broadphase.cu).
int run_broad_phase(d2g_ctx* ctx, const float* d_aabb, int* n_out, int32_t* d_err);
int run_clusters(d2g_ctx* ctx, const int32_t* d_pairs, int n_pairs, int n_dyn_total, int* n_clusters_out,
                 int* n_parts_out, int32_t* d_err);
int run_cluster_rollback(d2g_ctx* ctx, int32_t* d_err);
// Contact filtering and sequential impulses (d2g_solve.cu).
int run_filter(d2g_ctx* ctx, const int32_t* d_off, const double* d_rec, int n_pairs, int n_rec, double margin,
               int* n_out);
int run_solve(d2g_ctx* ctx, int n_clusters, const int32_t* d_part_off, const int32_t* d_parts, int n_parts,
              const int32_t* d_con_off, int n_con, const double* d_rec, const int32_t* d_pair_cnt,
              const double* d_warm, const double* d_step, double gravity_z, int32_t* d_status, int32_t* d_iters,
              double* d_out_impulse, int32_t* d_out_ab, const int32_t* d_con_pair, double* d_pair_warm,
              const int32_t* h_con_off = nullptr, const int32_t* h_part_off = nullptr);
}  // namespace d2g
