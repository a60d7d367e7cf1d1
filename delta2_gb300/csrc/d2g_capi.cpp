// extern "C" entry points of include/d2g.h: context and device memory,
// input validation, host set-up glue.  Compute lives in d2g_engine.cu.
#include <cuda_runtime.h>

#include <cstring>
#include <algorithm>
#include <cmath>
#include <memory>
#include <string>
#include <vector>

#include "../../include/d2g.h"
#include "d2g_internal.hpp"
#include "host/d2g_scene.hpp"

namespace d2g {
namespace {
thread_local std::string g_err;
}
void set_error(const std::string& msg) { g_err = msg; }
}  // namespace d2g

using d2g::set_error;

#define RC(x)                          \
    do {                               \
        if (int rc_ = (x)) return rc_; \
    } while (0)

struct d2g_scene {
    d2g::Scene s;
    std::unique_ptr<d2g::SceneBuilder> b;  // a scene of the caller's meshes, until finished
};

namespace {

template <class T>
int upload(d2g_ctx* ctx, d2g::DBuf<T>& dst, const T* src, size_t n) {
    RC(dst.ensure(n + 1));
    if (n) D2G_CUDA(cudaMemcpyAsync(dst.p, src, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    return D2G_OK;
}

template <class T>
int download(d2g_ctx* ctx, T* dst, const d2g::DBuf<T>& src, size_t n) {
    if (n) D2G_CUDA(cudaMemcpyAsync(dst, src.p, n * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
    return D2G_OK;
}

int check_ready(d2g_ctx* ctx) {
    if (!ctx) {
        set_error("null context");
        return D2G_ERR_INVALID;
    }
    if (ctx->n_nodes == 0 || ctx->n_bodies == 0) {
        set_error("trees and bodies must be set before a query");
        return D2G_ERR_STATE;
    }
    return D2G_OK;
}

int check_pairs(d2g_ctx* ctx, const int32_t* pairs, int n) {
    if (n < 0 || (n > 0 && !pairs)) {
        set_error("invalid pair list");
        return D2G_ERR_INVALID;
    }
    for (int i = 0; i < 2 * n; i++) {
        if (pairs[i] < 0 || pairs[i] >= ctx->n_bodies) {
            set_error("pair " + std::to_string(i / 2) + " names body " + std::to_string(pairs[i]) +
                      " outside [0, " + std::to_string(ctx->n_bodies) + ")");
            return D2G_ERR_INVALID;
        }
    }
    return D2G_OK;
}

// Copy the results of the last engine call to the caller's host buffers.
int copy_out(d2g_ctx* ctx, int n_pairs, int n_rec, double* contacts, int capacity, int32_t* offsets) {
    if (offsets) RC(download(ctx, offsets, ctx->eng.out_off, (size_t)n_pairs + 1));
    const int n_copy = n_rec < capacity ? n_rec : (capacity > 0 ? capacity : 0);
    if (contacts && n_copy > 0) RC(download(ctx, contacts, ctx->eng.rec_sorted, 14 * (size_t)n_copy));
    D2G_CUDA(cudaStreamSynchronize(ctx->stream));
    if (n_rec > capacity) {
        set_error("contact capacity " + std::to_string(capacity) + " < " + std::to_string(n_rec));
        return D2G_CAPACITY;
    }
    return D2G_OK;
}

}  // namespace

extern "C" {

const char* d2g_last_error(void) { return d2g::g_err.c_str(); }
const char* d2g_version(void) { return "delta2_gb300 0.1 (sm_103a)"; }

// ------------------------------------------------------------- scenes -----
int d2g_scene_make(const d2g_scene_opts* o, d2g_scene** out) {
    if (!o || !out) {
        set_error("null argument");
        return D2G_ERR_INVALID;
    }
    d2g::SceneOpts so;
    so.config = o->config;
    so.nx = o->nx;
    so.ny = o->ny;
    so.nz = o->nz;
    so.spacing = o->spacing;
    so.speed_sigma = o->speed_sigma;
    so.seed = o->seed;
    so.dt = o->dt;
    so.gravity_z = o->gravity_z;
    so.mu = o->mu;
    so.hull_points = o->hull_points > 3 ? o->hull_points : 64;
    so.count = o->count;
    if (o->tree_file) so.tree_file = o->tree_file;
    d2g_scene* s = new d2g_scene();
    std::string err;
    if (!d2g::make_scene(so, s->s, &err)) {
        delete s;
        set_error(err);
        return D2G_ERR_INVALID;
    }
    *out = s;
    return D2G_OK;
}

void d2g_scene_free(d2g_scene* s) { delete s; }

int d2g_scene_create(float dt, double gravity_z, d2g_scene** out) {
    if (!out || !(dt > 0.0f)) {
        set_error("null argument or non-positive time step");
        return D2G_ERR_INVALID;
    }
    d2g_scene* sc = new d2g_scene();
    sc->b.reset(new d2g::SceneBuilder());
    sc->b->s.opt_dt = dt;
    sc->b->s.gravity_z = gravity_z;
    *out = sc;
    return D2G_OK;
}

int d2g_scene_add_mesh(d2g_scene* sc, const double* vertices, int32_t n_vertices, const int32_t* faces,
                       int32_t n_faces, int32_t surface, double* com, int32_t* mesh_id) {
    if (!sc || !sc->b || !com || !mesh_id) {
        set_error(sc && !sc->b ? "the scene is finished" : "null argument");
        return D2G_ERR_INVALID;
    }
    std::string err;
    const int id = d2g::builder_add_mesh(*sc->b, vertices, n_vertices, faces, n_faces, surface != 0, com, &err);
    if (id < 0) {
        set_error(err);
        return D2G_ERR_INVALID;
    }
    *mesh_id = id;
    return D2G_OK;
}

int d2g_scene_add_obj(d2g_scene* sc, const char* path, int32_t surface, double* com, int32_t* mesh_id) {
    if (!sc || !sc->b || !path || !com || !mesh_id) {
        set_error(sc && !sc->b ? "the scene is finished" : "null argument");
        return D2G_ERR_INVALID;
    }
    std::vector<double> V;
    std::vector<int32_t> F;
    std::string err;
    if (!d2g::read_obj(path, V, F, &err)) {
        set_error(err);
        return D2G_ERR_INVALID;
    }
    if (V.size() / 3 > (size_t)INT32_MAX || F.size() / 3 > (size_t)INT32_MAX) {
        set_error("mesh too large");
        return D2G_ERR_INVALID;
    }
    return d2g_scene_add_mesh(sc, V.data(), (int32_t)(V.size() / 3), F.data(), (int32_t)(F.size() / 3), surface, com,
                              mesh_id);
}

int d2g_scene_add_body(d2g_scene* sc, int32_t mesh_id, int32_t is_static, double density, double geo_eps, double mu,
                       const double* position, const double* quaternion, const double* velocity) {
    if (!sc || !sc->b) {
        set_error(sc ? "the scene is finished" : "null scene");
        return D2G_ERR_INVALID;
    }
    std::string err;
    if (!d2g::builder_add_body(*sc->b, mesh_id, is_static != 0, density, geo_eps, mu, position, quaternion, velocity,
                               &err)) {
        set_error(err);
        return D2G_ERR_INVALID;
    }
    return D2G_OK;
}

int d2g_scene_finish(d2g_scene* sc) {
    if (!sc) {
        set_error("null scene");
        return D2G_ERR_INVALID;
    }
    if (!sc->b) return D2G_OK;
    std::string err;
    if (!d2g::builder_finish(*sc->b, &err)) {
        set_error(err);
        return D2G_ERR_INVALID;
    }
    sc->s = std::move(sc->b->s);
    sc->b.reset();
    return D2G_OK;
}

struct d2g_tree_file {
    d2g::TreeSet t;
};

int d2g_trees_save(const d2g_trees* t, const char* path) {
    if (!t || !path || t->n_meshes < 0 || !t->mesh_node_off) {
        set_error("null argument");
        return D2G_ERR_INVALID;
    }
    d2g::TreeSet ts;
    const int M = t->n_meshes;
    const int N = t->mesh_node_off[M];
    if (N < 0 || (N > 0 && (!t->nodes || !t->ntris || !t->tris || !t->eps || !t->inner_eps))) {
        set_error("invalid tree arrays");
        return D2G_ERR_INVALID;
    }
    ts.mesh_node_off.assign(t->mesh_node_off, t->mesh_node_off + M + 1);
    ts.nodes.assign(t->nodes, t->nodes + 4 * (size_t)N);
    ts.ntris.assign(t->ntris, t->ntris + N);
    ts.tris.assign(t->tris, t->tris + 72 * (size_t)N);
    ts.eps.assign(t->eps, t->eps + 8 * (size_t)N);
    ts.inner_eps.assign(t->inner_eps, t->inner_eps + 8 * (size_t)N);
    for (int m = 0; m < M; m++) {  // a mesh's triangles are its leaf buckets'
        int n = 0;
        for (int i = ts.mesh_node_off[m]; i < ts.mesh_node_off[m + 1]; i++)
            if (ts.nodes[4 * (size_t)i] == -1) n += ts.ntris[i];
        ts.mesh_ntris.push_back(n);
    }
    std::string err;
    if (!d2g::save_trees(ts, path, &err)) {
        set_error(err);
        return D2G_ERR_INVALID;
    }
    return D2G_OK;
}

int d2g_trees_load(const char* path, d2g_tree_file** out) {
    if (!path || !out) {
        set_error("null argument");
        return D2G_ERR_INVALID;
    }
    d2g_tree_file* f = new d2g_tree_file();
    std::string err;
    if (!d2g::load_trees(path, f->t, &err)) {
        delete f;
        set_error(err);
        return D2G_ERR_INVALID;
    }
    *out = f;
    return D2G_OK;
}

int d2g_tree_file_view(d2g_tree_file* f, d2g_trees* t) {
    if (!f || !t) {
        set_error("null argument");
        return D2G_ERR_INVALID;
    }
    t->n_meshes = (int32_t)f->t.mesh_ntris.size();
    t->mesh_node_off = f->t.mesh_node_off.data();
    t->nodes = f->t.nodes.data();
    t->ntris = f->t.ntris.data();
    t->tris = f->t.tris.data();
    t->eps = f->t.eps.data();
    t->inner_eps = f->t.inner_eps.data();
    return D2G_OK;
}

void d2g_tree_file_free(d2g_tree_file* f) { delete f; }

int d2g_scene_view(d2g_scene* sc, d2g_trees* t, d2g_bodies* b, const float** local_aabb, float* opt_dt,
                   double* gravity_z) {
    if (!sc) {
        set_error("null scene");
        return D2G_ERR_INVALID;
    }
    if (sc->b) {
        set_error("the scene is still being built: call d2g_scene_finish first");
        return D2G_ERR_INVALID;
    }
    d2g::Scene& s = sc->s;
    if (t) {
        t->n_meshes = (int32_t)s.mesh_node_off.size() - 1;
        t->mesh_node_off = s.mesh_node_off.data();
        t->nodes = s.nodes.data();
        t->ntris = s.ntris.data();
        t->tris = s.tris.data();
        t->eps = s.eps.data();
        t->inner_eps = s.inner_eps.data();
    }
    if (b) {
        b->n = s.n_bodies();
        b->mesh = s.mesh.data();
        b->is_static = s.is_static.data();
        b->geo_eps = s.geo_eps.data();
        b->mu = s.mu.data();
        b->mass = s.mass.data();
        b->inv_inertia = s.inv_inertia.data();
        b->last = s.last.data();
        b->cur = s.cur.data();
        b->fut = s.fut.data();
        b->last_dt = s.last_dt.data();
        b->sleep_steps = s.sleep_steps.data();
        b->sleeping = s.sleeping.data();
        b->bounding_radius = s.bounding_radius.data();
    }
    if (local_aabb) *local_aabb = s.local_aabb.data();
    if (opt_dt) *opt_dt = s.opt_dt;
    if (gravity_z) *gravity_z = s.gravity_z;
    return D2G_OK;
}

int d2g_tree_build(const double* V, int32_t nv, const int32_t* F, int32_t nf, uint64_t* rng, int32_t* n_nodes,
                   int32_t* nodes, int32_t* ntris, double* tris, double* eps, double* inner_eps, int32_t capacity) {
    if (!V || !F || nv < 3 || nf < 1 || !rng || !n_nodes) {
        set_error("invalid mesh");
        return D2G_ERR_INVALID;
    }
    for (int i = 0; i < 3 * nf; i++)
        if (F[i] < 0 || F[i] >= nv) {
            set_error("face index out of range");
            return D2G_ERR_INVALID;
        }
    d2g::Mesh m;
    m.V.assign(V, V + 3 * (size_t)nv);
    m.F.assign(F, F + 3 * (size_t)nf);
    d2g::Pcg32 r;
    r.state = rng[0];
    r.inc = rng[1];
    d2g::Tree t;
    std::string err;
    if (!d2g::build_tree(m, r, t, &err)) {
        set_error(err);
        return D2G_ERR_INVALID;
    }
    *n_nodes = t.n();
    if (!nodes) return D2G_OK;  // size query: rng untouched
    if (capacity < t.n()) {
        set_error("tree capacity too small");
        return D2G_CAPACITY;
    }
    rng[0] = r.state;
    rng[1] = r.inc;
    std::memcpy(nodes, t.nodes.data(), t.nodes.size() * sizeof(int32_t));
    std::memcpy(ntris, t.ntris.data(), t.ntris.size() * sizeof(int32_t));
    std::memcpy(tris, t.tris.data(), t.tris.size() * sizeof(double));
    std::memcpy(eps, t.eps.data(), t.eps.size() * sizeof(double));
    std::memcpy(inner_eps, t.inner_eps.data(), t.inner_eps.size() * sizeof(double));
    return D2G_OK;
}

// ------------------------------------------------------------ context -----
int d2g_ctx_create(int32_t device, d2g_ctx** out) {
    if (!out) {
        set_error("null argument");
        return D2G_ERR_INVALID;
    }
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        set_error("no CUDA device");
        return D2G_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= n) {
        set_error("device index out of range");
        return D2G_ERR_INVALID;
    }
    D2G_CUDA(cudaSetDevice(device));
    d2g_ctx* c = new d2g_ctx();
    c->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&c->h_pinned, 64 * sizeof(int32_t));
    if (e != cudaSuccess) {
        set_error(std::string("context creation: ") + cudaGetErrorString(e));
        delete c;
        return D2G_ERR_CUDA;
    }
    *out = c;
    return D2G_OK;
}

void d2g_ctx_destroy(d2g_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    d2g::mlp_orphan_all(c);  // its networks keep their memory until d2g_mlp_destroy
    d2g::world_free(c->world);
    c->world = nullptr;
    c->mesh_node_off.release();
    c->ntris.release();
    c->nodes.release();
    c->tris.release();
    c->eps.release();
    c->inner_eps.release();
    c->mesh.release();
    c->sleep_steps.release();
    c->is_static.release();
    c->sleeping.release();
    c->geo_eps.release();
    c->mu.release();
    c->mass.release();
    c->inv_inertia.release();
    c->last.release();
    c->cur.release();
    c->fut.release();
    c->last_dt.release();
    c->bounding_radius.release();
    d2g::Engine& E = c->eng;
    E.soup.release();
    E.conn.release();
    E.soup_next.release();
    E.conn_next.release();
    E.entry_hits.release();
    E.cnt_a.release();
    E.cnt_b.release();
    E.off_a.release();
    E.off_b.release();
    E.flags.release();
    E.flag_off.release();
    E.items.release();
    E.res.release();
    E.hit.release();
    E.sub.release();
    E.cres.release();
    E.chit.release();
    E.cflag_off.release();
    E.nn_cnt.release();
    E.nn_off.release();
    E.citem_off.release();
    E.st_mt.release();
    E.st_new_dt.release();
    E.st_step.release();
    E.st_out.release();
    E.st_has.release();
    E.st_cl_pair_off.release();
    E.st_cl_part_off.release();
    E.st_cl_parts.release();
    E.pm.release();
    E.pfut.release();
    E.search.release();
    E.last_pair.release();
    E.rec.release();
    E.rec_sorted.release();
    E.rec_pair.release();
    E.rec_pair_sorted.release();
    E.rec_idx.release();
    E.rec_idx_sorted.release();
    E.out_off.release();
    E.pair_cnt.release();
    E.d_pairs.release();
    E.d_max_time.release();
    E.cub_tmp.release();
    E.cub_tmp2.release();
    E.scratch_i32.release();
    for (auto& p : E.pending) {
        cudaEventDestroy(p.e0);
        cudaEventDestroy(p.e1);
    }
    for (auto ev : E.event_pool) cudaEventDestroy(ev);
    if (c->h_pinned) cudaFreeHost(c->h_pinned);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->stream2) cudaStreamDestroy(c->stream2);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int d2g_ctx_stream(d2g_ctx* c, void** stream) {
    if (!c || !stream) {
        set_error("null argument");
        return D2G_ERR_INVALID;
    }
    *stream = (void*)c->stream;
    return D2G_OK;
}

int d2g_ctx_sync(d2g_ctx* c) {
    if (!c) {
        set_error("null context");
        return D2G_ERR_INVALID;
    }
    D2G_CUDA(cudaStreamSynchronize(c->stream));
    return D2G_OK;
}

int d2g_ctx_set_trees(d2g_ctx* c, const d2g_trees* t) {
    if (!c || !t || t->n_meshes <= 0 || !t->mesh_node_off) {
        set_error("invalid trees");
        return D2G_ERR_INVALID;
    }
    const int N = t->mesh_node_off[t->n_meshes];
    if (N <= 0 || t->mesh_node_off[0] != 0) {
        set_error("invalid mesh_node_off");
        return D2G_ERR_INVALID;
    }
    for (int m = 0; m < t->n_meshes; m++)
        if (t->mesh_node_off[m + 1] <= t->mesh_node_off[m]) {
            set_error("every mesh needs at least one node");
            return D2G_ERR_INVALID;
        }
    for (int g = 0; g < N; g++) {
        const int32_t* nd = t->nodes + 4 * (size_t)g;
        if (t->ntris[g] < 0 || t->ntris[g] > 8 || nd[1] < 0 || nd[1] > 8 ||
            (nd[2] && (nd[0] < 0 || nd[0] + nd[1] > N)) || (!nd[2] && nd[1] != 0)) {
            set_error("invalid node " + std::to_string(g));
            return D2G_ERR_INVALID;
        }
    }
    D2G_CUDA(cudaSetDevice(c->device));
    RC(upload(c, c->mesh_node_off, t->mesh_node_off, (size_t)t->n_meshes + 1));
    RC(upload(c, c->nodes, (const int4*)t->nodes, (size_t)N));
    RC(upload(c, c->ntris, t->ntris, (size_t)N));
    RC(upload(c, c->tris, t->tris, 72 * (size_t)N));
    RC(upload(c, c->eps, t->eps, 8 * (size_t)N));
    RC(upload(c, c->inner_eps, t->inner_eps, 8 * (size_t)N));
    {
        // FP32 bounding spheres of the bucket triangles and eps rounded up,
        // for the discrete narrow phase's candidate prefilter.
        std::vector<float4> sph(8 * (size_t)N, make_float4(0.f, 0.f, 0.f, 0.f));
        std::vector<float> eu(8 * (size_t)N, 0.f);
        for (size_t k = 0; k < 8 * (size_t)N; k++) {
            const double* v = t->tris + 9 * k;
            const double cx = (v[0] + v[3] + v[6]) / 3.0, cy = (v[1] + v[4] + v[7]) / 3.0,
                         cz = (v[2] + v[5] + v[8]) / 3.0;
            double r = 0.0;
            for (int j = 0; j < 3; j++) {
                const double dx = v[3 * j] - cx, dy = v[3 * j + 1] - cy, dz = v[3 * j + 2] - cz;
                r = std::max(r, std::sqrt(dx * dx + dy * dy + dz * dz));
            }
            const float fx = (float)cx, fy = (float)cy, fz = (float)cz;
            // the FP32 centre moved by at most |c - fc|: add it to the radius
            const double moved = std::sqrt((cx - fx) * (cx - fx) + (cy - fy) * (cy - fy) + (cz - fz) * (cz - fz));
            sph[k] = make_float4(fx, fy, fz, std::nextafter((float)(r + moved), INFINITY));
            eu[k] = std::nextafter((float)t->eps[k], INFINITY);
        }
        RC(upload(c, c->tri_sph, sph.data(), sph.size()));
        std::vector<float> t32(72 * (size_t)N);
        for (size_t k = 0; k < t32.size(); k++) t32[k] = (float)t->tris[k];
        RC(upload(c, c->tri32, t32.data(), t32.size()));
        RC(upload(c, c->eps_up, eu.data(), eu.size()));
    }
    D2G_CUDA(cudaStreamSynchronize(c->stream));
    c->n_meshes = t->n_meshes;
    c->n_nodes = N;
    return D2G_OK;
}

int d2g_ctx_set_bodies(d2g_ctx* c, const d2g_bodies* b) {
    if (!c || !b || b->n <= 0) {
        set_error("invalid bodies");
        return D2G_ERR_INVALID;
    }
    if (c->n_meshes == 0) {
        set_error("set trees before bodies");
        return D2G_ERR_STATE;
    }
    for (int i = 0; i < b->n; i++)
        if (b->mesh[i] < 0 || b->mesh[i] >= c->n_meshes) {
            set_error("body " + std::to_string(i) + " has mesh id out of range");
            return D2G_ERR_INVALID;
        }
    const size_t n = (size_t)b->n;
    RC(upload(c, c->mesh, b->mesh, n));
    RC(upload(c, c->is_static, b->is_static, n));
    RC(upload(c, c->geo_eps, b->geo_eps, n));
    RC(upload(c, c->mu, b->mu, n));
    RC(upload(c, c->mass, b->mass, n));
    RC(upload(c, c->inv_inertia, b->inv_inertia, 9 * n));
    RC(upload(c, c->last, (const double*)b->last, 14 * n));
    RC(upload(c, c->cur, (const double*)b->cur, 14 * n));
    RC(upload(c, c->fut, (const double*)b->fut, 14 * n));
    RC(upload(c, c->last_dt, (const double*)b->last_dt, n));
    if (b->sleep_steps) RC(upload(c, c->sleep_steps, (const int32_t*)b->sleep_steps, n));
    if (b->sleeping) RC(upload(c, c->sleeping, (const uint8_t*)b->sleeping, n));
    if (b->bounding_radius) RC(upload(c, c->bounding_radius, b->bounding_radius, n));
    if (!b->sleep_steps) {
        RC(c->sleep_steps.ensure(n));
        D2G_CUDA(cudaMemsetAsync(c->sleep_steps.p, 0, n * sizeof(int32_t), c->stream));
    }
    if (!b->sleeping) {
        RC(c->sleeping.ensure(n));
        D2G_CUDA(cudaMemsetAsync(c->sleeping.p, 0, n, c->stream));
    }
    // one scene until d2g_ctx_set_scenes says otherwise
    RC(c->scene.ensure(n));
    D2G_CUDA(cudaMemsetAsync(c->scene.p, 0, n * sizeof(int32_t), c->stream));
    c->h_scene.assign(n, 0);
    c->n_scenes = 1;
    c->h_is_static.assign(b->is_static, b->is_static + n);
    c->h_geo_eps.assign(b->geo_eps, b->geo_eps + n);
    if (b->bounding_radius)
        c->h_bounding_radius.assign(b->bounding_radius, b->bounding_radius + n);
    else
        c->h_bounding_radius.clear();
    D2G_CUDA(cudaStreamSynchronize(c->stream));
    c->n_bodies = b->n;
    return D2G_OK;
}

int d2g_ctx_set_scenes(d2g_ctx* c, const int32_t* scene_of_body) {
    if (!c || !scene_of_body || c->n_bodies <= 0) {
        set_error("set the bodies before their scenes");
        return D2G_ERR_STATE;
    }
    int n_scenes = 1;
    for (int i = 0; i < c->n_bodies; i++) {
        if (scene_of_body[i] < 0) {
            set_error("negative scene index");
            return D2G_ERR_INVALID;
        }
        n_scenes = std::max(n_scenes, scene_of_body[i] + 1);
    }
    D2G_CUDA(cudaSetDevice(c->device));
    RC(upload(c, c->scene, scene_of_body, (size_t)c->n_bodies));
    D2G_CUDA(cudaStreamSynchronize(c->stream));
    c->h_scene.assign(scene_of_body, scene_of_body + c->n_bodies);
    c->n_scenes = n_scenes;
    return D2G_OK;
}

int d2g_ctx_get_bodies(d2g_ctx* c, d2g_bodies* b) {
    if (!c || !b || b->n != c->n_bodies) {
        set_error("body count mismatch");
        return D2G_ERR_INVALID;
    }
    const size_t n = (size_t)b->n;
    RC(download(c, b->last, c->last, 14 * n));
    RC(download(c, b->cur, c->cur, 14 * n));
    RC(download(c, b->fut, c->fut, 14 * n));
    RC(download(c, b->last_dt, c->last_dt, n));
    if (b->sleep_steps && c->sleep_steps.p) RC(download(c, b->sleep_steps, c->sleep_steps, n));
    if (b->sleeping && c->sleeping.p) RC(download(c, b->sleeping, c->sleeping, n));
    D2G_CUDA(cudaStreamSynchronize(c->stream));
    return D2G_OK;
}

int d2g_ctx_set_fp32_bounds(d2g_ctx* c, int32_t enable) {
    if (!c) {
        set_error("null context");
        return D2G_ERR_INVALID;
    }
    c->eng.fp32_bounds = enable != 0;
    return D2G_OK;
}

int d2g_ctx_set_ccd_certificates(d2g_ctx* c, int32_t enable) {
    if (!c) {
        set_error("null context");
        return D2G_ERR_INVALID;
    }
    c->eng.certificates = enable != 0;
    return D2G_OK;
}

int d2g_mass_properties(d2g_ctx* c, const double* V, int32_t n_vertices, const int32_t* F, int32_t n_faces,
                        const int32_t* mesh_vertex_off, const int32_t* mesh_face_off, const uint8_t* surface,
                        int32_t n_meshes, double thickness, double* out) {
    if (!c || n_meshes < 0 || n_vertices < 0 || n_faces < 0 || (n_meshes > 0 && (!mesh_vertex_off ||
                                                                               !mesh_face_off || !out)) ||
        (n_vertices > 0 && !V) || (n_faces > 0 && !F) || !(thickness > 0.0)) {
        set_error("invalid mesh set");
        return D2G_ERR_INVALID;
    }
    if (n_meshes > 0 && (mesh_vertex_off[0] != 0 || mesh_face_off[0] != 0 ||
                         mesh_vertex_off[n_meshes] != n_vertices || mesh_face_off[n_meshes] != n_faces)) {
        set_error("mesh offsets must start at 0 and end at the vertex and face counts");
        return D2G_ERR_INVALID;
    }
    for (int m = 0; m < n_meshes; m++) {
        const int nv = mesh_vertex_off[m + 1] - mesh_vertex_off[m], nf = mesh_face_off[m + 1] - mesh_face_off[m];
        if (nv < 3 || nf < 1) {
            set_error("mesh " + std::to_string(m) + " needs 3 vertices and a face");
            return D2G_ERR_INVALID;
        }
        for (int i = 3 * mesh_face_off[m]; i < 3 * mesh_face_off[m + 1]; i++)
            if (F[i] < 0 || F[i] >= nv) {
                set_error("mesh " + std::to_string(m) + " has a face index outside its vertices");
                return D2G_ERR_INVALID;
            }
    }
    D2G_CUDA(cudaSetDevice(c->device));
    d2g::Engine& E = c->eng;
    std::vector<uint8_t> surf((size_t)n_meshes + 1, 0);
    if (surface)
        for (int m = 0; m < n_meshes; m++) surf[m] = surface[m] ? 1 : 0;
    RC(upload(c, E.ms_V, V, 3 * (size_t)n_vertices));
    RC(upload(c, E.ms_F, F, 3 * (size_t)n_faces));
    RC(upload(c, E.ms_voff, mesh_vertex_off, (size_t)n_meshes + 1));
    RC(upload(c, E.ms_foff, mesh_face_off, (size_t)n_meshes + 1));
    RC(upload(c, E.ms_surface, surf.data(), (size_t)n_meshes));
    RC(E.ms_out.ensure(22 * (size_t)n_meshes + 1));
    RC(d2g::run_mass_properties(c, E.ms_V.p, E.ms_F.p, E.ms_voff.p, E.ms_foff.p, E.ms_surface.p, n_meshes,
                                thickness, E.ms_out.p));
    RC(download(c, out, E.ms_out, 22 * (size_t)n_meshes));
    D2G_CUDA(cudaStreamSynchronize(c->stream));
    return D2G_OK;
}

int d2g_ccd_features(d2g_ctx* c, const int32_t* pairs, const double* max_time, int32_t n_pairs, float* features) {
    RC(check_ready(c));
    RC(check_pairs(c, pairs, n_pairs));
    if (n_pairs > 0 && (!max_time || !features)) {
        set_error("null max_time or output");
        return D2G_ERR_INVALID;
    }
    D2G_CUDA(cudaSetDevice(c->device));
    RC(upload(c, c->eng.d_pairs, pairs, 2 * (size_t)n_pairs));
    RC(upload(c, c->eng.d_max_time, max_time, (size_t)n_pairs));
    RC(d2g::run_ccd_features(c, c->eng.d_pairs.p, c->eng.d_max_time.p, n_pairs));
    if (n_pairs > 0)
        D2G_CUDA(cudaMemcpyAsync(features, c->eng.pp_feat.p, sizeof(float) * 20 * (size_t)n_pairs,
                                 cudaMemcpyDeviceToHost, c->stream));
    D2G_CUDA(cudaStreamSynchronize(c->stream));
    return D2G_OK;
}

int d2g_ctx_set_ccd_proposal(d2g_ctx* c, d2g_mlp* mlp, float threshold) {
    if (!c || (mlp && d2g::mlp_context(mlp) != c) || !(threshold >= 0.0f && threshold <= 1.0f)) {
        set_error("null context, a network of another context, or a threshold outside [0, 1]");
        return D2G_ERR_INVALID;
    }
    c->eng.proposal = mlp;
    // predicted contact-free: sigmoid(logit) < threshold, i.e. logit < log(threshold / (1 - threshold))
    c->eng.proposal_logit = threshold >= 1.0f ? INFINITY
                            : threshold <= 0.0f ? -INFINITY
                                                : (float)std::log((double)threshold / (1.0 - (double)threshold));
    return D2G_OK;
}

int d2g_ctx_set_ccd_witnesses(d2g_ctx* c, int32_t enable) {
    if (!c) {
        set_error("null context");
        return D2G_ERR_INVALID;
    }
    c->eng.witnesses = enable != 0;
    return D2G_OK;
}

int d2g_ctx_ccd_stats(d2g_ctx* c, int32_t reset, int64_t* stats, int32_t n) {
    if (!c || !stats || n < 0) {
        set_error("null context or output");
        return D2G_ERR_INVALID;
    }
    D2G_CUDA(cudaSetDevice(c->device));
    return d2g::read_ccd_stats(c, stats, n, reset != 0);
}

int d2g_ctx_set_tuning(d2g_ctx* c, int32_t key, int32_t value) {
    if (!c || key < 0 || key >= D2G_TUNE_KEYS) {
        set_error("null context or unknown tuning key");
        return D2G_ERR_INVALID;
    }
    if (value < 0 || (key == D2G_TUNE_EE_FIRST_ITERS && value > 10) ||
        (key == D2G_TUNE_SOLVE_LANES && value != 0 && value != 4 && value != 16) ||
        ((key == D2G_TUNE_SPIN_LIMIT || key == D2G_TUNE_GRID_CONTACTS) && value < 1) ||
        (key == D2G_TUNE_SOLVE_CLUSTER && value != 0 && value != 1 && value != 2 && value != 4 && value != 8 &&
         value != 16)) {
        set_error("tuning value out of range");
        return D2G_ERR_INVALID;
    }
    c->eng.tune[key] = value;
    return D2G_OK;
}

int d2g_ctx_set_level_budget(d2g_ctx* c, int64_t bytes) {
    if (!c || bytes < 0) {
        set_error("null context or negative budget");
        return D2G_ERR_INVALID;
    }
    c->eng.level_budget = bytes;
    c->eng.ccd_chunk = c->eng.np_chunk = 0;  // sizes learned under the old budget
    return D2G_OK;
}

int d2g_ctx_get_tuning(d2g_ctx* c, int32_t key, int32_t* value) {
    if (!c || !value || key < 0 || key >= D2G_TUNE_KEYS) {
        set_error("null argument or unknown tuning key");
        return D2G_ERR_INVALID;
    }
    *value = c->eng.tune[key];
    return D2G_OK;
}

int d2g_ctx_solve_layout(d2g_ctx* c, int32_t* layout, int32_t n) {
    if (!c || !layout || n < D2G_SOLVE_LAYOUT) {
        set_error("null argument or fewer than D2G_SOLVE_LAYOUT entries");
        return D2G_ERR_INVALID;
    }
    for (int i = 0; i < D2G_SOLVE_LAYOUT; i++) layout[i] = c->eng.sv_layout[i];
    return D2G_OK;
}

int d2g_ctx_launches(d2g_ctx* c, int64_t* launches) {
    if (!c || !launches) {
        set_error("null argument");
        return D2G_ERR_INVALID;
    }
    *launches = c->eng.launches;
    return D2G_OK;
}

int d2g_ctx_set_profiling(d2g_ctx* c, int32_t enable) {
    if (!c) {
        set_error("null context");
        return D2G_ERR_INVALID;
    }
    D2G_CUDA(cudaStreamSynchronize(c->stream));
    d2g::Engine& E = c->eng;
    for (auto& p : E.pending) {
        E.event_pool.push_back(p.e0);
        E.event_pool.push_back(p.e1);
    }
    E.pending.clear();
    for (int k = 0; k < d2g::D2G_PROF_KINDS; k++) {
        E.prof_ms[k] = 0;
        E.prof_launches[k] = 0;
        E.prof_items[k] = 0;
    }
    E.profiling = enable != 0;
    return D2G_OK;
}

int d2g_ctx_profile(d2g_ctx* c, int32_t kind, double* ms, int64_t* launches, int64_t* items) {
    if (!c || kind < 0 || kind >= d2g::D2G_PROF_KINDS) {
        set_error("invalid profile query");
        return D2G_ERR_INVALID;
    }
    if (ms) *ms = c->eng.prof_ms[kind];
    if (launches) *launches = c->eng.prof_launches[kind];
    if (items) *items = c->eng.prof_items[kind];
    return D2G_OK;
}

// ------------------------------------------------------------ queries -----
int d2g_compare_trees_full(d2g_ctx* c, const int32_t* pairs, int32_t n_pairs, double* contacts, int32_t capacity,
                           int32_t* offsets, int64_t* counters) {
    RC(check_ready(c));
    RC(check_pairs(c, pairs, n_pairs));
    D2G_CUDA(cudaSetDevice(c->device));
    RC(upload(c, c->eng.d_pairs, pairs, 2 * (size_t)n_pairs));
    int n_rec = 0;
    RC(d2g::run_narrowphase(c, c->eng.d_pairs.p, n_pairs, &n_rec, counters));
    return copy_out(c, n_pairs, n_rec, contacts, capacity, offsets);
}

int d2g_find_contacts_bucket_comparison(d2g_ctx* c, int32_t body_a, int32_t body_b, const int32_t* node_pairs,
                                        int32_t n_node_pairs, double* hits, int32_t capacity, int32_t* pair_used) {
    RC(check_ready(c));
    const int32_t ab[2] = {body_a, body_b};
    RC(check_pairs(c, ab, 1));
    if (n_node_pairs < 0 || (n_node_pairs > 0 && (!node_pairs || !pair_used)) || capacity < 0 ||
        (capacity > 0 && !hits) || n_node_pairs > (INT32_MAX >> 6)) {
        set_error("invalid node pair list or output buffers");
        return D2G_ERR_INVALID;
    }
    for (int i = 0; i < 2 * n_node_pairs; i++)
        if (node_pairs[i] < 0 || node_pairs[i] >= c->n_nodes) {
            set_error("node pair " + std::to_string(i / 2) + " names node " + std::to_string(node_pairs[i]) +
                      " outside [0, " + std::to_string(c->n_nodes) + ")");
            return D2G_ERR_INVALID;
        }
    D2G_CUDA(cudaSetDevice(c->device));
    d2g::Engine& E = c->eng;
    RC(upload(c, E.d_pairs, ab, 2));
    RC(upload(c, E.bucket_nodes, node_pairs, 2 * (size_t)n_node_pairs));
    int n_hits = 0;
    RC(d2g::run_bucket_comparison(c, E.d_pairs.p, E.bucket_nodes.p, n_node_pairs, &n_hits));
    if (n_node_pairs > 0)
        D2G_CUDA(cudaMemcpyAsync(pair_used, E.off_a.p + 1, sizeof(int32_t) * n_node_pairs, cudaMemcpyDeviceToHost,
                                 c->stream));
    const int n_copy = std::min(n_hits, capacity);
    if (n_copy > 0)
        D2G_CUDA(cudaMemcpyAsync(hits, E.rec.p, sizeof(double) * 14 * (size_t)n_copy, cudaMemcpyDeviceToHost,
                                 c->stream));
    D2G_CUDA(cudaStreamSynchronize(c->stream));
    if (n_hits > capacity) {
        set_error("hit capacity " + std::to_string(capacity) + " < " + std::to_string(n_hits));
        return D2G_CAPACITY;
    }
    return D2G_OK;
}

int d2g_compare_trees_full_continuous(d2g_ctx* c, const int32_t* pairs, const double* max_time, int32_t n_pairs,
                                      double* contacts, int32_t capacity, int32_t* offsets, int64_t* counters) {
    RC(check_ready(c));
    RC(check_pairs(c, pairs, n_pairs));
    if (n_pairs > 0 && !max_time) {
        set_error("null max_time");
        return D2G_ERR_INVALID;
    }
    D2G_CUDA(cudaSetDevice(c->device));
    RC(upload(c, c->eng.d_pairs, pairs, 2 * (size_t)n_pairs));
    RC(upload(c, c->eng.d_max_time, max_time, (size_t)n_pairs));
    int n_rec = 0;
    RC(d2g::run_ccd(c, c->eng.d_pairs.p, c->eng.d_max_time.p, n_pairs, &n_rec, counters));
    return copy_out(c, n_pairs, n_rec, contacts, capacity, offsets);
}

int d2g_compare_trees_full_continuous_device(d2g_ctx* c, const int32_t* d_pairs, const double* d_max_time,
                                             int32_t n_pairs, int32_t* n_contacts, const double** d_contacts,
                                             const int32_t** d_offsets, int64_t* counters) {
    RC(check_ready(c));
    if (n_pairs < 0 || (n_pairs > 0 && (!d_pairs || !d_max_time))) {
        set_error("invalid device pair list");
        return D2G_ERR_INVALID;
    }
    D2G_CUDA(cudaSetDevice(c->device));
    // every call checks the caller's device pairs against the current bodies
    // (the buffer's contents, and the bodies, may have changed since the last
    // call) before any kernel indexes by them
    RC(d2g::check_device_pairs(c, d_pairs, n_pairs));
    int n_rec = 0;
    RC(d2g::run_ccd(c, d_pairs, d_max_time, n_pairs, &n_rec, counters));
    D2G_CUDA(cudaStreamSynchronize(c->stream));
    if (n_contacts) *n_contacts = n_rec;
    if (d_contacts) *d_contacts = c->eng.rec_sorted.p;
    if (d_offsets) *d_offsets = c->eng.out_off.p;
    return D2G_OK;
}

int d2g_filter_contacts(d2g_ctx* c, const double* contacts, const int32_t* offsets, int32_t n_groups, double margin,
                        double* out, int32_t capacity, int32_t* out_offsets) {
    RC(check_ready(c));
    if (n_groups < 0 || !offsets || !out_offsets || offsets[0] != 0) {
        set_error("invalid contact groups");
        return D2G_ERR_INVALID;
    }
    for (int g = 0; g < n_groups; g++)
        if (offsets[g + 1] < offsets[g]) {
            set_error("contact group offsets decrease");
            return D2G_ERR_INVALID;
        }
    const int n = offsets[n_groups];
    if (n > 0 && !contacts) {
        set_error("null contacts");
        return D2G_ERR_INVALID;
    }
    D2G_CUDA(cudaSetDevice(c->device));
    d2g::Engine& E = c->eng;
    RC(upload(c, E.up_rec, contacts, 14 * (size_t)n));
    RC(upload(c, E.up_off, offsets, (size_t)n_groups + 1));
    int kept = 0;
    RC(d2g::run_filter(c, E.up_off.p, E.up_rec.p, n_groups, n, margin, &kept));
    RC(download(c, out_offsets, E.flt_off, (size_t)n_groups + 1));
    if (out && kept <= capacity) RC(download(c, out, E.flt, 14 * (size_t)kept));
    D2G_CUDA(cudaStreamSynchronize(c->stream));
    if (kept > capacity) {
        set_error("filtered contacts exceed the capacity");
        return D2G_CAPACITY;
    }
    return D2G_OK;
}

int d2g_solve_clusters(d2g_ctx* c, int32_t n_clusters, const int32_t* particle_off, const int32_t* particles,
                       const double* step, const double* contacts, const int32_t* contact_off,
                       const int32_t* pair_count, const double* warm, double gravity_z, int32_t* status,
                       int32_t* iterations, double* impulse_out, int32_t* pair_out) {
    RC(check_ready(c));
    if (n_clusters < 0 || !particle_off || !contact_off || (n_clusters > 0 && (!particles || !step || !status))) {
        set_error("invalid cluster arrays");
        return D2G_ERR_INVALID;
    }
    if (particle_off[0] != 0 || contact_off[0] != 0) {
        set_error("cluster offsets must start at 0");
        return D2G_ERR_INVALID;
    }
    const int nb = c->n_bodies;
    std::vector<int32_t> owner(nb, -1);
    for (int k = 0; k < n_clusters; k++) {
        if (particle_off[k + 1] < particle_off[k] || contact_off[k + 1] < contact_off[k]) {
            set_error("cluster " + std::to_string(k) + " has decreasing offsets");
            return D2G_ERR_INVALID;
        }
        for (int i = particle_off[k]; i < particle_off[k + 1]; i++) {
            const int g = particles[i];
            if (g < 0 || g >= nb) {
                set_error("cluster particle index out of range");
                return D2G_ERR_INVALID;
            }
            if (!c->h_is_static[g]) {  // a moving body's work area is per body
                if (owner[g] >= 0) {
                    set_error("moving body " + std::to_string(g) + " is in more than one cluster or listed twice");
                    return D2G_ERR_INVALID;
                }
                owner[g] = k;
            }
        }
    }
    const int np = particle_off[n_clusters];
    const int n = contact_off[n_clusters];
    if (n > 0 && (!contacts || !pair_count || !warm)) {
        set_error("null contact arrays");
        return D2G_ERR_INVALID;
    }
    for (int k = 0; k < n_clusters; k++)
        for (int i = contact_off[k]; i < contact_off[k + 1]; i++) {
            const double* h = contacts + 14 * (size_t)i;
            for (int q = 11; q <= 12; q++) {
                const double v = h[q];
                const int g = (v >= 0.0 && v < (double)nb) ? (int)v : -1;
                bool in = g >= 0 && (double)g == v;
                if (in) {
                    bool found = false;
                    for (int j = particle_off[k]; j < particle_off[k + 1] && !found; j++) found = particles[j] == g;
                    in = found;
                }
                if (!in) {
                    set_error("contact " + std::to_string(i) + " names a body outside its cluster");
                    return D2G_ERR_INVALID;
                }
            }
            if (pair_count[i] < 1) {
                set_error("contact pair counts must be positive");
                return D2G_ERR_INVALID;
            }
        }
    D2G_CUDA(cudaSetDevice(c->device));
    d2g::Engine& E = c->eng;
    RC(upload(c, E.up_part_off, particle_off, (size_t)n_clusters + 1));
    RC(upload(c, E.up_parts, particles, (size_t)np));
    RC(upload(c, E.up_step, step, (size_t)n_clusters));
    RC(upload(c, E.up_con_off, contact_off, (size_t)n_clusters + 1));
    RC(upload(c, E.up_rec, contacts, 14 * (size_t)n));
    RC(upload(c, E.up_cnt, pair_count, (size_t)n));
    RC(upload(c, E.up_warm, warm, (size_t)n));
    RC(E.up_status.ensure(n_clusters + 1));
    RC(E.up_iters.ensure(2 * (size_t)n_clusters + 2));
    RC(E.up_imp.ensure(n + 1));
    RC(E.up_ab.ensure(2 * (size_t)n + 2));
    RC(d2g::run_solve(c, n_clusters, E.up_part_off.p, E.up_parts.p, np, E.up_con_off.p, n, E.up_rec.p, E.up_cnt.p,
                      E.up_warm.p, E.up_step.p, gravity_z, E.up_status.p, E.up_iters.p, E.up_imp.p, E.up_ab.p, nullptr,
                      nullptr, contact_off, particle_off));
    RC(download(c, status, E.up_status, (size_t)n_clusters));
    if (iterations) RC(download(c, iterations, E.up_iters, 2 * (size_t)n_clusters));
    if (impulse_out) RC(download(c, impulse_out, E.up_imp, (size_t)n));
    if (pair_out) RC(download(c, pair_out, E.up_ab, 2 * (size_t)n));
    D2G_CUDA(cudaStreamSynchronize(c->stream));
    for (int k = 0; k < n_clusters; k++)
        if (status[k] == 3) {
            set_error("a grid barrier of the sequential-impulse solve gave up waiting");
            return D2G_SPIN_LIMIT;
        }
    for (int k = 0; k < n_clusters; k++)
        if (status[k] != 0) return D2G_SOLVE_FAILED;
    return D2G_OK;
}

int d2g_ctx_broad_phase(d2g_ctx* c, const float* local_aabb, int32_t* pairs, int32_t capacity, int32_t* n_pairs) {
    RC(check_ready(c));
    if (!local_aabb || !n_pairs || (int)c->h_bounding_radius.size() != c->n_bodies) {
        set_error("the device broad phase needs local boxes and the bodies' bounding radii");
        return D2G_ERR_INVALID;
    }
    D2G_CUDA(cudaSetDevice(c->device));
    d2g::Engine& E = c->eng;
    RC(upload(c, E.up_aabb, local_aabb, 6 * (size_t)c->n_bodies));
    RC(E.up_err.ensure(2));
    D2G_CUDA(cudaMemsetAsync(E.up_err.p, 0, sizeof(int32_t), c->stream));
    int n = 0;
    RC(d2g::run_broad_phase(c, E.up_aabb.p, &n, E.up_err.p));
    *n_pairs = n;
    if (pairs && n <= capacity) RC(download(c, pairs, E.bp_pairs, 2 * (size_t)n));
    int32_t err = 0;
    D2G_CUDA(cudaMemcpyAsync(&err, E.up_err.p, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
    D2G_CUDA(cudaStreamSynchronize(c->stream));
    if (err) {
        set_error("invalid state interpolation in the broad phase (the reference throws here)");
        return D2G_ERR_STATE;
    }
    if (pairs && n > capacity) {
        set_error("broad-phase pair capacity too small");
        return D2G_CAPACITY;
    }
    return D2G_OK;
}

int d2g_ctx_separate_clusters(d2g_ctx* c, const int32_t* pairs, int32_t n_pairs, int32_t* n_clusters,
                              int32_t* particle_off, int32_t* particles, int32_t* pair_off, int32_t* cluster_pairs,
                              double* min_current_time, double* step, uint8_t* sleeping) {
    RC(check_ready(c));
    RC(check_pairs(c, pairs, n_pairs));
    if (!n_clusters || !particle_off || !particles || !pair_off || !min_current_time || !step || !sleeping ||
        (n_pairs > 0 && !cluster_pairs)) {
        set_error("null output");
        return D2G_ERR_INVALID;
    }
    for (int k = 0; k < n_pairs; k++)
        if (c->h_is_static[pairs[2 * k]] && c->h_is_static[pairs[2 * k + 1]]) {
            set_error("pair " + std::to_string(k) + " joins two static bodies");
            return D2G_ERR_INVALID;
        }
    D2G_CUDA(cudaSetDevice(c->device));
    d2g::Engine& E = c->eng;
    RC(upload(c, E.d_pairs, pairs, 2 * (size_t)n_pairs));
    RC(E.up_err.ensure(2));
    D2G_CUDA(cudaMemsetAsync(E.up_err.p, 0, sizeof(int32_t), c->stream));
    int n_dyn = 0;
    for (int g = 0; g < c->n_bodies; g++) n_dyn += c->h_is_static[g] ? 0 : 1;
    int nc = 0, np = 0;
    RC(d2g::run_clusters(c, E.d_pairs.p, n_pairs, n_dyn, &nc, &np, E.up_err.p));
    RC(d2g::run_cluster_rollback(c, E.up_err.p));
    *n_clusters = nc;
    RC(download(c, particle_off, E.cl_part_off, (size_t)nc + 1));
    RC(download(c, particles, E.cl_parts, (size_t)np));
    RC(download(c, pair_off, E.cl_pair_off, (size_t)nc + 1));
    RC(download(c, cluster_pairs, E.cl_pairs, 2 * (size_t)n_pairs));
    RC(download(c, min_current_time, E.cl_mct, (size_t)nc));
    RC(download(c, step, E.cl_step, (size_t)nc));
    std::vector<int32_t> sl(nc + 1);
    if (nc) RC(download(c, sl.data(), E.cl_sleep, (size_t)nc));
    int32_t err = 0;
    D2G_CUDA(cudaMemcpyAsync(&err, E.up_err.p, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
    D2G_CUDA(cudaStreamSynchronize(c->stream));
    for (int k = 0; k < nc; k++) sleeping[k] = sl[k] ? 1 : 0;
    if (err) {
        set_error("invalid state interpolation in separateCollisionClusters (the reference throws here)");
        return D2G_ERR_STATE;
    }
    return D2G_OK;
}

int d2g_select_time_steps(d2g_ctx* c, const int32_t* pairs, int32_t n_pairs, const int32_t* cluster_pair_off,
                          const int32_t* cluster_particle_off, const int32_t* cluster_particles, int32_t n_clusters,
                          float opt_dt, double* step_out, int64_t* counters) {
    RC(check_ready(c));
    RC(check_pairs(c, pairs, n_pairs));
    if (n_clusters < 0 || !cluster_pair_off || !cluster_particle_off || (n_clusters > 0 && (!cluster_particles ||
        !step_out))) {
        set_error("invalid cluster arrays");
        return D2G_ERR_INVALID;
    }
    if (cluster_pair_off[0] != 0 || cluster_pair_off[n_clusters] != n_pairs || cluster_particle_off[0] != 0) {
        set_error("cluster offsets must start at 0 and end at the pair count");
        return D2G_ERR_INVALID;
    }
    for (int k = 0; k < n_clusters; k++) {
        if (cluster_pair_off[k + 1] < cluster_pair_off[k] || cluster_particle_off[k + 1] <= cluster_particle_off[k]) {
            set_error("cluster " + std::to_string(k) + " has decreasing offsets or no particles");
            return D2G_ERR_INVALID;
        }
    }
    const int np = cluster_particle_off[n_clusters];
    for (int i = 0; i < np; i++)
        if (cluster_particles[i] < 0 || cluster_particles[i] >= c->n_bodies) {
            set_error("cluster particle index out of range");
            return D2G_ERR_INVALID;
        }
    // a moving body belongs to one cluster, and every interaction's bodies to its cluster
    int max_parts = 0;
    {
        std::vector<int32_t> owner(c->n_bodies, -1), mark(c->n_bodies, -1);
        for (int k = 0; k < n_clusters; k++) {
            max_parts = std::max(max_parts, cluster_particle_off[k + 1] - cluster_particle_off[k]);
            for (int i = cluster_particle_off[k]; i < cluster_particle_off[k + 1]; i++) {
                const int g = cluster_particles[i];
                mark[g] = k;
                if (c->h_is_static[g]) continue;
                if (owner[g] >= 0) {
                    set_error("moving body " + std::to_string(g) + " is in more than one cluster or listed twice");
                    return D2G_ERR_INVALID;
                }
                owner[g] = k;
            }
            for (int i = cluster_pair_off[k]; i < cluster_pair_off[k + 1]; i++)
                if (mark[pairs[2 * i]] != k || mark[pairs[2 * i + 1]] != k) {
                    set_error("interaction " + std::to_string(i) + " names a body outside its cluster");
                    return D2G_ERR_INVALID;
                }
        }
    }
    D2G_CUDA(cudaSetDevice(c->device));
    d2g::Engine& E = c->eng;
    RC(upload(c, E.d_pairs, pairs, 2 * (size_t)n_pairs));
    RC(upload(c, E.st_cl_pair_off, cluster_pair_off, (size_t)n_clusters + 1));
    RC(upload(c, E.st_cl_part_off, cluster_particle_off, (size_t)n_clusters + 1));
    RC(upload(c, E.st_cl_parts, cluster_particles, (size_t)np));
    RC(E.st_out.ensure(n_clusters + 1));
    RC(d2g::run_select_steps(c, E.d_pairs.p, n_pairs, E.st_cl_pair_off.p, E.st_cl_part_off.p, E.st_cl_parts.p,
                             n_clusters, np, max_parts, (double)opt_dt, E.st_out.p, counters));
    RC(download(c, step_out, E.st_out, (size_t)n_clusters));
    D2G_CUDA(cudaStreamSynchronize(c->stream));
    return D2G_OK;
}

}  // extern "C"
