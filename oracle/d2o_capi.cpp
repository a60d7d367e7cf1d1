// Oracle (test infrastructure only): extern "C" entry points over the CPU
// restatement, loaded by tests/ and by bench.py's CPU-baseline leg through
// ctypes.  Never linked into the product library.
#include <cstring>
#include <vector>

#include "d2o_collide.hpp"
#include "d2o_solve.hpp"
#include "d2o_mass.hpp"
#include "d2o_tree.hpp"

using namespace d2o;

extern "C" {

// Flat scene views.  Layout-identical to d2g_trees / d2g_bodies in include/d2g.h.
typedef struct {
    int32_t n_meshes;
    const int32_t* mesh_node_off;
    const int32_t* nodes;
    const int32_t* ntris;
    const double* tris;
    const double* eps;
    const double* inner_eps;
} o_trees;

typedef struct {
    int32_t n;
    const int32_t* mesh;
    const uint8_t* is_static;
    const double* geo_eps;
    const double* mu;
    const double* mass;
    const double* inv_inertia;  // [n][9]
    double* last;               // [n][14]
    double* cur;                // [n][14]
    double* fut;                // [n][14]
    double* last_dt;            // [n]
    int32_t* sleep_steps;       // [n]
    uint8_t* sleeping;          // [n]
    const double* bounding_radius;
} o_bodies;
}

namespace {

V3 rd3(const double* p) { return V3{p[0], p[1], p[2]}; }
void wr3(double* p, V3 v) {
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}
Tri rdtri(const double* p) { return Tri{rd3(p), rd3(p + 3), rd3(p + 6)}; }
M4 rdm4(const double* p) {
    M4 m;
    for (int i = 0; i < 16; i++) m.m[i / 4][i % 4] = p[i];
    return m;
}
void wrm4(double* p, const M4& m) {
    for (int i = 0; i < 16; i++) p[i] = m.m[i / 4][i % 4];
}
State rdstate(const double* p) {
    State s;
    s.time = p[0];
    s.q = Quat{p[1], p[2], p[3], p[4]};
    s.L = rd3(p + 5);
    s.x = rd3(p + 8);
    s.v = rd3(p + 11);
    return s;
}
void wrstate(double* p, const State& s) {
    p[0] = s.time;
    p[1] = s.q.w;
    p[2] = s.q.x;
    p[3] = s.q.y;
    p[4] = s.q.z;
    wr3(p + 5, s.L);
    wr3(p + 8, s.x);
    wr3(p + 11, s.v);
}
void wrccd(double* out, const CcdResult& r) {
    out[0] = r.dist;
    wr3(out + 1, r.P);
    wr3(out + 4, r.Q);
    out[7] = r.toc;
}
// Contact record: A(3) B(3) eps_a eps_b eps_inner_a eps_inner_b toc pa pb pad = 14 doubles.
void wrcontact(double* p, const Contact& c) {
    wr3(p, c.A);
    wr3(p + 3, c.B);
    p[6] = c.eps_a;
    p[7] = c.eps_b;
    p[8] = c.eps_inner_a;
    p[9] = c.eps_inner_b;
    p[10] = c.toc;
    p[11] = c.pa;
    p[12] = c.pb;
    p[13] = 0.0;
}
Contact rdcontact(const double* p) {
    Contact c;
    c.A = rd3(p);
    c.B = rd3(p + 3);
    c.eps_a = p[6];
    c.eps_b = p[7];
    c.eps_inner_a = p[8];
    c.eps_inner_b = p[9];
    c.toc = p[10];
    c.pa = (int)p[11];
    c.pb = (int)p[12];
    return c;
}

TreeSet to_trees(const o_trees* t) {
    TreeSet T;
    T.n_meshes = t->n_meshes;
    T.mesh_node_off = t->mesh_node_off;
    T.nodes = t->nodes;
    T.ntris = t->ntris;
    T.tris = t->tris;
    T.eps = t->eps;
    T.inner_eps = t->inner_eps;
    return T;
}

M3 rdm3(const double* p) {
    M3 m;
    for (int i = 0; i < 9; i++) m.m[i / 3][i % 3] = p[i];
    return m;
}

std::vector<Body> to_bodies(const o_bodies* b) {
    std::vector<Body> out(b->n);
    for (int i = 0; i < b->n; i++) {
        Body& B = out[i];
        B.mesh = b->mesh[i];
        B.is_static = b->is_static[i] != 0;
        B.geo_eps = b->geo_eps[i];
        B.mu = b->mu[i];
        B.mass = b->mass[i];
        B.ii = rdm3(b->inv_inertia + 9 * (size_t)i);
        B.last = rdstate(b->last + 14 * (size_t)i);
        B.cur = rdstate(b->cur + 14 * (size_t)i);
        B.fut = rdstate(b->fut + 14 * (size_t)i);
        B.last_dt = b->last_dt[i];
        B.sleep_not_moved_steps = b->sleep_steps ? b->sleep_steps[i] : 0;
        B.sleeping = b->sleeping ? b->sleeping[i] != 0 : false;
        B.bounding_radius = b->bounding_radius ? b->bounding_radius[i] : 0.0;
    }
    return out;
}

void from_bodies(const std::vector<Body>& bs, o_bodies* b) {
    for (int i = 0; i < b->n; i++) {
        wrstate(b->last + 14 * (size_t)i, bs[i].last);
        wrstate(b->cur + 14 * (size_t)i, bs[i].cur);
        wrstate(b->fut + 14 * (size_t)i, bs[i].fut);
        b->last_dt[i] = bs[i].last_dt;
        if (b->sleep_steps) b->sleep_steps[i] = bs[i].sleep_not_moved_steps;
        if (b->sleeping) b->sleeping[i] = bs[i].sleeping ? 1 : 0;
    }
}

}  // namespace

extern "C" {

double o_sin(double x) { return psin(x); }
double o_cos(double x) { return pcos(x); }
double o_acos(double x) { return pacos(x); }
double o_log(double x) { return plog(x); }

void o_transformation_euler(const double* euler3, const double* pos3, double* out16) {
    wrm4(out16, transformation(euler_to_quat(rd3(euler3)), rd3(pos3)));
}
void o_transformation_quat(const double* q4, const double* pos3, double* out16) {
    wrm4(out16, transformation(Quat{q4[0], q4[1], q4[2], q4[3]}, rd3(pos3)));
}
void o_mat_inverse(const double* in16, double* out16) { wrm4(out16, mat_inverse(rdm4(in16))); }
void o_xform(const double* p3, const double* m16, double* out3) { wr3(out3, xform(rd3(p3), rdm4(m16))); }
void o_tri_xform(const double* tri9, const double* m16, double* out9) {
    const Tri t = tri_xform(rdtri(tri9), rdm4(m16));
    wr3(out9, t.A);
    wr3(out9 + 3, t.B);
    wr3(out9 + 6, t.C);
}
void o_bary(const double* tri9, const double* p3, double* out3) {
    tri_bary(rdtri(tri9), rd3(p3), out3[0], out3[1], out3[2]);
}
void o_intersect_segment(const double* tri9, const double* e6, double* out_pt3, double* t, int* t_inf, int* is_int) {
    bool ti, ii;
    const V3 p = tri_intersect_segment(rdtri(tri9), Edge{rd3(e6), rd3(e6 + 3)}, *t, ti, ii);
    wr3(out_pt3, p);
    *t_inf = ti;
    *is_int = ii;
}
void o_project_to_plane(const double* tri9, const double* p3, double* out3, int* in_tri) {
    bool in;
    wr3(out3, tri_project_to_plane(rdtri(tri9), rd3(p3), in));
    *in_tri = in;
}
double o_edge_closest(const double* s6, const double* e6, double* P3, double* Q3) {
    V3 P, Q;
    const double d = edge_closest(Edge{rd3(s6), rd3(s6 + 3)}, Edge{rd3(e6), rd3(e6 + 3)}, P, Q);
    wr3(P3, P);
    wr3(Q3, Q);
    return d;
}
void o_tri_tri_dist(const double* a9, const double* b9, double* out7) {
    const DistResult r = tri_tri_dist(rdtri(a9), rdtri(b9));
    out7[0] = r.dist;
    wr3(out7 + 1, r.P);
    wr3(out7 + 4, r.Q);
}
double o_sphere_sphere(const double* ap, const double* av, double ar, const double* bp, const double* bv, double br) {
    return sphere_sphere_first_intersect(rd3(ap), rd3(av), ar, rd3(bp), rd3(bv), br);
}
void o_point_tri_ccd(const double* pt3, const double* pS, const double* pE, const double* tri9, const double* tS,
                     const double* tE, double* out8) {
    wrccd(out8, point_tri_ccd(rd3(pt3), rdm4(pS), rdm4(pE), rdtri(tri9), rdm4(tS), rdm4(tE)));
}
void o_edge_edge_ccd(const double* aS6, const double* aE6, const double* bS6, const double* bE6, double* out8) {
    wrccd(out8, edge_edge_ccd(Edge{rd3(aS6), rd3(aS6 + 3)}, Edge{rd3(aE6), rd3(aE6 + 3)}, Edge{rd3(bS6), rd3(bS6 + 3)},
                              Edge{rd3(bE6), rd3(bE6 + 3)}));
}
void o_tri_tri_ccd(const double* a9, const double* aS, const double* aE, const double* b9, const double* bS,
                   const double* bE, double* out8) {
    const PairMats M = pair_mats(rdm4(aS), rdm4(aE), rdm4(bS), rdm4(bE));
    wrccd(out8, tri_tri_ccd(rdtri(a9), rdtri(b9), M));
}
void o_state_extrapolate(const double* s14, double t, const double* ii9, double* out14) {
    wrstate(out14, state_extrapolate(rdstate(s14), t, rdm3(ii9)));
}
int o_state_interpolate(const double* cur14, const double* last14, double time, double* out14) {
    State o;
    if (!state_interpolate(rdstate(cur14), rdstate(last14), time, o)) return -1;
    wrstate(out14, o);
    return 0;
}

// One level of findContactsBucketComparison over explicit node pairs.
int o_bucket_comparison(const o_trees* t, const o_bodies* b, int ia, int ib, const int32_t* node_pairs, int n,
                        double* out, int cap, int32_t* pair_used) {
    const TreeSet T = to_trees(t);
    std::vector<Body> bs = to_bodies(b);
    std::vector<NodePair> dc(n);
    for (int i = 0; i < n; i++) dc[i] = NodePair{node_pairs[2 * i], node_pairs[2 * i + 1]};
    std::vector<Contact> hits;
    std::vector<int> used;
    bucket_comparison(T, dc, bs[ia], bs[ib], ia, ib, hits, used, nullptr);
    for (int i = 0; i < n; i++) pair_used[i] = used[i];
    if ((int)hits.size() > cap) return -(int)hits.size();
    for (size_t i = 0; i < hits.size(); i++) wrcontact(out + 14 * i, hits[i]);
    return (int)hits.size();
}

// One level of findContactsBucketContinuousComparison (soup stage) with the
// bodies' current and future states as given.
int o_bucket_continuous(const o_trees* t, const o_bodies* b, int ia, int ib, const int32_t* node_pairs, int n,
                        int connected, double* out, int cap, int32_t* pair_used) {
    const TreeSet T = to_trees(t);
    std::vector<Body> bs = to_bodies(b);
    std::vector<NodePair> dc(n);
    for (int i = 0; i < n; i++) dc[i] = NodePair{node_pairs[2 * i], node_pairs[2 * i + 1]};
    const Body &A = bs[ia], &B = bs[ib];
    const PairMats M =
        pair_mats(state_transform(A.cur), state_transform(A.fut), state_transform(B.cur), state_transform(B.fut));
    std::vector<Contact> hits;
    std::vector<int> used;
    if (connected)
        bucket_continuous_connected(T, dc, A, B, ia, ib, M, hits, used, nullptr);
    else
        bucket_continuous_soup(T, dc, A, B, ia, ib, M, hits, used, nullptr);
    for (int i = 0; i < n; i++) pair_used[i] = used[i];
    if ((int)hits.size() > cap) return -(int)hits.size();
    for (size_t i = 0; i < hits.size(); i++) wrcontact(out + 14 * i, hits[i]);
    return (int)hits.size();
}

int o_filter_contacts(const double* in, int n, double margin, int unstable, int continuous, double* out) {
    std::vector<Contact> v(n);
    for (int i = 0; i < n; i++) v[i] = rdcontact(in + 14 * (size_t)i);
    const std::vector<Contact> f = continuous ? filter_continuous_contacts(v, margin) : filter_contacts(v, margin, unstable != 0);
    for (size_t i = 0; i < f.size(); i++) wrcontact(out + 14 * i, f[i]);
    return (int)f.size();
}

// compareTreesFull for each listed body pair (future poses as given).
// counters: [node_pairs, tri_pairs, leaf_pairs]
int o_narrowphase(const o_trees* t, const o_bodies* b, const int32_t* pairs, int n_pairs, double* out, int cap,
                  int32_t* offsets, long long* counters) {
    const TreeSet T = to_trees(t);
    std::vector<Body> bs = to_bodies(b);
    Counters cnt;
    int total = 0;
    offsets[0] = 0;
    for (int p = 0; p < n_pairs; p++) {
        const int ia = pairs[2 * p], ib = pairs[2 * p + 1];
        const std::vector<Contact> r = compare_trees_full(T, bs[ia], bs[ib], ia, ib, &cnt);
        for (const Contact& c : r) {
            if (total < cap) wrcontact(out + 14 * (size_t)total, c);
            total++;
        }
        offsets[p + 1] = total;
    }
    if (counters) {
        counters[0] = cnt.node_pairs;
        counters[1] = cnt.tri_pairs;
        counters[2] = cnt.leaf_pairs;
    }
    return total > cap ? -total : total;
}

// compareTreesFullContinuous for each listed body pair, in order; each call
// re-projects both future states over the pair's max_time (written back).
int o_ccd(const o_trees* t, o_bodies* b, const int32_t* pairs, const double* max_time, int n_pairs, double* out,
          int cap, int32_t* offsets, double* min_time_out, long long* counters) {
    const TreeSet T = to_trees(t);
    std::vector<Body> bs = to_bodies(b);
    Counters cnt;
    int total = 0;
    offsets[0] = 0;
    for (int p = 0; p < n_pairs; p++) {
        const int ia = pairs[2 * p], ib = pairs[2 * p + 1];
        double mt = 0;
        const std::vector<Contact> r =
            compare_trees_full_continuous(T, bs[ia], bs[ib], ia, ib, max_time[p], mt, &cnt);
        if (min_time_out) min_time_out[p] = mt;
        for (const Contact& c : r) {
            if (total < cap) wrcontact(out + 14 * (size_t)total, c);
            total++;
        }
        offsets[p + 1] = total;
    }
    from_bodies(bs, b);
    if (counters) {
        counters[0] = cnt.node_pairs;
        counters[1] = cnt.tri_pairs;
        counters[2] = cnt.leaf_pairs;
    }
    return total > cap ? -total : total;
}


// ---------------------------------------------------------------- world ----
struct o_world {
    World w;
    std::vector<int32_t> mesh_node_off, nodes, ntris;
    std::vector<double> tris, eps, inner_eps;
};

// Copies the trees and bodies into an oracle-owned world.
o_world* o_world_create(const o_trees* t, const o_bodies* b, const float* local_aabb6, float opt_dt,
                        double gravity_z) {
    o_world* W = new o_world();
    int N = t->mesh_node_off[t->n_meshes];
    W->mesh_node_off.assign(t->mesh_node_off, t->mesh_node_off + t->n_meshes + 1);
    W->nodes.assign(t->nodes, t->nodes + 4 * (size_t)N);
    W->ntris.assign(t->ntris, t->ntris + N);
    W->tris.assign(t->tris, t->tris + 72 * (size_t)N);
    W->eps.assign(t->eps, t->eps + 8 * (size_t)N);
    W->inner_eps.assign(t->inner_eps, t->inner_eps + 8 * (size_t)N);
    W->w.T.n_meshes = t->n_meshes;
    W->w.T.mesh_node_off = W->mesh_node_off.data();
    W->w.T.nodes = W->nodes.data();
    W->w.T.ntris = W->ntris.data();
    W->w.T.tris = W->tris.data();
    W->w.T.eps = W->eps.data();
    W->w.T.inner_eps = W->inner_eps.data();
    W->w.bodies = to_bodies(b);
    W->w.local_aabb.assign(local_aabb6, local_aabb6 + 6 * (size_t)b->n);
    W->w.opt_dt = opt_dt;
    W->w.so.gravity_z = gravity_z;
    return W;
}
void o_world_destroy(o_world* W) { delete W; }
void o_world_set_unstable_filter(o_world* W, int u) { W->w.unstable_filter = u != 0; }
int o_world_get_bodies(o_world* W, o_bodies* b) {
    from_bodies(W->w.bodies, b);
    return 0;
}
int o_world_set_bodies(o_world* W, const o_bodies* b) {
    W->w.bodies = to_bodies(b);
    return 0;
}
// Runs n outer steps; returns 0, or -1 if the restated reference hit an
// invalid interpolation (the reference would throw).
int o_world_step(o_world* W, int n) {
    for (int i = 0; i < n; i++) {
        world_step(W->w);
        if (W->w.error) return -1;
    }
    return 0;
}
// stats: ccd_pairs ccd_contacts np_pairs np_contacts solves failures normal_iters friction_iters
//        ccd_node_pairs ccd_tri_pairs ccd_leaf_pairs np_node_pairs np_tri_pairs
void o_world_stats(o_world* W, long long* out13) {
    const StepStats& s = W->w.stats;
    const long long v[13] = {s.ccd_pairs,           s.ccd_contacts,         s.np_pairs,         s.np_contacts,
                             s.solves,              s.failures,             s.normal_iters,     s.friction_iters,
                             s.ccd_cnt.node_pairs,  s.ccd_cnt.tri_pairs,    s.ccd_cnt.leaf_pairs, s.np_cnt.node_pairs,
                             s.np_cnt.tri_pairs};
    for (int i = 0; i < 13; i++) out13[i] = v[i];
}
// Broad phase over the world's current bodies: pairs written as (i, j).
int o_world_broad_phase(o_world* W, int32_t* out_pairs, int cap) {
    const auto B = broad_phase(W->w.bodies, W->w.local_aabb.data());
    if ((int)B.size() > cap) return -(int)B.size();
    for (size_t i = 0; i < B.size(); i++) {
        out_pairs[2 * i] = B[i].first;
        out_pairs[2 * i + 1] = B[i].second;
    }
    return (int)B.size();
}
// Time-step selection for one cluster given by its particles and interactions.
double o_world_select_dt(o_world* W, const int32_t* particles, int np, const int32_t* inter, int ni) {
    Cluster c;
    c.particles.assign(particles, particles + np);
    for (int i = 0; i < ni; i++) c.interactions.push_back(std::make_pair(inter[2 * i], inter[2 * i + 1]));
    return select_time_step(W->w.T, W->w.bodies, c, W->w.opt_dt, &W->w.stats);
}
// Sequential-impulse solve of one cluster over explicit contacts (14-double
// records).  Returns 1 on success, 0 when the solver rejects the step.
// iters_out: [normal, friction].
int o_world_solve(o_world* W, const int32_t* particles, int np, double step_size, const double* contacts, int nc,
                  int* iters_out) {
    Cluster c;
    c.particles.assign(particles, particles + np);
    c.step_size = step_size;
    std::vector<Contact> hits(nc);
    for (int i = 0; i < nc; i++) hits[i] = rdcontact(contacts + 14 * (size_t)i);
    SolveStats ss;
    const bool ok = si_solve(W->w.bodies, c, hits, W->w.warm, W->w.so, &ss);
    if (iters_out) {
        iters_out[0] = ss.normal_iters;
        iters_out[1] = ss.friction_iters;
    }
    return ok ? 1 : 0;
}
int o_world_warm_size(o_world* W) { return (int)W->w.warm.size(); }
int o_world_warm_get(o_world* W, int32_t* keys, double* vals, int cap) {
    int i = 0;
    for (const auto& kv : W->w.warm) {
        if (i >= cap) break;
        keys[2 * i] = kv.first.first;
        keys[2 * i + 1] = kv.first.second;
        vals[i] = kv.second;
        i++;
    }
    return i;
}

// SurrogateTree(V, F, opt) from the PCG32 stream (state, inc) in rng[2]
// (updated): sizes first (buffers null), then a second call with buffers of
// `capacity` nodes; layout as the library's d2g_tree_build.  Returns the node
// count, or -1 when the reference would throw.
int o_tree_build(const double* V, int nv, const int32_t* F, int nf, uint64_t* rng, int32_t* nodes, int32_t* ntris,
                 double* tris, double* eps, double* inner_eps, int capacity) {
    std::vector<Tri> T((size_t)nf);
    for (int f = 0; f < nf; f++) {
        V3 p[3];
        for (int k = 0; k < 3; k++) {
            const int v = F[3 * f + k];
            if (v < 0 || v >= nv) return -1;
            p[k] = V3{V[3 * v], V[3 * v + 1], V[3 * v + 2]};
        }
        T[f] = Tri{p[0], p[1], p[2]};
    }
    Pcg32 r;
    r.state = rng[0];
    r.inc = rng[1];
    FlatTree out;
    try {
        out = build_surrogate_tree(T, r);
    } catch (const std::exception&) {
        return -1;
    }
    const int n = out.size();
    if (nodes && n <= capacity) {
        std::memcpy(nodes, out.nodes.data(), sizeof(int32_t) * 4 * (size_t)n);
        std::memcpy(ntris, out.ntris.data(), sizeof(int32_t) * (size_t)n);
        std::memcpy(tris, out.tris.data(), sizeof(double) * 72 * (size_t)n);
        std::memcpy(eps, out.eps.data(), sizeof(double) * 8 * (size_t)n);
        std::memcpy(inner_eps, out.inner_eps.data(), sizeof(double) * 8 * (size_t)n);
        rng[0] = r.state;
        rng[1] = r.inc;
    }
    return n;
}

// MeshData's mass properties (model/mesh.cpp:53-130): out = volume, centre of
// mass (3), unit inertia tensor (9, row major, about the centre of mass).
void o_mass_properties(const double* V, int nv, const int32_t* F, int nf, int surface, double thickness,
                       double* out13) {
    std::vector<V3> P((size_t)nv);
    for (int i = 0; i < nv; i++) P[i] = V3{V[3 * i], V[3 * i + 1], V[3 * i + 2]};
    std::vector<int> FF(F, F + 3 * (size_t)nf);
    const MassOut o = surface ? mass_surface_model(P, FF, thickness) : mass_volume_model(P, FF);
    out13[0] = o.volume;
    out13[1] = o.com.x;
    out13[2] = o.com.y;
    out13[3] = o.com.z;
    for (int k = 0; k < 9; k++) out13[4 + k] = o.unit_inertia.m[k / 3][k % 3];
}

// Replaces the warm-start store (a state taken from another run).
void o_world_warm_set(o_world* W, const int32_t* keys, const double* vals, int n) {
    W->w.warm.clear();
    for (int i = 0; i < n; i++) W->w.warm[std::make_pair((int)keys[2 * i], (int)keys[2 * i + 1])] = vals[i];
}

}  // extern "C"
