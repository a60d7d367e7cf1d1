/*
 * d2g.hpp — header-only C++17 layer over the C ABI (d2g.h) with the
 * reference's names and conventions, for C++ hosts such as the reference's
 * own strategy classes (namespace delta2_gb300, as the Python package).
 *
 *   collision::compareTreesFull            -> Context::compareTreesFull
 *   collision::compareTreesFullContinuous  -> Context::compareTreesFullContinuous
 *   collision::filterContacts              -> Context::filterContacts
 *   collision::separateCollisionClusters   -> Context::separateCollisionClusters
 *   SequentialImpulses::solve              -> Context::solve (bool, as the reference)
 *   BroadPhaseEmbreeCluster::step          -> Context::step
 *   broadPhaseEmbree                       -> Scene::broadPhase (host) / Context::broadPhase (device)
 *   Mesh(path) + Particle set-up           -> SceneBuilder
 *
 * Errors: a negative status becomes a delta2_gb300::Error exception carrying the code
 * and d2g_last_error()'s message (the reference throws on programmer and
 * geometry errors); D2G_SOLVE_FAILED is the reference's `false`; output
 * capacity is handled inside (D2G_CAPACITY triggers one resized retry).
 */
#ifndef D2G_HPP
#define D2G_HPP

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "d2g.h"

namespace delta2_gb300 {

class Error : public std::runtime_error {
   public:
    Error(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
    int code() const { return code_; }

   private:
    int code_;
};

inline int check(int rc) {
    if (rc < 0) {
        const char* m = d2g_last_error();
        throw Error(rc, m ? m : "d2g error");
    }
    return rc;
}

using Vec3 = std::array<double, 3>;
using Pair = std::array<int32_t, 2>;

// Contact<double> / ContinuousContact<double> (collision_detection/contact.h:
// 9-28, 73-83) as the library's 14-double record: A, B, eps_a, eps_b,
// eps_inner_a, eps_inner_b, toc, body indices.
struct Contact {
    Vec3 A{}, B{};
    double eps_a = 0, eps_b = 0, eps_inner_a = 0, eps_inner_b = 0, toc = 0;
    int32_t p_a = -1, p_b = -1;

    static Contact fromRecord(const double* r) {
        Contact c;
        for (int k = 0; k < 3; k++) {
            c.A[k] = r[k];
            c.B[k] = r[3 + k];
        }
        c.eps_a = r[6];
        c.eps_b = r[7];
        c.eps_inner_a = r[8];
        c.eps_inner_b = r[9];
        c.toc = r[10];
        c.p_a = (int32_t)r[11];
        c.p_b = (int32_t)r[12];
        return c;
    }
    void toRecord(double* r) const {
        for (int k = 0; k < 3; k++) {
            r[k] = A[k];
            r[3 + k] = B[k];
        }
        r[6] = eps_a;
        r[7] = eps_b;
        r[8] = eps_inner_a;
        r[9] = eps_inner_b;
        r[10] = toc;
        r[11] = (double)p_a;
        r[12] = (double)p_b;
        r[13] = 0.0;
    }
};

// Contacts per body pair, in the reference's order.
using PairContacts = std::vector<std::vector<Contact>>;

namespace detail {
inline PairContacts split(const std::vector<double>& rec, const std::vector<int32_t>& off) {
    PairContacts out(off.empty() ? 0 : off.size() - 1);
    for (size_t i = 0; i + 1 < off.size(); i++)
        for (int32_t k = off[i]; k < off[i + 1]; k++)
            out[i].push_back(Contact::fromRecord(rec.data() + (size_t)D2G_CONTACT_LEN * k));
    return out;
}
}  // namespace detail

// A view of a scene's flattened trees and bodies (valid while its Scene lives).
struct SceneView {
    d2g_trees trees{};
    d2g_bodies bodies{};
    const float* local_aabb = nullptr;
    float opt_dt = 0;
    double gravity_z = 0;
};

// A scene: generated (d2g_scene_make) or built from the caller's meshes.
class Scene {
   public:
    explicit Scene(const d2g_scene_opts& opts) { check(d2g_scene_make(&opts, &s_)); }
    Scene(Scene&& o) noexcept : s_(o.s_) { o.s_ = nullptr; }
    Scene& operator=(Scene&& o) noexcept {
        std::swap(s_, o.s_);
        return *this;
    }
    Scene(const Scene&) = delete;
    Scene& operator=(const Scene&) = delete;
    ~Scene() {
        if (s_) d2g_scene_free(s_);
    }

    SceneView view() const {
        SceneView v;
        check(d2g_scene_view(s_, &v.trees, &v.bodies, &v.local_aabb, &v.opt_dt, &v.gravity_z));
        return v;
    }
    // broadPhaseEmbree on the host: pairs i < j in ascending order.
    std::vector<Pair> broadPhase() const {
        const SceneView v = view();
        int32_t n = 0;
        check(d2g_broad_phase(&v.bodies, v.local_aabb, nullptr, 0, &n));
        std::vector<Pair> pairs((size_t)n);
        if (n) check(d2g_broad_phase(&v.bodies, v.local_aabb, pairs[0].data(), n, &n));
        return pairs;
    }
    d2g_scene* handle() const { return s_; }

   private:
    friend class SceneBuilder;
    Scene() = default;
    d2g_scene* s_ = nullptr;
};

// Mesh loading and particle set-up (model/mesh.cpp:9-130,
// model/particle.cpp:7-40): meshes centred at their centre of mass.
class SceneBuilder {
   public:
    SceneBuilder(float dt, double gravity_z) { check(d2g_scene_create(dt, gravity_z, &scene_.s_)); }
    // Returns the mesh id and the centre of mass the mesh was centred at.
    std::pair<int32_t, Vec3> addMesh(const std::vector<Vec3>& V, const std::vector<std::array<int32_t, 3>>& F,
                                     bool surface = false) {
        std::pair<int32_t, Vec3> r{-1, Vec3{}};
        check(d2g_scene_add_mesh(scene_.s_, V.empty() ? nullptr : V[0].data(), (int32_t)V.size(),
                                 F.empty() ? nullptr : F[0].data(), (int32_t)F.size(), surface ? 1 : 0,
                                 r.second.data(), &r.first));
        return r;
    }
    std::pair<int32_t, Vec3> addObj(const std::string& path, bool surface = false) {
        std::pair<int32_t, Vec3> r{-1, Vec3{}};
        check(d2g_scene_add_obj(scene_.s_, path.c_str(), surface ? 1 : 0, r.second.data(), &r.first));
        return r;
    }
    void addBody(int32_t mesh, bool is_static, const Vec3& position,
                 const std::array<double, 4>& quaternion = {1, 0, 0, 0}, const Vec3& velocity = {0, 0, 0},
                 double density = 1000.0, double geo_eps = 0.01, double mu = 0.5) {
        check(d2g_scene_add_body(scene_.s_, mesh, is_static ? 1 : 0, density, geo_eps, mu, position.data(),
                                 quaternion.data(), velocity.data()));
    }
    // Builds the surrogate trees and hands the scene over.
    Scene finish() {
        check(d2g_scene_finish(scene_.s_));
        return std::move(scene_);
    }

   private:
    Scene scene_;
};

// collision::Cluster (collision_detection/cluster.h:9-41): moving members
// ascending, then the static bodies it touches in order of first
// interaction; its interactions in the given order.
struct Cluster {
    std::vector<int32_t> particles;
    std::vector<Pair> interactions;
    double min_current_time = 0, step_size = 0;
    bool sleeping = false;
};

// One cluster for Context::solve: its particles, step and hits.
struct ClusterHits {
    std::vector<int32_t> particles;
    double step = 0;
    std::vector<Contact> hits;
};

// A context on one GPU: device trees and bodies, stream, buffers.
class Context {
   public:
    // Throws Error(D2G_ERR_NO_DEVICE) when there is no usable GPU.
    explicit Context(int32_t device = 0) { check(d2g_ctx_create(device, &c_)); }
    Context(Context&& o) noexcept : c_(o.c_) { o.c_ = nullptr; }
    Context& operator=(Context&& o) noexcept {
        std::swap(c_, o.c_);
        return *this;
    }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    ~Context() {
        if (c_) d2g_ctx_destroy(c_);
    }
    d2g_ctx* handle() const { return c_; }

    void setScene(const Scene& s) {
        const SceneView v = s.view();
        check(d2g_ctx_set_trees(c_, &v.trees));
        check(d2g_ctx_set_bodies(c_, &v.bodies));
    }
    // The device body states back into the scene's arrays.
    void getBodies(const Scene& s) {
        SceneView v = s.view();
        check(d2g_ctx_get_bodies(c_, &v.bodies));
    }

    // compareTreesFull for each pair over the bodies' future states.
    PairContacts compareTreesFull(const std::vector<Pair>& pairs) {
        return query(pairs, [&](double* out, int32_t cap, int32_t* off) {
            return d2g_compare_trees_full(c_, flat(pairs), (int32_t)pairs.size(), out, cap, off, nullptr);
        });
    }
    // ContactDetectionStrategy::findContactsBucketComparison
    // (strategies/contact_detection/contact_detection_strategy.h:11): one
    // level of body pair (a, b)'s discrete traversal over node_pairs (global
    // node ids), with the reference's outputs: hits in its order and the
    // cumulative pair_used_out.
    void findContactsBucketComparison(int32_t a, int32_t b, const std::vector<Pair>& node_pairs,
                                      std::vector<Contact>& hits, std::vector<int>& pair_used_out) {
        const int32_t n = (int32_t)node_pairs.size();
        std::vector<int32_t> used((size_t)n + 1, 0);
        int32_t cap = std::max<int32_t>(64, 64 * n);
        std::vector<double> rec;
        for (int attempt = 0; attempt < 2; attempt++) {
            rec.assign((size_t)D2G_CONTACT_LEN * cap, 0.0);
            const int rc = check(d2g_find_contacts_bucket_comparison(c_, a, b, flat(node_pairs), n, rec.data(), cap,
                                                                     used.data()));
            if (rc != D2G_CAPACITY) break;
            cap = used[n - 1];
        }
        const int32_t total = n ? used[n - 1] : 0;
        hits.clear();
        for (int32_t k = 0; k < total; k++) hits.push_back(Contact::fromRecord(rec.data() + (size_t)D2G_CONTACT_LEN * k));
        pair_used_out.assign(used.begin(), used.begin() + n);
    }
    // compareTreesFullContinuous for each pair over max_time[i].
    PairContacts compareTreesFullContinuous(const std::vector<Pair>& pairs, const std::vector<double>& max_time) {
        if (max_time.size() != pairs.size()) throw Error(D2G_ERR_INVALID, "one max_time per pair");
        return query(pairs, [&](double* out, int32_t cap, int32_t* off) {
            return d2g_compare_trees_full_continuous(c_, flat(pairs), max_time.data(), (int32_t)pairs.size(), out,
                                                     cap, off, nullptr);
        });
    }
    // filterContacts(contacts, margin) of one interaction's contacts.
    std::vector<Contact> filterContacts(const std::vector<Contact>& contacts, double margin = 0.0) {
        std::vector<double> rec(D2G_CONTACT_LEN * (contacts.size() + 1));
        for (size_t i = 0; i < contacts.size(); i++) contacts[i].toRecord(rec.data() + D2G_CONTACT_LEN * i);
        const int32_t off[2] = {0, (int32_t)contacts.size()};
        std::vector<double> out(rec.size());
        int32_t out_off[2] = {0, 0};
        check(d2g_filter_contacts(c_, rec.data(), off, 1, margin, out.data(), (int32_t)contacts.size(), out_off));
        std::vector<Contact> kept;
        for (int32_t k = 0; k < out_off[1]; k++)
            kept.push_back(Contact::fromRecord(out.data() + (size_t)D2G_CONTACT_LEN * k));
        return kept;
    }
    // SequentialImpulses::solve of one cluster with its hits (no warm start
    // entries): true when accepted, false when rejected as the reference
    // rejects; the device future states of its moving bodies are replaced.
    bool solve(const ClusterHits& cl, double gravity_z = -9.8) {
        const int32_t n = (int32_t)cl.hits.size();
        const int32_t part_off[2] = {0, (int32_t)cl.particles.size()}, con_off[2] = {0, n};
        std::vector<double> rec(D2G_CONTACT_LEN * (size_t)(n + 1)), warm((size_t)n + 1, std::nan(""));
        std::vector<int32_t> cnt((size_t)n + 1, 0), ab(2 * (size_t)n + 2);
        for (int32_t i = 0; i < n; i++) {
            cl.hits[i].toRecord(rec.data() + D2G_CONTACT_LEN * (size_t)i);
            const int32_t lo = std::min(cl.hits[i].p_a, cl.hits[i].p_b);
            const int32_t hi = std::max(cl.hits[i].p_a, cl.hits[i].p_b);
            for (int32_t j = 0; j < n; j++)
                cnt[i] += (std::min(cl.hits[j].p_a, cl.hits[j].p_b) == lo &&
                           std::max(cl.hits[j].p_a, cl.hits[j].p_b) == hi)
                              ? 1
                              : 0;
        }
        std::vector<double> imp((size_t)n + 1);
        int32_t status = 0, iters[2] = {0, 0};
        const int rc = check(d2g_solve_clusters(c_, 1, part_off, cl.particles.data(), &cl.step, rec.data(), con_off,
                                                cnt.data(), warm.data(), gravity_z, &status, iters, imp.data(),
                                                ab.data()));
        return rc != D2G_SOLVE_FAILED && status == 0;
    }
    // separateCollisionClusters over the device bodies of scene s (which the
    // context holds): rolls the moving bodies back to their cluster's
    // minimum current time, as the reference does.
    std::vector<Cluster> separateCollisionClusters(const Scene& s, const std::vector<Pair>& pairs) {
        const int32_t nb = s.view().bodies.n, np = (int32_t)pairs.size();
        std::vector<int32_t> poff((size_t)nb + 1), parts((size_t)nb + np + 1), qoff((size_t)nb + 1),
            cp(2 * (size_t)np + 2);
        std::vector<double> mct((size_t)nb + 1), st((size_t)nb + 1);
        std::vector<uint8_t> sl((size_t)nb + 1);
        int32_t ncl = 0;
        check(d2g_ctx_separate_clusters(c_, flat(pairs), np, &ncl, poff.data(), parts.data(), qoff.data(), cp.data(),
                                        mct.data(), st.data(), sl.data()));
        std::vector<Cluster> out((size_t)ncl);
        for (int32_t k = 0; k < ncl; k++) {
            out[k].particles.assign(parts.begin() + poff[k], parts.begin() + poff[k + 1]);
            for (int32_t q = qoff[k]; q < qoff[k + 1]; q++) out[k].interactions.push_back({cp[2 * q], cp[2 * q + 1]});
            out[k].min_current_time = mct[k];
            out[k].step_size = st[k];
            out[k].sleeping = sl[k] != 0;
        }
        return out;
    }
    // broadPhaseEmbree over the device bodies.
    std::vector<Pair> broadPhase(const Scene& s) {
        const SceneView v = s.view();
        int32_t n = 0;
        check(d2g_ctx_broad_phase(c_, v.local_aabb, nullptr, 0, &n));
        std::vector<Pair> pairs((size_t)n);
        if (n) check(d2g_ctx_broad_phase(c_, v.local_aabb, pairs[0].data(), n, &n));
        return pairs;
    }
    // BroadPhaseEmbreeCluster set-up and outer steps over the device bodies.
    void configure(const Scene& s) {
        const SceneView v = s.view();
        check(d2g_world_configure(c_, v.local_aabb, v.opt_dt, v.gravity_z));
    }
    void step(int32_t n = 1) { check(d2g_world_step(c_, n)); }

   private:
    static const int32_t* flat(const std::vector<Pair>& p) { return p.empty() ? nullptr : p[0].data(); }
    template <class Call>
    PairContacts query(const std::vector<Pair>& pairs, Call call) {
        int32_t cap = (int32_t)std::max<size_t>(4096, 64 * pairs.size());
        std::vector<int32_t> off(pairs.size() + 1);
        std::vector<double> rec;
        for (int attempt = 0; attempt < 2; attempt++) {
            rec.assign((size_t)D2G_CONTACT_LEN * cap, 0.0);
            const int rc = check(call(rec.data(), cap, off.data()));
            if (rc != D2G_CAPACITY) return detail::split(rec, off);
            cap = off.back();
        }
        throw Error(D2G_CAPACITY, "contact capacity");
    }
    d2g_ctx* c_ = nullptr;
};

}  // namespace delta2_gb300

#endif
