// Oracle (test infrastructure only): CCD-driven time-step selection, the
// per-cluster sequential-impulse solve, broad phase, cluster separation and
// the adaptive cluster stepper, restated from the reference.
#pragma once
#include <algorithm>
#include <map>
#include <utility>
#include <vector>

#include "d2o_collide.hpp"

namespace d2o {

// collision_detection/cluster.h:9-41
struct Cluster {
    std::vector<int> particles;                      // global body indices (local id = position)
    std::vector<std::pair<int, int>> interactions;   // broad-phase pairs (a < b)
    double step_size = 0;
    bool sleeping = true;
    double min_current_time = 0;
    bool is_static = true;
    int local(int g) const {
        for (size_t i = 0; i < particles.size(); i++)
            if (particles[i] == g) return (int)i;
        return -1;
    }
};

struct StepStats {
    long long ccd_pairs = 0, ccd_contacts = 0, np_pairs = 0, np_contacts = 0, solves = 0, failures = 0;
    long long normal_iters = 0, friction_iters = 0;
    Counters ccd_cnt, np_cnt;
};

// -------------------------------------------------- time-step selection ----
// collision_detection/separate_clusters.cpp:497-554: the step scale a single
// continuous contact asks for (1.0 = no restriction).  Returns false when the
// contact is skipped (`continue`).
inline double contact_step_scale(const Contact& c, const Body& A, const Body& B, double max_dt) {
    double scale = 1.0;
    const V3 hit_normal = c.A - c.B;
    const double interaction_dist = c.eps_a + c.eps_b;
    const V3 a_vel = future_point_velocity(A.fut, A.ii, c.A);
    const V3 b_vel = future_point_velocity(B.fut, B.ii, c.B);
    const V3 rel = a_vel - b_vel;
    if (dot(normalized(hit_normal), normalized(rel)) <= 0.0 || norm(hit_normal) < 1e-4) {
        if (norm(hit_normal) < 1e-4) {
            if (c.toc == 0.0) return 1.0;
            const double toc_start = dmax(0.0, c.toc - (norm(rel) * max_dt) / interaction_dist);
            const double new_step = lerp(toc_start, c.toc, 0.75);
            scale = dmin(scale, new_step);
        } else if (c.toc < 1.0) {
            const double proj_vel = -(dot(normalized(hit_normal), rel));
            const double depth = interaction_dist - norm(hit_normal);
            const double proj_dist = (proj_vel * c.toc) * max_dt;
            if (proj_dist > 1e-6) {
                if (depth < proj_dist) {
                    const double new_step = lerp(c.toc * (1.0 - depth / proj_dist), c.toc, 0.5);
                    scale = dmin(scale, new_step);
                } else {
                    const double future_point = c.toc + ((1.0 - c.toc) * interaction_dist) / (proj_vel * max_dt);
                    const double new_step = lerp(c.toc, dmin(future_point, 1.0), 0.8);
                    scale = dmin(scale, new_step);
                }
            }
        }
    }
    return scale;
}

// collision_detection/separate_clusters.cpp:462-599
// fineCollisionClustersWithTimeStepSelection, then the clamp of
// strategies/time_step_size/time_step_selection_dynamic_continuous.cpp:17-21.
inline double select_time_step(const TreeSet& T, std::vector<Body>& bodies, Cluster& cl, float opt_dt,
                               StepStats* st = nullptr) {
    const int n = (int)cl.particles.size();
    std::vector<double> step(n);
    for (int i = 0; i < n; i++) step[i] = bodies[cl.particles[i]].last_dt;
    cl.step_size = -1.0;
    for (const auto& it : cl.interactions) {
        const int ga = it.first, gb = it.second;
        const int la = cl.local(ga), lb = cl.local(gb);
        Body &A = bodies[ga], &B = bodies[gb];
        const double max_dt = dmin(A.last_dt, B.last_dt);
        double mt;
        const std::vector<Contact> ccs =
            compare_trees_full_continuous(T, A, B, ga, gb, max_dt, mt, st ? &st->ccd_cnt : nullptr);
        if (st) {
            st->ccd_pairs++;
            st->ccd_contacts += (long long)ccs.size();
        }
        if (!ccs.empty()) {
            double min_scaling = 1.0;
            for (const Contact& c : ccs) min_scaling = dmin(min_scaling, contact_step_scale(c, A, B, max_dt));
            const double new_dt = max_dt * min_scaling;
            const double use = dmin(new_dt, dmin(step[la], step[lb]));
            if (!A.is_static) step[la] = use;
            if (!B.is_static) step[lb] = use;
        }
    }
    for (const auto& it : cl.interactions) {
        const int la = cl.local(it.first), lb = cl.local(it.second);
        const bool sa = bodies[it.first].is_static, sb = bodies[it.second].is_static;
        int id;
        if (!sa && !sb)
            id = la;
        else if (sa && sb)
            continue;
        else if (sa)
            id = lb;
        else
            id = la;
        if (cl.step_size < 0.0)
            cl.step_size = step[la];
        else
            cl.step_size = dmin(cl.step_size, step[id]);
    }
    if (cl.step_size < 0.0) cl.step_size = bodies[cl.particles[0]].last_dt;
    cl.step_size = dmax(1e-3, dmin(cl.step_size, (double)opt_dt));
    return cl.step_size;
}

// ---------------------------------------------------- sequential impulses --
// strategies/contact_force/LocalContact.h:6-23
struct LocalContact {
    V3 local_A, local_B, global_centre, global_normal;
    double mass_eff_normal;
    double start_dist;
    double impulse, impulse_offset;
    V3 last_friction_impulse, last_rot_A, last_rot_B;
};

// model/forces.h:101-108 calcTorque
inline V3 calc_torque(V3 force, V3 point, V3 com) { return cross(-force, point - com); }

// strategies/contact_force/sequential_impulses.cpp:46-70 updateState
inline State update_state(const State& f, double t, V3 imp, V3 imp_off, V3 rimp, V3 rimp_off, const Body& p) {
    State u = f;
    u.v = f.v + imp / p.mass;
    u.x = f.x + (imp_off / p.mass) * t;
    u.L = f.L + rimp;
    const M3 R = qmat(f.q);
    const M3 Iinv = m3_mul(m3_mul(R, p.ii), m3_transpose(R));
    const V3 omega = m3_vec(Iinv, f.L + t * rimp_off);
    const Quat d = qexp((0.5 * omega) * t);
    u.q = qmul(d, f.q);
    return u;
}

// strategies/contact_force/sequential_impulses.cpp:72-96 updateStateImmediate
inline State update_state_immediate(const State& f, double t, V3 imp, V3 imp_off, V3 rimp, V3 rimp_off,
                                    const Body& p) {
    State u = f;
    u.v = f.v + imp / p.mass;
    u.x = (f.x + (imp_off / p.mass) * t) + (imp / p.mass) * t;
    u.L = f.L + rimp;
    const M3 R = qmat(f.q);
    const M3 Iinv = m3_mul(m3_mul(R, p.ii), m3_transpose(R));
    const V3 omega = m3_vec(Iinv, (f.L + t * rimp_off) + t * rimp);
    const Quat d = qexp((0.5 * omega) * t);
    u.q = qmul(d, f.q);
    return u;
}

using WarmStore = std::map<std::pair<int, int>, double>;

// Solver options: gravity (contact_force_strategy.cpp:10-13 uses -9.8).
struct SolveOpts {
    double gravity_z = -9.8;
};

struct SolveStats {
    int normal_iters = 0, friction_iters = 0;
};

// Sort key of Contact::operator< (collision_detection/contact.h:17-21).
inline double contact_proportion(const Contact& c) { return norm(c.A - c.B) / (c.eps_a + c.eps_b); }

// strategies/contact_force/sequential_impulses.cpp:104-638 SequentialImpulses::solve.
// `hits` are sorted in place with std::stable_sort (the reference uses the
// unstable std::sort; ties keep interaction order here and on the GPU).
inline bool si_solve(std::vector<Body>& bodies, const Cluster& cl, std::vector<Contact>& hits, WarmStore& warm,
                     const SolveOpts& o, SolveStats* ss = nullptr) {
    std::stable_sort(hits.begin(), hits.end(),
                     [](const Contact& a, const Contact& b) { return contact_proportion(a) < contact_proportion(b); });
    const int nc = (int)hits.size();
    const int np = (int)cl.particles.size();
    std::vector<LocalContact> C;
    std::vector<int> la(nc), lb(nc);
    for (int c = 0; c < nc; c++) {
        LocalContact lc;
        lc.start_dist = norm(hits[c].A - hits[c].B);
        if (lc.start_dist < 1e-6 && cl.step_size > 1e-4) return false;
        const Body& A = bodies[hits[c].pa];
        const Body& B = bodies[hits[c].pb];
        lc.local_A = xform(hits[c].A, mat_inverse(state_transform(A.fut)));
        lc.local_B = xform(hits[c].B, mat_inverse(state_transform(B.fut)));
        lc.global_centre = (hits[c].A + hits[c].B) / 2.0;
        lc.global_normal = (hits[c].B - hits[c].A) / 2.0;
        const V3 rA = hits[c].A - A.fut.x;
        const V3 rB = hits[c].B - B.fut.x;
        const V3 rnA = cross(rA, lc.global_normal);
        const V3 rnB = cross(rB, lc.global_normal);
        const double imA = 1.0 / A.mass, imB = 1.0 / B.mass;
        double k = 0.0;
        if (!A.is_static) k += imA + quad_form(rnA, A.ii);
        if (!B.is_static) k += imB + quad_form(rnB, B.ii);
        lc.mass_eff_normal = k < 1e-6 ? 0.0 : 1.0 / k;
        lc.impulse = 0.0;
        lc.impulse_offset = 0.0;
        lc.last_friction_impulse = V3{0, 0, 0};
        lc.last_rot_A = V3{0, 0, 0};
        lc.last_rot_B = V3{0, 0, 0};
        C.push_back(lc);
        la[c] = cl.local(hits[c].pa);
        lb[c] = cl.local(hits[c].pb);
    }
    const double t = cl.step_size;
    std::vector<V3> imp(np), rimp(np), ioff(np), roff(np);
    std::vector<State> FS(np), FSf(np);
    for (int p = 0; p < np; p++) {
        const Body& B = bodies[cl.particles[p]];
        const V3 f = V3{B.mass * 0.0, B.mass * 0.0, B.mass * o.gravity_z};
        imp[p] = f * t;
        rimp[p] = V3{0, 0, 0};
        ioff[p] = V3{0, 0, 0};
        roff[p] = V3{0, 0, 0};
        FS[p] = B.fut;
        FSf[p] = B.fut;
    }
    // Warm start apply (sequential_impulses_warm_start.cpp:11-26).
    for (int c = 0; c < nc; c++) {
        const int lo = std::min(hits[c].pa, hits[c].pb), hi = std::max(hits[c].pa, hits[c].pb);
        auto f = warm.find(std::make_pair(lo, hi));
        if (f != warm.end()) C[c].impulse = f->second * 0.75;
    }
    for (int c = 0; c < nc; c++) {
        const int a = la[c], b = lb[c];
        const V3 n = normalized(C[c].global_normal);
        const V3 p1A = xform(C[c].local_A, state_transform(FS[a]));
        const V3 p1B = xform(C[c].local_B, state_transform(FS[b]));
        const V3 u = (-n) * C[c].impulse;
        imp[a] = imp[a] + u;
        imp[b] = imp[b] - u;
        const V3 rA = calc_torque(u, p1A, FS[a].x);
        const V3 rB = calc_torque(-u, p1B, FS[b].x);
        rimp[a] = rimp[a] + rA;
        rimp[b] = rimp[b] + rB;
    }
    auto integrate = [&](int p) {
        const Body& B = bodies[cl.particles[p]];
        if (B.is_static) return;
        FS[p] = update_state(B.fut, t, imp[p], ioff[p], rimp[p], roff[p], B);
        FSf[p] = update_state_immediate(B.fut, t, imp[p], ioff[p], rimp[p], roff[p], B);
    };
    for (int p = 0; p < np; p++) integrate(p);

    if (nc > 0) {
        bool converged = false;
        int it = 0;
        while (!converged && it < 1000) {
            std::vector<V3> last_imp = imp;
            for (int c = 0; c < nc; c++) {
                const int a = la[c], b = lb[c];
                const Body& A = bodies[hits[c].pa];
                const Body& B = bodies[hits[c].pb];
                const V3 n = normalized(C[c].global_normal);
                const double outer = (hits[c].eps_a + hits[c].eps_b) * 0.25;
                const V3 p1A = xform(C[c].local_A, state_transform(FS[a]));
                const V3 p1B = xform(C[c].local_B, state_transform(FS[b]));
                const double d1 = dot(p1B, n) - dot(p1A, n);
                const V3 v1A = state_point_velocity(FS[a], p1A, A.ii);
                const V3 v1B = state_point_velocity(FS[b], p1B, B.ii);
                const double v1 = dot(v1A, n) - dot(v1B, n);
                const double m = C[c].mass_eff_normal;
                const double damp = 0.1;
                const double dimp = d1 < outer ? (v1 * m) * damp : -C[c].impulse;
                const double last_mag = C[c].impulse;
                C[c].impulse = dmax(C[c].impulse + dimp, 0.0);
                const double upd = C[c].impulse - last_mag;
                const V3 u = (-n) * upd;
                imp[a] = imp[a] + u;
                imp[b] = imp[b] - u;
                rimp[a] = rimp[a] + calc_torque(u, p1A, FS[a].x);
                rimp[b] = rimp[b] + calc_torque(-u, p1B, FS[b].x);
                const double lower_slop = dmax(outer * 0.2, outer - C[c].start_dist);
                const double slop = lerp(lower_slop, outer * 0.2, 0.3);
                const double pen = outer - d1;
                const double doff = d1 < outer ? ((damp * m) * dmax(0.0, pen - slop)) / t : -C[c].impulse_offset;
                const double last_off = C[c].impulse_offset;
                C[c].impulse_offset = dmax(C[c].impulse_offset + doff, 0.0);
                const double upd_off = C[c].impulse_offset - last_off;
                const V3 uo = (-n) * upd_off;
                ioff[a] = ioff[a] + uo;
                ioff[b] = ioff[b] - uo;
                integrate(a);
                integrate(b);
            }
            converged = true;
            for (int p = 0; p < np; p++) {
                if (norm(imp[p] - last_imp[p]) > 1e-6) {
                    converged = false;
                    break;
                }
            }
            it++;
        }
        if (ss) ss->normal_iters = it;

        std::vector<V3> upd_total(nc, V3{0, 0, 0});
        it = 0;
        converged = false;
        while (!converged && it < 100) {
            std::map<std::pair<int, int>, int> per_pair;
            for (int c = 0; c < nc; c++) {
                const int a = la[c], b = lb[c];
                const Body& A = bodies[hits[c].pa];
                const Body& B = bodies[hits[c].pb];
                const V3 n = normalized(C[c].global_normal);
                const V3 p1A = xform(C[c].local_A, state_transform(FS[a]));
                const V3 p1B = xform(C[c].local_B, state_transform(FS[b]));
                const V3 v1A = A.is_static ? V3{0, 0, 0} : state_point_velocity(FS[a], p1A, A.ii);
                const V3 v1B = B.is_static ? V3{0, 0, 0} : state_point_velocity(FS[b], p1B, B.ii);
                const V3 lpA = xform(C[c].local_A, state_transform(A.cur));
                const V3 fpA = xform(C[c].local_A, state_transform(FSf[a]));
                const V3 vdA = (fpA - lpA) / cl.step_size;
                const V3 lpB = xform(C[c].local_B, state_transform(B.cur));
                const V3 fpB = xform(C[c].local_B, state_transform(FSf[b]));
                const V3 vdB = (fpB - lpB) / cl.step_size;
                const V3 vAB = v1A - v1B;
                const V3 vABd = vdA - vdB;
                const V3 vt = vAB - dot(vAB, n) * n;
                const V3 vtd = vABd - dot(vABd, n) * n;
                const double mu = dmin(A.mu, B.mu);
                const double max_force = (C[c].impulse * mu) * 10;
                const V3 rA = hits[c].A - A.fut.x;
                const V3 rB = hits[c].B - B.fut.x;
                const V3 tan = normalized(vt);
                const V3 rtA = cross(rA, tan), rtB = cross(rB, tan);
                const V3 tand = normalized(vtd);
                const V3 rtAd = cross(rA, tand), rtBd = cross(rB, tand);
                const double imA = 1.0 / A.mass, imB = 1.0 / B.mass;
                double kt = 0.0, ktd = 0.0;
                if (!A.is_static) {
                    kt += imA + quad_form(rtA, A.ii);
                    ktd += imA + quad_form(rtAd, A.ii);
                }
                if (!B.is_static) {
                    kt += imB + quad_form(rtB, B.ii);
                    ktd += imB + quad_form(rtBd, B.ii);
                }
                const double mit = kt < 1e-6 ? 0.0 : 1.0 / kt;
                (void)ktd;
                const V3 dfi = ((-vt) * mit) * 0.9;
                V3 total = C[c].last_friction_impulse + dfi;
                total = normalized(total) * dclamp(norm(total), 0.0, max_force);
                upd_total[c] = total;
                per_pair[std::make_pair(std::min(a, b), std::max(a, b))]++;
            }
            converged = true;
            for (int c = 0; c < nc; c++) {
                const int a = la[c], b = lb[c];
                const double cnt = (double)per_pair[std::make_pair(std::min(a, b), std::max(a, b))];
                const V3 p1A = xform(C[c].local_A, state_transform(FS[a]));
                const V3 p1B = xform(C[c].local_B, state_transform(FS[b]));
                const V3 u = (upd_total[c] - C[c].last_friction_impulse) / cnt;
                C[c].last_friction_impulse = upd_total[c];
                imp[a] = imp[a] + u;
                imp[b] = imp[b] - u;
                if (norm(u) > 1e-4) converged = false;
                const V3 rfA = calc_torque(C[c].last_friction_impulse, p1A, FS[a].x);
                const V3 rfB = calc_torque(-C[c].last_friction_impulse, p1B, FS[b].x);
                rimp[a] = rimp[a] - C[c].last_rot_A;
                rimp[b] = rimp[b] - C[c].last_rot_B;
                C[c].last_rot_A = rfA;
                C[c].last_rot_B = rfB;
                rimp[a] = rimp[a] + C[c].last_rot_A;
                rimp[b] = rimp[b] + C[c].last_rot_B;
                // Friction offsets are never populated (:522-524 commented out):
                // a zero update is still added, as the reference does.
                const V3 uo = (V3{0, 0, 0} - V3{0, 0, 0}) / cnt;
                ioff[a] = ioff[a] + uo;
                ioff[b] = ioff[b] - uo;
                if (norm(uo) > 1e-4) converged = false;
                roff[a] = roff[a] + calc_torque(uo, p1A, FS[a].x);
                roff[b] = roff[b] + calc_torque(-uo, p1B, FS[b].x);
            }
            for (int p = 0; p < np; p++) integrate(p);
            it++;
        }
        if (ss) ss->friction_iters = it;
    }
    for (int p = 0; p < np; p++) bodies[cl.particles[p]].fut = FS[p];
    // Warm start update (sequential_impulses_warm_start.cpp:28-54): the
    // inverted find() stores the last contact's impulse for each body pair.
    std::map<std::pair<int, int>, std::pair<double, int>> acc;
    for (int c = 0; c < nc; c++) {
        const auto key = std::make_pair(std::min(hits[c].pa, hits[c].pb), std::max(hits[c].pa, hits[c].pb));
        auto f = acc.find(key);
        if (f != acc.end()) {
            f->second = std::make_pair(C[c].impulse, 1);
        } else {
            acc[key] = std::make_pair(0.0 + C[c].impulse, 1);
        }
    }
    for (auto& kv : acc) warm[kv.first] = kv.second.first / kv.second.second;
    return true;
}

// ------------------------------------------------------------ broad phase --
// collision_detection/broad_phase_embree.cpp:87-116 (bounds, float) and
// :186-238 (filter).  Embree's rtcCollide pair order is not deterministic; the
// declared order here is ascending (i, j).
struct FBox {
    float lo[3], hi[3];
};

inline void fbox_extend(FBox& b, const float lo[3], const float hi[3]) {
    for (int k = 0; k < 3; k++) {
        b.lo[k] = std::min(b.lo[k], lo[k]);
        b.hi[k] = std::max(b.hi[k], hi[k]);
    }
}

inline FBox body_bounds(const Body& p, const float* local_aabb6) {
    FBox b;
    for (int k = 0; k < 3; k++) {
        b.lo[k] = std::numeric_limits<float>::infinity();
        b.hi[k] = -std::numeric_limits<float>::infinity();
    }
    if (p.is_static) {
        // model/mesh.cpp:137-155: the 8 corners of the local AABB through the float transform.
        const M4 Td = state_transform(p.cur);
        float T[4][4];
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) T[i][j] = (float)Td.m[i][j];
        for (int xi = 0; xi < 2; xi++)
            for (int yi = 0; yi < 2; yi++)
                for (int zi = 0; zi < 2; zi++) {
                    const float v[3] = {xi == 0 ? local_aabb6[0] : local_aabb6[3],
                                        yi == 0 ? local_aabb6[1] : local_aabb6[4],
                                        zi == 0 ? local_aabb6[2] : local_aabb6[5]};
                    float r[4];
                    for (int i = 0; i < 4; i++) r[i] = ((T[i][0] * v[0] + T[i][1] * v[1]) + T[i][2] * v[2]) + T[i][3] * 1.0f;
                    const float w[3] = {r[0] / r[3], r[1] / r[3], r[2] / r[3]};
                    fbox_extend(b, w, w);
                }
    } else {
        const float br = (float)p.bounding_radius;
        const State* s[3] = {&p.last, &p.cur, &p.fut};
        for (int i = 0; i < 3; i++) {
            const float t[3] = {(float)s[i]->x.x, (float)s[i]->x.y, (float)s[i]->x.z};
            const float lo[3] = {-br + t[0], -br + t[1], -br + t[2]};
            const float hi[3] = {br + t[0], br + t[1], br + t[2]};
            fbox_extend(b, lo, hi);
        }
    }
    const float e = (float)p.geo_eps;
    for (int k = 0; k < 3; k++) {
        b.lo[k] = b.lo[k] - e;
        b.hi[k] = b.hi[k] + e;
    }
    return b;
}

// `ok` (optional) turns false on an invalid interpolation, where the
// reference's State::interpolate throws (model/state.cpp:56-58).
inline std::vector<std::pair<int, int>> broad_phase(const std::vector<Body>& bodies, const float* local_aabbs,
                                                    bool* ok = nullptr) {
    const int n = (int)bodies.size();
    std::vector<FBox> boxes(n);
    for (int i = 0; i < n; i++) boxes[i] = body_bounds(bodies[i], local_aabbs + 6 * (size_t)i);
    std::vector<std::pair<int, int>> out;
    for (int i = 0; i < n; i++) {
        for (int j = i + 1; j < n; j++) {
            const Body &a = bodies[i], &b = bodies[j];
            if (a.is_static && b.is_static) continue;
            bool ov = true;
            for (int k = 0; k < 3; k++)
                ov = ov && boxes[i].lo[k] <= boxes[j].hi[k] && boxes[j].lo[k] <= boxes[i].hi[k];
            if (!ov) continue;
            State as = a.cur, bs = b.cur;
            if (!a.is_static && !b.is_static) {
                const bool good = a.cur.time < b.cur.time ? state_interpolate(b.cur, b.last, a.cur.time, bs)
                                                          : state_interpolate(a.cur, a.last, b.cur.time, as);
                if (!good && ok) *ok = false;
            }
            const double t = sphere_sphere_first_intersect(as.x, as.v, a.bounding_radius + a.geo_eps, bs.x, bs.v,
                                                           b.bounding_radius + b.geo_eps);
            if (t >= 0.0 && t < dmax(a.last_dt, b.last_dt)) out.push_back(std::make_pair(i, j));
        }
    }
    return out;
}

// ------------------------------------------------------ cluster separation --
// collision_detection/separate_clusters.cpp:355-459.  Components are labelled
// by breadth-first search from the lowest unlabelled index (igl's labelling
// is assumed to give the same order).  Returns false on an invalid rollback.
inline bool separate_clusters(const std::vector<std::pair<int, int>>& B, std::vector<Body>& bodies,
                              std::vector<Cluster>& out) {
    const int n = (int)bodies.size();
    std::vector<std::vector<int>> adj(n);
    for (const auto& e : B) {
        if (!bodies[e.first].is_static && !bodies[e.second].is_static) {
            adj[e.first].push_back(e.second);
            adj[e.second].push_back(e.first);
        }
    }
    std::vector<int> comp(n, -1);
    int nc = 0;
    for (int s = 0; s < n; s++) {
        if (comp[s] >= 0) continue;
        std::vector<int> q{s};
        comp[s] = nc;
        for (size_t h = 0; h < q.size(); h++)
            for (int v : adj[q[h]])
                if (comp[v] < 0) {
                    comp[v] = nc;
                    q.push_back(v);
                }
        nc++;
    }
    std::vector<Cluster> cls(nc);
    for (auto& c : cls) {
        c.sleeping = true;
        c.min_current_time = std::numeric_limits<double>::infinity();
        c.step_size = std::numeric_limits<double>::infinity();
        c.is_static = true;
    }
    for (int p = 0; p < n; p++) {
        Cluster& c = cls[comp[p]];
        c.particles.push_back(p);
        c.min_current_time = dmin(c.min_current_time, bodies[p].cur.time);
        c.step_size = dmin(c.step_size, bodies[p].last_dt);
        if (!(bodies[p].sleeping || bodies[p].is_static)) c.sleeping = false;
    }
    for (const auto& e : B) {
        const int a = e.first, b = e.second;
        if (bodies[a].is_static && bodies[b].is_static) continue;
        for (auto& c : cls) {
            const bool a_in = std::find(c.particles.begin(), c.particles.end(), a) != c.particles.end();
            const bool b_in = std::find(c.particles.begin(), c.particles.end(), b) != c.particles.end();
            if (a_in) {
                if (b_in)
                    c.interactions.push_back(e);
                else if (bodies[b].is_static) {
                    c.particles.push_back(b);
                    c.interactions.push_back(e);
                }
            } else if (b_in && bodies[a].is_static) {
                c.particles.push_back(a);
                c.interactions.push_back(e);
            }
        }
    }
    for (auto& c : cls) {
        for (int p : c.particles) {
            if (!bodies[p].is_static) {
                State r;
                if (!state_interpolate(bodies[p].cur, bodies[p].last, c.min_current_time, r)) return false;
                bodies[p].cur = r;
                c.is_static = false;
            }
        }
    }
    out.clear();
    for (auto& c : cls)
        if (!c.is_static) out.push_back(c);
    return true;
}

// ----------------------------------------------------------------- stepper -
struct World {
    TreeSet T;
    std::vector<Body> bodies;
    std::vector<float> local_aabb;  // [n][6]
    float opt_dt = 0.01f;
    WarmStore warm;
    SolveOpts so;
    StepStats stats;
    bool unstable_filter = false;
    bool error = false;
};

// strategies/PDE/PDE_explicit.cpp:30-142 PDEExplicit::step
inline bool pde_step(World& w, Cluster& cl) {
    for (int p : cl.particles) {
        Body& B = w.bodies[p];
        B.last_dt = cl.step_size;
        if (!B.is_static) {
            State r;
            if (!state_interpolate(B.cur, B.last, cl.min_current_time, r)) {
                w.error = true;
                return true;
            }
            B.cur = r;
            B.fut = state_extrapolate(B.cur, B.last_dt, B.ii);
        }
    }
    std::vector<Contact> hits;
    for (const auto& it : cl.interactions) {
        std::vector<Contact> cs = compare_trees_full(w.T, w.bodies[it.first], w.bodies[it.second], it.first,
                                                     it.second, &w.stats.np_cnt);
        w.stats.np_pairs++;
        std::vector<Contact> f = filter_contacts(cs, 0.0, w.unstable_filter);
        w.stats.np_contacts += (long long)f.size();
        hits.insert(hits.end(), f.begin(), f.end());
    }
    SolveStats ss;
    w.stats.solves++;
    if (!si_solve(w.bodies, cl, hits, w.warm, w.so, &ss)) {
        w.stats.failures++;
        return false;
    }
    w.stats.normal_iters += ss.normal_iters;
    w.stats.friction_iters += ss.friction_iters;
    bool will_sleep = true;
    for (int p : cl.particles) {
        Body& B = w.bodies[p];
        if (B.is_static) continue;
        bool can = state_stationary(B.last) && state_stationary(B.cur) && state_stationary(B.fut);
        can = can && B.last.time < B.cur.time && B.cur.time < B.fut.time;
        if (!can)
            B.sleep_not_moved_steps = 0;
        else
            B.sleep_not_moved_steps++;
        if (B.sleep_not_moved_steps < 20) will_sleep = false;
        B.last = B.cur;
        B.cur = B.fut;
        B.fut = state_extrapolate(B.cur, cl.step_size, B.ii);
    }
    for (int p : cl.particles) w.bodies[p].sleeping = will_sleep;
    return true;
}

// strategies/broad_phase/broad_phase_embree_cluster.cpp:16-123 stepRecursive
inline void step_recursive(World& w, Cluster& cl, int depth = 0) {
    const double start_step = cl.step_size;
    if (w.error) return;
    if (depth > 60) {  // the reference recurses without bound; stop a runaway halving
        w.error = true;
        return;
    }
    const bool ok = pde_step(w, cl);
    if (!ok) {
        double new_min = 0.0;
        for (int p : cl.particles)
            if (!w.bodies[p].is_static)
                new_min = dmax(new_min, (w.bodies[p].last.time + w.bodies[p].cur.time) / 2.0);
        cl.min_current_time = new_min;
        double step_size = 0.0;
        for (int p : cl.particles) {
            Body& B = w.bodies[p];
            if (B.is_static) continue;
            B.fut = B.cur;
            State r;
            if (!state_interpolate(B.cur, B.last, new_min, r)) {
                w.error = true;
                return;
            }
            B.cur = r;
            step_size = B.fut.time - new_min;
        }
        cl.step_size = step_size;
        step_recursive(w, cl, depth + 1);
        std::vector<State> last_final;
        for (int p : cl.particles)
            if (!w.bodies[p].is_static) last_final.push_back(w.bodies[p].cur);
        cl.step_size = start_step / 2.0;
        for (int p : cl.particles) {
            Body& B = w.bodies[p];
            if (B.is_static) continue;
            cl.min_current_time = B.cur.time;
            B.fut = state_extrapolate(B.cur, cl.step_size, B.ii);
        }
        step_recursive(w, cl, depth + 1);
        for (int p : cl.particles)
            if (!w.bodies[p].is_static) cl.min_current_time = w.bodies[p].cur.time;
        step_recursive(w, cl, depth + 1);
        int i = 0;
        for (int p : cl.particles) {
            Body& B = w.bodies[p];
            if (B.is_static) continue;
            B.last = last_final[i++];
            B.last_dt = dmin(B.last_dt, start_step / 2.0);
        }
    }
    cl.step_size = start_step;
}

// strategies/broad_phase/broad_phase_embree_cluster.cpp:125-257 step.
// The "same cluster as last step" reuse (:178-185) relies on
// Cluster::hasAdvanced, which falls off the end without a return value when
// the clusters match (undefined behaviour); it is treated as never matching.
inline void world_step(World& w) {
    for (Body& p : w.bodies) {
        p.last_dt *= 2.0;
        p.last_dt = dmin(p.last_dt, (double)w.opt_dt);
        p.fut = state_extrapolate(p.cur, p.last_dt, p.ii);
    }
    bool bp_ok = true;
    const auto B = broad_phase(w.bodies, w.local_aabb.data(), &bp_ok);
    if (!bp_ok) {
        w.error = true;
        return;
    }
    std::vector<Cluster> cls;
    if (!separate_clusters(B, w.bodies, cls)) {
        w.error = true;
        return;
    }
    double min_final = std::numeric_limits<double>::infinity();
    for (const Cluster& c : cls)
        if (!c.is_static) min_final = dmin(min_final, c.min_current_time + c.step_size);
    double fine_min_final = std::numeric_limits<double>::infinity();
    for (Cluster& c : cls) {
        if (c.min_current_time > min_final) continue;
        if (c.is_static) continue;
        if (c.sleeping) {
            fine_min_final = dmin(fine_min_final, c.min_current_time + (double)w.opt_dt);
            continue;
        }
        const double step = select_time_step(w.T, w.bodies, c, w.opt_dt, &w.stats);
        fine_min_final = dmin(fine_min_final, c.min_current_time + step);
    }
    for (Cluster& c : cls) {
        if (c.min_current_time > fine_min_final) continue;
        if (c.is_static) continue;
        if (c.sleeping) {
            for (int p : c.particles) {  // PDE_strategy.cpp:11-15 staticApply(apply=true)
                Body& B = w.bodies[p];
                B.cur.time = B.cur.time + c.step_size;
                B.fut = B.cur;
            }
        } else {
            step_recursive(w, c);
        }
        if (w.error) return;
    }
}

}  // namespace d2o
