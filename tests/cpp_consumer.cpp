// A C++17 host of the library through include/d2g.hpp, the layer with the
// reference's names: scenes generated and built from OBJ files, the host
// broad phase, and (when a GPU is present) the narrow phase, the per-level
// bucket comparison, CCD, filter, cluster separation and solve on the
// device.  Built and run by test_c_abi_consumer.py (CPU) and
// test_gpu_cpp_layer.py (GPU); prints key=value results on one line and, with
// a GPU, writes the device results as raw little-endian arrays into the
// output folder for the GPU test to compare with the oracle.
#include <cstdio>
#include <fstream>
#include <string>

#include "d2g.hpp"

namespace {

void write_contacts(const std::string& path, const std::vector<delta2_gb300::Contact>& cs) {
    std::vector<double> rec(D2G_CONTACT_LEN * (cs.size() + 1));
    for (size_t i = 0; i < cs.size(); i++) cs[i].toRecord(rec.data() + D2G_CONTACT_LEN * i);
    std::ofstream f(path, std::ios::binary);
    f.write((const char*)rec.data(), (std::streamsize)(sizeof(double) * D2G_CONTACT_LEN * cs.size()));
}

void write_i32(const std::string& path, const std::vector<int32_t>& v) {
    std::ofstream f(path, std::ios::binary);
    f.write((const char*)v.data(), (std::streamsize)(sizeof(int32_t) * v.size()));
}

// Device half: a 2x2x2 cube scene (spacing 1.12 m, seed 1, speed 3 m/s per
// axis) through every device method of the C++ layer.
void device_run(const std::string& dir) {
    d2g_scene_opts o{};
    o.config = 1;
    o.nx = o.ny = o.nz = 2;
    o.spacing = 1.12;
    o.speed_sigma = 3.0;
    o.seed = 1;
    o.gravity_z = -9.8;
    const delta2_gb300::Scene sc(o);
    const auto pairs = sc.broadPhase();
    delta2_gb300::Context ctx(0);
    ctx.setScene(sc);
    // compareTreesFull per pair, then filterContacts per pair
    const auto np = ctx.compareTreesFull(pairs);
    std::vector<delta2_gb300::Contact> all, kept_all;
    std::vector<int32_t> off{0}, kept_off{0};
    for (const auto& c : np) {
        all.insert(all.end(), c.begin(), c.end());
        off.push_back((int32_t)all.size());
        const auto k = ctx.filterContacts(c);
        kept_all.insert(kept_all.end(), k.begin(), k.end());
        kept_off.push_back((int32_t)kept_all.size());
    }
    write_contacts(dir + "/np.bin", all);
    write_i32(dir + "/np_off.bin", off);
    write_contacts(dir + "/kept.bin", kept_all);
    write_i32(dir + "/kept_off.bin", kept_off);
    // the first level of pair 0's traversal through the strategy interface
    const delta2_gb300::SceneView v = sc.view();
    const int32_t a = pairs[0][0], b = pairs[0][1];
    std::vector<delta2_gb300::Pair> level{{v.trees.mesh_node_off[v.bodies.mesh[a]], v.trees.mesh_node_off[v.bodies.mesh[b]]}};
    std::vector<delta2_gb300::Contact> hits;
    std::vector<int> used;
    ctx.findContactsBucketComparison(a, b, level, hits, used);
    write_contacts(dir + "/bucket.bin", hits);
    write_i32(dir + "/bucket_used.bin", std::vector<int32_t>(used.begin(), used.end()));
    // clusters (rolls back to each cluster's minimum current time: a no-op
    // here, every body starts at the same time) and the solve of the first
    // cluster with its interactions' filtered contacts
    const auto clusters = ctx.separateCollisionClusters(sc, pairs);
    const auto& cl = clusters.at(0);
    delta2_gb300::ClusterHits ch;
    ch.particles = cl.particles;
    ch.step = (double)v.opt_dt;
    for (const auto& it : cl.interactions)
        for (size_t p = 0; p < pairs.size(); p++)
            if (pairs[p] == it)
                for (int32_t q = kept_off[p]; q < kept_off[p + 1]; q++) ch.hits.push_back(kept_all[q]);
    const bool accepted = ctx.solve(ch);
    ctx.getBodies(sc);
    {
        std::ofstream f(dir + "/fut.bin", std::ios::binary);
        f.write((const char*)v.bodies.fut, (std::streamsize)(sizeof(double) * D2G_STATE_LEN * v.bodies.n));
    }
    write_i32(dir + "/cluster0.bin", cl.particles);
    // compareTreesFullContinuous over 0.05 s per pair (projects the futures again)
    ctx.setScene(sc);
    const auto ccd = ctx.compareTreesFullContinuous(pairs, std::vector<double>(pairs.size(), 0.05));
    std::vector<delta2_gb300::Contact> call;
    std::vector<int32_t> coff{0};
    for (const auto& c : ccd) {
        call.insert(call.end(), c.begin(), c.end());
        coff.push_back((int32_t)call.size());
    }
    write_contacts(dir + "/ccd.bin", call);
    write_i32(dir + "/ccd_off.bin", coff);
    std::printf(" dev_pairs=%zu dev_np=%zu dev_kept=%zu dev_bucket=%zu dev_clusters=%zu dev_hits=%zu dev_accepted=%d "
                "dev_ccd=%zu",
                pairs.size(), all.size(), kept_all.size(), hits.size(), clusters.size(), ch.hits.size(),
                accepted ? 1 : 0, call.size());
}

}  // namespace

int main(int argc, char** argv) {
    const std::string dir = argc > 1 ? argv[1] : ".";
    {
        std::ofstream cube(dir + "/cube.obj");
        cube << "v 0.5 0.5 0.5\nv 0.5 0.5 -0.5\nv 0.5 -0.5 0.5\nv 0.5 -0.5 -0.5\n"
                "v -0.5 0.5 0.5\nv -0.5 0.5 -0.5\nv -0.5 -0.5 0.5\nv -0.5 -0.5 -0.5\n"
                "f 1 3 2\nf 2 3 4\nf 3 7 4\nf 4 7 8\nf 5 6 7\nf 6 8 7\nf 5 1 2\nf 5 2 6\nf 1 5 7\nf 1 7 3\n"
                "f 4 8 2\nf 8 6 2\n";
        std::ofstream plane(dir + "/plane.obj");
        plane << "v 50 50 0\nv 50 -50 0\nv -50 50 0\nv -50 -50 0\nf 1 3 2\nf 2 3 4\n";
    }
    try {
        d2g_scene_opts o{};
        o.config = 1;
        o.speed_sigma = -1.0;
        const delta2_gb300::Scene gen(o);
        const auto gen_pairs = gen.broadPhase();

        delta2_gb300::SceneBuilder b(1.0f / 240.0f, -9.8);
        const auto plane = b.addObj(dir + "/plane.obj", true);
        const auto cube = b.addObj(dir + "/cube.obj");
        b.addBody(plane.first, true, {0, 0, 0});
        for (int k = 0; k < 3; k++) b.addBody(cube.first, false, {1.5 * k, 0.0, 0.6}, {1, 0, 0, 0}, {0, 0, -1});
        const delta2_gb300::Scene own = b.finish();
        const auto own_pairs = own.broadPhase();
        const delta2_gb300::SceneView v = own.view();
        std::printf("gen_bodies=%d gen_pairs=%zu own_bodies=%d own_nodes=%d own_pairs=%zu", gen.view().bodies.n,
                    gen_pairs.size(), v.bodies.n, v.trees.mesh_node_off[v.trees.n_meshes], own_pairs.size());
        try {
            delta2_gb300::Context ctx(0);
            ctx.setScene(gen);
            const auto np = ctx.compareTreesFull(gen_pairs);
            const auto ccd = ctx.compareTreesFullContinuous(gen_pairs, std::vector<double>(gen_pairs.size(), 0.05));
            size_t n_np = 0, n_ccd = 0, n_kept = 0;
            for (size_t i = 0; i < np.size(); i++) {
                n_np += np[i].size();
                n_ccd += ccd[i].size();
                n_kept += ctx.filterContacts(np[i]).size();
            }
            const auto clusters = ctx.separateCollisionClusters(gen, gen_pairs);
            std::printf(" ctx=0 np=%zu ccd=%zu kept=%zu clusters=%zu", n_np, n_ccd, n_kept, clusters.size());
            device_run(dir);
            std::printf("\n");
        } catch (const delta2_gb300::Error& e) {
            std::printf(" ctx=%d\n", e.code());
        }
    } catch (const delta2_gb300::Error& e) {
        std::printf("FAIL %d %s\n", e.code(), e.what());
        return 1;
    }
    return 0;
}
