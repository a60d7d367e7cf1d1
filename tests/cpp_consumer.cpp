// A C++17 host of the library through include/d2g.hpp, the layer with the
// reference's names: scenes generated and built from OBJ files, the host
// broad phase, and (when a GPU is present) the narrow phase, CCD, filter and
// cluster separation on the device.  Built and run by test_c_abi_consumer.py;
// prints key=value results on one line.
#include <cstdio>
#include <fstream>
#include <string>

#include "d2g.hpp"

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
            std::printf(" ctx=0 np=%zu ccd=%zu kept=%zu clusters=%zu\n", n_np, n_ccd, n_kept, clusters.size());
        } catch (const delta2_gb300::Error& e) {
            std::printf(" ctx=%d\n", e.code());
        }
    } catch (const delta2_gb300::Error& e) {
        std::printf("FAIL %d %s\n", e.code(), e.what());
        return 1;
    }
    return 0;
}
