/* A plain C11 host of the C ABI: the scene builder, the tree file, the
 * broad phase on the host, and context creation (which must report the
 * missing device when there is none).  Built and run by
 * test_c_abi_consumer.py; prints one line of results. */
#include <stdio.h>
#include <string.h>

#include "d2g.h"

static const double cube_v[8][3] = {{0.5, 0.5, 0.5},   {0.5, 0.5, -0.5},   {0.5, -0.5, 0.5},   {0.5, -0.5, -0.5},
                                    {-0.5, 0.5, 0.5},  {-0.5, 0.5, -0.5},  {-0.5, -0.5, 0.5},  {-0.5, -0.5, -0.5}};
static const int32_t cube_f[12][3] = {{0, 2, 1}, {1, 2, 3}, {2, 6, 3}, {3, 6, 7}, {4, 5, 6}, {5, 7, 6},
                                      {4, 0, 1}, {4, 1, 5}, {0, 4, 6}, {0, 6, 2}, {3, 7, 1}, {7, 5, 1}};
static const double plane_v[4][3] = {{50, 50, 0}, {50, -50, 0}, {-50, 50, 0}, {-50, -50, 0}};
static const int32_t plane_f[2][3] = {{0, 2, 1}, {1, 2, 3}};

#define CHECK(call)                                                            \
    do {                                                                       \
        int rc_ = (call);                                                      \
        if (rc_ != D2G_OK) {                                                   \
            printf("FAIL %s: %d %s\n", #call, rc_, d2g_last_error());          \
            return 1;                                                          \
        }                                                                      \
    } while (0)

int main(int argc, char** argv) {
    const char* tree_path = argc > 1 ? argv[1] : "c_consumer.trees";
    d2g_scene* sc = NULL;
    double com[3];
    int32_t plane = -1, cube = -1;
    const double q[4] = {1, 0, 0, 0}, zero[3] = {0, 0, 0};
    d2g_trees trees, loaded;
    d2g_bodies bodies;
    const float* aabb = NULL;
    float dt = 0.0f;
    double g = 0.0;
    d2g_tree_file* tf = NULL;
    int32_t pairs[64], n_pairs = 0, k, i;
    d2g_ctx* ctx = NULL;
    int rc;

    CHECK(d2g_scene_create(1.0f / 240.0f, -9.8, &sc));
    CHECK(d2g_scene_add_mesh(sc, &plane_v[0][0], 4, &plane_f[0][0], 2, 1, com, &plane));
    CHECK(d2g_scene_add_mesh(sc, &cube_v[0][0], 8, &cube_f[0][0], 12, 0, com, &cube));
    CHECK(d2g_scene_add_body(sc, plane, 1, 1000.0, 0.01, 0.5, zero, q, zero));
    for (k = 0; k < 3; k++) {
        const double x[3] = {1.5 * k, 0.0, 0.6}, v[3] = {0.0, 0.0, -1.0};
        CHECK(d2g_scene_add_body(sc, cube, 0, 1000.0, 0.01, 0.5, x, q, v));
    }
    CHECK(d2g_scene_finish(sc));
    CHECK(d2g_scene_view(sc, &trees, &bodies, &aabb, &dt, &g));
    CHECK(d2g_trees_save(&trees, tree_path));
    CHECK(d2g_trees_load(tree_path, &tf));
    CHECK(d2g_tree_file_view(tf, &loaded));
    for (i = 0; i <= trees.n_meshes; i++)
        if (loaded.mesh_node_off[i] != trees.mesh_node_off[i]) {
            printf("FAIL tree file offsets\n");
            return 1;
        }
    if (memcmp(loaded.tris, trees.tris, sizeof(double) * 72 * (size_t)trees.mesh_node_off[trees.n_meshes]) != 0) {
        printf("FAIL tree file triangles\n");
        return 1;
    }
    d2g_tree_file_free(tf);
    CHECK(d2g_broad_phase(&bodies, aabb, pairs, 32, &n_pairs));
    rc = d2g_ctx_create(0, &ctx);
    if (rc == D2G_OK) d2g_ctx_destroy(ctx);
    printf("ok meshes=%d nodes=%d bodies=%d mass1=%.17g pairs=%d ctx=%d\n", trees.n_meshes,
           trees.mesh_node_off[trees.n_meshes], bodies.n, bodies.mass[1], n_pairs, rc);
    d2g_scene_free(sc);
    return 0;
}
