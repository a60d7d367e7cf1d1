// Host-side scene set-up: meshes, mass properties, surrogate trees and the
// synthetic benchmark scenes.  None of this is on the hot path; it produces
// the flattened tree and body arrays the kernels read.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace d2g {

// PCG32 (O'Neill, "PCG: A Family of Simple Fast Space-Efficient Statistically
// Good Algorithms for Random Number Generation", 2014): 64-bit LCG state with
// the XSH-RR output permutation; bounded draws by rejection of the low
// 2^32 mod bound values.  The reference seeds one stream (42, 54) in its
// Options and draws surrogate-triangle vertices from it
// (common/cli_options.h:45-49, common/pcg_basic.cpp:42-110).
struct Pcg32 {
    uint64_t state = 0, inc = 1;
    void seed(uint64_t initstate, uint64_t initseq);
    uint32_t next();
    uint32_t bounded(uint32_t bound);
    double uniform();  // [0, 1) with 53 random bits
};

struct Mesh {
    std::vector<double> V;   // [nv][3]
    std::vector<int32_t> F;  // [nf][3]
    int nv() const { return (int)V.size() / 3; }
    int nf() const { return (int)F.size() / 3; }
};

Mesh make_cube(double half_extent);         // common/primitive_geo.cpp:6-31 scaled by half_extent
Mesh make_plane(double width);              // common/primitive_geo.cpp:76-89
Mesh make_open_box(double w, double h);     // floor w x w at z = 0, walls of height h, open top
Mesh make_icosphere(int subdiv, double radius, double noise, Pcg32* rng);
Mesh make_hull(int npts, double radius, Pcg32& rng);  // convex hull of points uniform in a ball

struct MassProps {
    double volume = 0;
    double com[3] = {0, 0, 0};
    double unit_inertia[9] = {0};
    double unit_inertia_inv[9] = {0};
};
MassProps mass_volume(const Mesh& m);                    // closed surface, unit density
MassProps mass_surface(const Mesh& m, double thickness);  // model/mesh.cpp:93-130
void shift_vertices(Mesh& m, const double* c);

struct Tree {
    std::vector<int32_t> nodes;  // [n][4] child_first (local), num_children, is_inner, depth
    std::vector<int32_t> ntris;  // [n]
    std::vector<double> tris;    // [n][8][9]
    std::vector<double> eps;     // [n][8]
    std::vector<double> inner_eps;
    int n() const { return (int)ntris.size(); }
};
// model/surrogate_tree.cpp:39-112 buildSurrogateTreeKMean, drawing from rng.
bool build_tree(const Mesh& m, Pcg32& rng, Tree& out, std::string* err);

// Flattened scene: the layout of d2g_trees / d2g_bodies plus host metadata.
struct Scene {
    std::vector<int32_t> mesh_node_off;
    std::vector<int32_t> nodes, ntris;
    std::vector<double> tris, eps, inner_eps;
    std::vector<int32_t> mesh;
    std::vector<uint8_t> is_static;
    std::vector<double> geo_eps, mu, mass, inv_inertia, last, cur, fut, last_dt, bounding_radius;
    std::vector<int32_t> sleep_steps;
    std::vector<uint8_t> sleeping;
    std::vector<float> local_aabb;  // [n][6]
    std::vector<int32_t> mesh_ntris;
    float opt_dt = 0.01f;
    double gravity_z = -9.8;
    int n_bodies() const { return (int)mesh.size(); }
};

struct SceneOpts {
    int config = 1;          // 1: cubes, 2: convex hulls, 3: mixed shapes, 5: noisy icospheres in an open box
    int nx = 0, ny = 0, nz = 0;
    double spacing = 0;
    double speed_sigma = -1;  // per-axis initial velocity std-dev
    uint64_t seed = 0;
    float dt = 0;
    double gravity_z = -9.8;
    double mu = 0;
    int hull_points = 64;
    int count = 0;  // > 0: bodies only in the first `count` grid cells
    std::string tree_file;  // non-empty: load the trees from this file, or build and save them there
};
bool make_scene(const SceneOpts& o, Scene& s, std::string* err);

// A scene of the caller's meshes and bodies (d2g_scene_create and friends).
struct SceneBuilder {
    Scene s;
    std::vector<Mesh> meshes;
    std::vector<MassProps> mass;
    bool finished = false;
};
// Returns the mesh id (and the centre of mass it was centred at), or -1.
int builder_add_mesh(SceneBuilder& b, const double* V, int nv, const int32_t* F, int nf, bool surface, double* com,
                     std::string* err);
bool builder_add_body(SceneBuilder& b, int mesh, bool is_static, double density, double geo_eps, double mu,
                      const double* x, const double* q, const double* v, std::string* err);
bool builder_finish(SceneBuilder& b, std::string* err);
// Vertices [n][3] and triangles [m][3] of a Wavefront OBJ file (d2g_obj.cpp).
bool read_obj(const char* path, std::vector<double>& V, std::vector<int32_t>& F, std::string* err);

// Flattened trees of a scene's meshes and the versioned binary file they are
// saved to (d2g_treefile.cpp).
struct TreeSet {
    std::vector<int32_t> mesh_node_off, mesh_ntris, nodes, ntris;
    std::vector<double> tris, eps, inner_eps;
};
bool save_trees(const TreeSet& t, const char* path, std::string* err);
bool load_trees(const char* path, TreeSet& t, std::string* err);

// Adds one mesh (tree built with rng) and returns its mesh id.
int scene_add_mesh(Scene& s, const Mesh& m, Pcg32& tree_rng, std::string* err);
// Adds a built tree of a mesh with n_faces triangles; returns its mesh id.
int scene_add_tree(Scene& s, const Tree& t, int n_faces);

}  // namespace d2g
