/*
 * d2g.h — C ABI of the GB300 contact hot path (delta2_gb300).
 *
 * The reference (Peter-Noble/Delta2) has no C ABI: its hot path is reached
 * through C++ virtual strategies and free functions.  Each entry point below
 * names the reference interface it replaces (file:line within the reference
 * project).  Conventions:
 *   - plain pointers and sizes, no C++ or torch types;
 *   - every call returns an int status: 0 = ok, > 0 = recoverable
 *     (D2G_SOLVE_FAILED, D2G_CAPACITY, D2G_SPIN_LIMIT), < 0 = fatal;
 *     d2g_last_error() gives the message of the calling thread's last error;
 *   - "host" entry points take host buffers and copy in and out inside the
 *     call; "_device" entry points take pointers in the GPU's memory;
 *   - one host thread per context; all work is ordered on the context's stream.
 *
 * Records shared by all entry points:
 *   body state (14 doubles): time, qw qx qy qz, L(3), x(3), v(3)
 *   contact (14 doubles): A(3) B(3) eps_a eps_b eps_inner_a eps_inner_b toc pa pb 0
 *     (collision_detection/contact.h:9-28 Contact and :73-83 ContinuousContact;
 *      pa/pb are body indices stored as doubles)
 *   tree node (4 int32): child_first (global node index, -1 for leaves),
 *     num_children, is_inner, depth; node i owns bucket i (<= 8 triangles of
 *     9 doubles, eps[8], inner_eps[8])  (model/surrogate_components.h:11-88)
 */
#ifndef D2G_H
#define D2G_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    D2G_OK = 0,
    D2G_SOLVE_FAILED = 1, /* SequentialImpulses::solve returned false */
    D2G_CAPACITY = 2,     /* output larger than the caller's buffer; counts still written */
    D2G_SPIN_LIMIT = 3,   /* a bounded device wait gave up */
    D2G_ERR_INVALID = -1,
    D2G_ERR_CUDA = -2,
    D2G_ERR_NO_DEVICE = -3,
    D2G_ERR_STATE = -4
};

#define D2G_STATE_LEN 14
#define D2G_CONTACT_LEN 14

/* Surrogate trees of all meshes, concatenated (model/surrogate_tree.h:15-29). */
typedef struct d2g_trees {
    int32_t n_meshes;
    const int32_t* mesh_node_off; /* [n_meshes+1] first node of each mesh */
    const int32_t* nodes;         /* [N][4] */
    const int32_t* ntris;         /* [N] */
    const double* tris;           /* [N][8][9] */
    const double* eps;            /* [N][8] */
    const double* inner_eps;      /* [N][8] */
} d2g_trees;

/* Bodies (model/particle.h:9-64); index == reference Particle::id. */
typedef struct d2g_bodies {
    int32_t n;
    const int32_t* mesh;
    const uint8_t* is_static;
    const double* geo_eps;
    const double* mu;
    const double* mass;
    const double* inv_inertia; /* [n][9] body-frame inverse inertia, row major */
    double* last;              /* [n][14] */
    double* cur;               /* [n][14] */
    double* fut;               /* [n][14] */
    double* last_dt;           /* [n] */
    int32_t* sleep_steps;      /* [n] */
    uint8_t* sleeping;         /* [n] */
    const double* bounding_radius;
} d2g_bodies;

/* ------------------------------------------------------------ errors ---- */
const char* d2g_last_error(void);
const char* d2g_version(void);

/* --------------------------------------------------- scene set-up (host) --
 * Synthetic scenes of the benchmark configurations and their surrogate trees
 * (the reference builds scenes in src/runner/main.cpp:65-126 and trees in
 * model/surrogate_tree.cpp:39-112).  No GPU is used. */
typedef struct d2g_scene_opts {
    int32_t config;     /* 1 cubes, 2 convex hulls, 3 mixed shapes, 5 noisy icospheres */
    int32_t nx, ny, nz; /* grid size, 0 = the configuration's default */
    double spacing;     /* 0 = default */
    double speed_sigma; /* initial velocity std-dev per axis; < 0 = default */
    uint64_t seed;
    float dt;           /* 0 = default */
    double gravity_z;
    double mu;          /* 0 = default */
    int32_t hull_points;
    int32_t count;      /* > 0: only the first `count` grid cells get a body */
    const char* tree_file; /* non-null: load the trees from this tree file when it
                              exists (d2g_trees_load's format, checked against the
                              meshes), else build them and save them there */
} d2g_scene_opts;

/* Tree files (no reference counterpart: the reference builds its trees when
 * it loads a mesh).  A versioned little-endian binary file of d2g_trees'
 * arrays plus each mesh's triangle count (the sum of its leaf buckets), with
 * a checksum; loading checks the structure (offsets, child links inside
 * their mesh, at most 8 triangles per bucket). */
typedef struct d2g_tree_file d2g_tree_file;
int d2g_trees_save(const d2g_trees* trees, const char* path);
int d2g_trees_load(const char* path, d2g_tree_file** out);
/* Pointers into the loaded file's storage (valid until d2g_tree_file_free). */
int d2g_tree_file_view(d2g_tree_file* f, d2g_trees* trees);
void d2g_tree_file_free(d2g_tree_file* f);

typedef struct d2g_scene d2g_scene;
int d2g_scene_make(const d2g_scene_opts* opts, d2g_scene** out);
void d2g_scene_free(d2g_scene* s);
/* Pointers into the scene's own storage (valid until d2g_scene_free). */
int d2g_scene_view(d2g_scene* s, d2g_trees* trees, d2g_bodies* bodies, const float** local_aabb, float* opt_dt,
                   double* gravity_z);

/* Scenes of the caller's meshes and bodies: the reference's mesh loading
 * and particle set-up (model/mesh.cpp:9-130: meshes centred at their centre
 * of mass, volume mass model of a closed surface or, with surface != 0, the
 * thin-shell surface model used for static planes; model/particle.cpp:7-40).
 * d2g_scene_add_mesh returns the mesh id and the centre of mass it centred
 * the mesh at (world position = body position + rotated local vertex).
 * d2g_scene_finish builds the trees (one PCG32 stream seeded (42, 54), in
 * mesh order); d2g_scene_view then works as for d2g_scene_make. */
int d2g_scene_create(float dt, double gravity_z, d2g_scene** out);
int d2g_scene_add_mesh(d2g_scene* s, const double* vertices, int32_t n_vertices, const int32_t* faces,
                       int32_t n_faces, int32_t surface, double* com, int32_t* mesh_id);
/* Reads a Wavefront OBJ file (v records; f records of three or more vertex
 * references, the first field of each v/vt/vn form, negative references
 * counting back from the last vertex read; polygons split into fans) and
 * adds it as d2g_scene_add_mesh does; the reference reads its meshes with
 * igl::readOBJ (model/mesh.cpp:9-21). */
int d2g_scene_add_obj(d2g_scene* s, const char* path, int32_t surface, double* com, int32_t* mesh_id);
int d2g_scene_add_body(d2g_scene* s, int32_t mesh_id, int32_t is_static, double density, double geo_eps, double mu,
                       const double* position, const double* quaternion, const double* velocity);
int d2g_scene_finish(d2g_scene* s);
/* Build one mesh's surrogate tree from a triangle mesh, drawing from the PCG32
 * stream (state, inc) in rng[2] (updated).  Sizes first, then a second call
 * with buffers: nodes [n][4] (child_first local to this mesh), ntris, tris
 * [n][72], eps [n][8], inner_eps [n][8].  Replaces SurrogateTree(V, F, opt). */
int d2g_tree_build(const double* V, int32_t nv, const int32_t* F, int32_t nf, uint64_t* rng, int32_t* n_nodes,
                   int32_t* nodes, int32_t* ntris, double* tris, double* eps, double* inner_eps, int32_t capacity);

/* Broad phase (host): body pairs i < j, not both static, whose float bounds
 * overlap (the mesh box through the float transform for static bodies, the
 * bounding-sphere box at last/current/future positions for moving ones, grown
 * by geo_eps) and whose swept bounding spheres meet within max(last_dt).
 * Replaces broadPhaseEmbree(ParticleHandler&)
 * (collision_detection/broad_phase_embree.cpp:87-116, 186-238, 266-289);
 * pairs come in ascending (i, j).  pairs may be NULL to count only. */
int d2g_broad_phase(const d2g_bodies* bodies, const float* local_aabb, int32_t* pairs, int32_t capacity,
                    int32_t* n_pairs);

/* ------------------------------------------------------------ context ---- */
typedef struct d2g_ctx d2g_ctx;
typedef struct d2g_mlp d2g_mlp; /* the learned proposal's network (d2g_mlp_create, below) */
int d2g_ctx_create(int32_t device, d2g_ctx** out);
void d2g_ctx_destroy(d2g_ctx* ctx);
/* The context's CUDA stream (cudaStream_t) for ordering caller work. */
int d2g_ctx_stream(d2g_ctx* ctx, void** stream);
int d2g_ctx_sync(d2g_ctx* ctx);
/* Copy trees / bodies into HBM (replaces the reference's in-memory
 * MeshData / ParticleHandler ownership). */
int d2g_ctx_set_trees(d2g_ctx* ctx, const d2g_trees* trees);
int d2g_ctx_set_bodies(d2g_ctx* ctx, const d2g_bodies* bodies);
/* Independent scenes batched in one context (no counterpart in the reference,
 * whose process steps one world): scene index of every body.  Bodies of
 * different scenes never pair, and the stepper schedules every scene as its
 * own world (BroadPhaseEmbreeCluster::step per scene), so each scene evolves
 * exactly as it would alone.  d2g_ctx_set_bodies resets all bodies to scene 0. */
int d2g_ctx_set_scenes(d2g_ctx* ctx, const int32_t* scene_of_body);
/* Copy the device body states (last/cur/fut, last_dt, sleep_steps, sleeping) back. */
int d2g_ctx_get_bodies(d2g_ctx* ctx, d2g_bodies* bodies);

/* Mass properties of many meshes on the device (model/mesh.cpp:53-130,
 * model/inertia.cpp:20-84, for large mesh sets): mesh m has vertices
 * V[mesh_vertex_off[m] .. +1) and faces F[mesh_face_off[m] .. +1) (vertex
 * indices local to the mesh); surface[m] != 0 takes the thin-shell model of
 * the given thickness (as static planes use), else the closed-surface volume
 * model (the reference's tetgen tetrahedralisation replaced by the faces'
 * tetrahedra with the origin).  out [n_meshes][22]: volume, centre of mass
 * (3), unit-density inertia tensor about it (9, row major), its inverse (9);
 * the same bits as the host scene set-up gives.  surface may be NULL. */
int d2g_mass_properties(d2g_ctx* ctx, const double* V, int32_t n_vertices, const int32_t* F, int32_t n_faces,
                        const int32_t* mesh_vertex_off, const int32_t* mesh_face_off, const uint8_t* surface,
                        int32_t n_meshes, double thickness, double* out);

/* Mixed precision (no reference counterpart): with enable != 0 (the
 * default) the discrete narrow phase and the CCD first bound every
 * primitive test in FP32 (bounding spheres and box gaps, with a margin far
 * above FP32 and FP64 rounding) and run the FP64 test only where a hit is
 * possible; with 0 every test runs in FP64.  Results are identical. */
int d2g_ctx_set_fp32_bounds(d2g_ctx* ctx, int32_t enable);
/* Conservative-advancement certificates (no reference counterpart): with
 * enable != 0 (the default) an edge-edge CCD test whose distance at a Newton
 * iterate, less the largest relative endpoint displacement times the time
 * still ahead, stays above the search distance (and whose distances so far
 * do too) is cut there: no later iterate can come closer, so it cannot hit and
 * is recorded as no contact, as the reference's min over its iterates would
 * leave it.  Results are identical; 0 runs every test to the end. */
int d2g_ctx_set_ccd_certificates(d2g_ctx* ctx, int32_t enable);
/* Learned proposal in the CCD (no reference counterpart): with a network of
 * this context (d2g_mlp_create), every CCD call (compareTreesFullContinuous,
 * the time-step selection, the stepper) computes each pair query's 20
 * features, runs the network, and for the queries it predicts contact-free
 * (hit probability below `threshold`) tries a root certificate: a proof,
 * over the linear motion the reference's CCD assumes, that no slot of the
 * root node pair can come within the search distance.  Proven queries are
 * skipped (they would yield no contact); any other query runs the exact
 * traversal, so results are unchanged.  threshold 1 sends every query to
 * the certificate (the certificate without the network); mlp NULL turns the
 * proposal off (the default).  The counters of d2g_ctx_ccd_stats report its
 * effect.  Destroying the network turns the proposal off. */
int d2g_ctx_set_ccd_proposal(d2g_ctx* ctx, d2g_mlp* mlp, float threshold);
/* The 20 proposal features of n pair queries (pairs [n][2], max_time [n]) over
 * the context's device bodies, as the proposal computes them (FP64, stored as
 * FP32; layout as d2g_mlp_predict's input): features [n][20]. */
int d2g_ccd_features(d2g_ctx* ctx, const int32_t* pairs, const double* max_time, int32_t n_pairs, float* features);
/* Separation witnesses (the temporal coherence of the reference's
 * collision_detection/contact_state.cpp:14-150 and full_tree_comparison.cpp:
 * 7-198, which are off its live path): with enable != 0 every CCD call keeps,
 * per (body pair, node pair) of the traversal's soup stage that had no hit,
 * an axis in the first body's frame that proved the pair separated, and at
 * later calls skips a node pair whose axis still proves every slot clear
 * over the query's motion (the same proof as the learned proposal's root
 * certificate).  A skipped node pair has no hit, so results are unchanged.
 * Off by default; the table takes 32 MiB of device memory once enabled. */
int d2g_ctx_set_ccd_witnesses(d2g_ctx* ctx, int32_t enable);
/* CCD counters since the context was created or last reset (reset != 0
 * clears them after reading), n of D2G_CCD_STATS entries:
 *   0 edge-edge tests cut by the certificates, 1 Newton iterations they did
 *   not run (of the reference's 10 per test), 2 pair queries the learned
 *   proposal predicted to have no contact, 3 of those the root certificate
 *   proved contact-free (skipped), 4 of those it could not prove (misses,
 *   traversed as usual), 5 pair queries seen by the proposal, 6 node pairs
 *   skipped by their separation witness, 7 witnesses written. */
#define D2G_CCD_STATS 8
int d2g_ctx_ccd_stats(d2g_ctx* ctx, int32_t reset, int64_t* stats, int32_t n);
/* Launch-shape settings (no reference counterpart).  They change only how
 * the work is spread over the GPU; every setting gives identical results.
 *   D2G_TUNE_EE_FIRST_ITERS (default 2, 0..10): Newton iterations an
 *     edge-edge CCD test runs on one lane before the tests still running
 *     continue on four lanes each.
 *   D2G_TUNE_GRID_MIN_PARTS (default 512, >= 0): a cluster with at least
 *     128 contacts and more parts than this is solved by a cooperative grid
 *     over the SMs, when at most 8 clusters of the solve call qualify.
 *   D2G_TUNE_SOLVE_LANES (default 0; 0, 4 or 16): lanes per contact in the
 *     solve's normal-impulse waves; 0 takes sixteen for a wave narrow enough
 *     that its warps each have an SM sub-partition to themselves, else four.
 *   D2G_TUNE_SPIN_LIMIT (default 33554432, >= 1): polls a block of the
 *     cooperative-grid solve makes at a grid barrier before it gives up
 *     (several seconds at the default); a call whose barrier gave up returns
 *     D2G_SPIN_LIMIT and leaves that solve's future states unspecified, and
 *     the context stays usable.  Unlike the settings above, a limit small
 *     enough to be reached changes the outcome: it exists to bound the wait.
 *   D2G_TUNE_GRID_CONTACTS (default 16, >= 1): a cooperative-grid solve
 *     takes one block per this many contacts of its cluster (at least 8
 *     blocks, at most one per SM): fewer blocks make each grid barrier
 *     cheaper, more spread a wide wave over more SMs.
 *   D2G_TUNE_SOLVE_CLUSTER (default 0; 0, 1, 2, 4, 8 or 16): a cluster with
 *     at least 32 contacts that does not take a grid is solved by a
 *     thread-block cluster of this many blocks (waves between them on the
 *     hardware cluster barrier); 0 takes the largest size at which every
 *     such cluster of the call is resident at once (one block each when
 *     none is), 1 solves them with one block each.
 * delta2_gb300/autotune.py measures candidate values on a workload and
 * writes them to a file that the Python layer applies. */
#define D2G_TUNE_EE_FIRST_ITERS 0
#define D2G_TUNE_GRID_MIN_PARTS 1
#define D2G_TUNE_SOLVE_LANES 2
#define D2G_TUNE_SPIN_LIMIT 3
#define D2G_TUNE_GRID_CONTACTS 4
#define D2G_TUNE_SOLVE_CLUSTER 5
#define D2G_TUNE_KEYS 6
int d2g_ctx_set_tuning(d2g_ctx* ctx, int32_t key, int32_t value);
int d2g_ctx_get_tuning(d2g_ctx* ctx, int32_t key, int32_t* value);
/* How the last solve call (d2g_solve_clusters or a stepper round) spread its
 * clusters (no reference counterpart; diagnostics): 0 clusters solved by one
 * block, 1 by thread-block clusters, 2 by cooperative grids, 3 the
 * thread-block clusters' blocks. */
#define D2G_SOLVE_LAYOUT 4
int d2g_ctx_solve_layout(d2g_ctx* ctx, int32_t* layout, int32_t n);
/* Memory cap (no reference counterpart): the bytes one level of a tree
 * traversal (discrete narrow phase or CCD) may use for its buffers; 0 (the
 * default) means a sixth of the device memory.  A call whose level would
 * exceed it traverses its body pairs in chunks (halving a chunk that still
 * exceeds it), with identical results.  The contact records themselves are
 * output and are not capped. */
int d2g_ctx_set_level_budget(d2g_ctx* ctx, int64_t bytes);
/* Instrumentation (no reference counterpart): the number of kernels this
 * library launched on the context, and, with profiling on, CUDA-event times
 * of the dominant kernels: kind 0 swept-box filter, 1 point-triangle CCD
 * tests, 2 edge-edge CCD tests, 3 discrete triangle distance,
 * 4 sequential-impulse solve.
 * Enabling (or disabling) profiling resets the totals. */
int d2g_ctx_launches(d2g_ctx* ctx, int64_t* launches);
int d2g_ctx_set_profiling(d2g_ctx* ctx, int32_t enable);
int d2g_ctx_profile(d2g_ctx* ctx, int32_t kind, double* ms, int64_t* launches, int64_t* items);

/* ------------------------------------------------- discrete narrow phase --
 * compareTreesFull<double,8,8> for each body pair (a, b), using the bodies'
 * current device future states (collision_detection/full_tree_comparison.h:
 * 13-67 with ContactDetectionComparison, comparison_dist.h:205-240).
 * pairs [n][2]; contacts [capacity][14]; offsets [n+1].  Contacts of pair i
 * are contacts[offsets[i] .. offsets[i+1]) in the reference's order.
 * counters (optional, 4 int64): node pairs, triangle pairs, leaf pairs, levels.
 * Returns D2G_CAPACITY when the total exceeds capacity (offsets still valid). */
int d2g_compare_trees_full(d2g_ctx* ctx, const int32_t* pairs, int32_t n_pairs, double* contacts,
                           int32_t capacity, int32_t* offsets, int64_t* counters);

/* findContactsBucketComparison for one body pair and one level of its
 * traversal: the reference's discrete detection strategy interface
 * (strategies/contact_detection/contact_detection_strategy.h:11, implemented
 * by ContactDetectionComparison, contact_detection_comparison.cpp:12-14 ->
 * comparison_dist.h:205-240), which compareTreesFull calls once per level
 * (full_tree_comparison.h:25).  node_pairs [n][2]: global node ids (a node of
 * body_a's tree, a node of body_b's tree), the reference's DeferredCompare
 * list.  Every (triangle of a's bucket, triangle of b's bucket) slot closer
 * than float(geo_eps_a + geo_eps_b) + eps_i + eps_j at the bodies' device
 * future states is a hit: hits [capacity][14] in the reference's order (node
 * pair, a's triangle, b's triangle); pair_used [n] receives the reference's
 * cumulative pair_used_out (hits of node pairs 0..i).  D2G_CAPACITY when the
 * hits exceed capacity (pair_used still written). */
int d2g_find_contacts_bucket_comparison(d2g_ctx* ctx, int32_t body_a, int32_t body_b, const int32_t* node_pairs,
                                        int32_t n_node_pairs, double* hits, int32_t capacity, int32_t* pair_used);

/* ------------------------------------------- continuous collision detection
 * compareTreesFullContinuous<double,8,8> for each pair over its max_time
 * (collision_detection/full_tree_comparison.h:69-219).  Each pair first
 * projects both bodies' futures from their current states over max_time; the
 * device future state of a body afterwards is the projection of the LAST pair
 * (in array order) that contains it, as the reference's sequential calls
 * leave it.  The reference's min_time_out is not produced (its live caller,
 * separate_clusters.cpp:494, ignores it). */
int d2g_compare_trees_full_continuous(d2g_ctx* ctx, const int32_t* pairs, const double* max_time, int32_t n_pairs,
                                      double* contacts, int32_t capacity, int32_t* offsets, int64_t* counters);
/* Same with pairs and max_time already in HBM; results stay on the device:
 * *d_contacts / *d_offsets point into context-owned buffers valid until the
 * next call.  *n_contacts receives the total. */
int d2g_compare_trees_full_continuous_device(d2g_ctx* ctx, const int32_t* d_pairs, const double* d_max_time,
                                             int32_t n_pairs, int32_t* n_contacts, const double** d_contacts,
                                             const int32_t** d_offsets, int64_t* counters);

/* ------------------------------------------ broad phase on the device --
 * broadPhaseEmbree(ParticleHandler&) over the context's device bodies
 * (collision_detection/broad_phase_embree.cpp:87-116, 186-238, 266-289): the
 * same pair set as d2g_broad_phase (float boxes, inclusive overlap, the
 * swept-sphere filter within max(last_dt)), ascending (i, j), found by a
 * sort-and-sweep on the GPU.  local_aabb: [n][6] host floats (Mesh::getAABB).
 * D2G_ERR_STATE on an invalid state interpolation (the reference throws). */
int d2g_ctx_broad_phase(d2g_ctx* ctx, const float* local_aabb, int32_t* pairs, int32_t capacity, int32_t* n_pairs);
/* separateCollisionClusters (collision_detection/separate_clusters.cpp:
 * 355-459) on the device: clusters are the components of the moving-moving
 * pairs, numbered by their smallest body index (igl's labelling taken as
 * breadth-first from the lowest index); a cluster's particles are its moving
 * members ascending, then the static bodies it interacts with in order of
 * first interaction; its interactions are the pairs in the given order.  The
 * moving bodies' current states are rolled back to their cluster's minimum
 * current time, as the reference does.  Clusters without a moving body are
 * dropped.  Output sizes: particle_off and pair_off [n_bodies + 1], particles
 * [n_bodies + n_pairs], cluster_pairs [2 n_pairs], min_current_time, step
 * (minimum last_dt) and sleeping [n_bodies]. */
int d2g_ctx_separate_clusters(d2g_ctx* ctx, const int32_t* pairs, int32_t n_pairs, int32_t* n_clusters,
                              int32_t* particle_off, int32_t* particles, int32_t* pair_off, int32_t* cluster_pairs,
                              double* min_current_time, double* step, uint8_t* sleeping);
/* --------------------------------------------------- time-step selection --
 * fineCollisionClustersWithTimeStepSelection followed by the clamp of
 * TimeStepSelectionDynamicContinuous::selectTimeStep, for many clusters in one
 * call (collision_detection/separate_clusters.cpp:462-599,
 * strategies/time_step_size/time_step_selection_dynamic_continuous.cpp:17-21).
 * Cluster k owns interactions pairs[cluster_pair_off[k] .. cluster_pair_off[k+1])
 * in the reference's order and particles cluster_particles[cluster_particle_off[k]
 * .. +1) (its first particle gives the fallback step).  Every interaction runs
 * a CCD query over min(last_dt_a, last_dt_b) of the device bodies; the device
 * future states are left as the reference leaves them (each body's last
 * query).  step_out[k] receives the clamped step in [1e-3, opt_dt].
 * counters (optional, 4 int64) as for the CCD entry points. */
int d2g_select_time_steps(d2g_ctx* ctx, const int32_t* pairs, int32_t n_pairs, const int32_t* cluster_pair_off,
                          const int32_t* cluster_particle_off, const int32_t* cluster_particles, int32_t n_clusters,
                          float opt_dt, double* step_out, int64_t* counters);

/* ------------------------------------------------------ contact filter --
 * filterContacts(contacts, margin) for each group of contacts
 * (collision_detection/contact.h:44-69; called per interaction with margin 0
 * at strategies/PDE/PDE_explicit.cpp:85): a stable sort by (eps_a + eps_b,
 * |A - B|), then a contact is kept unless its midpoint lies within
 * eps_a + eps_b + margin of an already kept contact's midpoint.  Group g is
 * contacts[offsets[g] .. offsets[g+1]); its kept contacts are
 * out[out_offsets[g] .. out_offsets[g+1]).  D2G_CAPACITY when more than
 * capacity contacts are kept (out_offsets still written). */
int d2g_filter_contacts(d2g_ctx* ctx, const double* contacts, const int32_t* offsets, int32_t n_groups, double margin,
                        double* out, int32_t capacity, int32_t* out_offsets);
/* ------------------------------------------------- sequential impulses --
 * SequentialImpulses::solve (strategies/contact_force/sequential_impulses.cpp:
 * 104-638) for many clusters in one call, one block per cluster.  Cluster k
 * has particles particles[particle_off[k] .. +1) (a moving body in one cluster
 * only), step step[k] and hits contacts[contact_off[k] .. +1) in the
 * reference's hit order; pair_count[i] is the number of hits of contact i's
 * body pair in its cluster (the friction split) and warm[i] the warm-start
 * impulse stored for that pair (NaN when none;
 * sequential_impulses_warm_start.cpp:11-26).  The device future states of the
 * cluster's moving bodies are replaced by the solved ones.  Outputs: status[k]
 * (0 ok, 1 rejected: a hit closer than 1e-6 with step > 1e-4),
 * iterations[2k..2k+1] (normal, friction), and per hit in the solver's sorted
 * order its final normal impulse and body pair.  Returns D2G_SOLVE_FAILED when
 * any cluster was rejected. */
int d2g_solve_clusters(d2g_ctx* ctx, int32_t n_clusters, const int32_t* particle_off, const int32_t* particles,
                       const double* step, const double* contacts, const int32_t* contact_off,
                       const int32_t* pair_count, const double* warm, double gravity_z, int32_t* status,
                       int32_t* iterations, double* impulse_out, int32_t* pair_out);
/* ----------------------------------------------- adaptive cluster stepper --
 * BroadPhaseEmbreeCluster::step (strategies/broad_phase/
 * broad_phase_embree_cluster.cpp:125-257) with stepRecursive, PDEExplicit::step
 * and SequentialImpulses over the context's device bodies: the broad phase
 * and scheduling run on the host, every cluster's time-step selection, narrow
 * phase, contact filter, solve and state updates run batched on the GPU.
 * d2g_world_configure takes each body's local mesh box (6 floats: min, max;
 * Mesh::getAABB) for the static bodies' broad-phase bounds, the option time
 * step and gravity; it clears the warm-start store and the statistics.
 * d2g_world_stats: ccd_pairs, ccd_contacts, np_pairs, np_contacts, solves,
 * failures, normal_iters, friction_iters, ccd_node_pairs, ccd_tri_pairs,
 * ccd_leaf_pairs, np_node_pairs, np_tri_pairs.  d2g_world_warm lists the
 * warm-start store in ascending body-pair order.  An invalid state
 * interpolation (where the reference throws) returns D2G_ERR_STATE. */
int d2g_world_configure(d2g_ctx* ctx, const float* local_aabb, float opt_dt, double gravity_z);
int d2g_world_step(d2g_ctx* ctx, int32_t n_steps);
int d2g_world_stats(d2g_ctx* ctx, int64_t* stats13);
int d2g_world_warm(d2g_ctx* ctx, int32_t* keys, double* values, int32_t capacity, int32_t* n);
/* Instrumentation (no reference counterpart): cumulative host wall time in ms
 * of the stepper's phases since d2g_world_configure: 0 state projection and
 * copy back, 1 broad phase, 2 cluster labelling and rollback, 3 time-step
 * selection (CCD), 4 sleeping clusters, 5 narrow phase, 6 contact filter,
 * 7 solve and state shift, 8 recursion bookkeeping and static bodies. */
#define D2G_WORLD_PHASES 10
int d2g_world_timing(d2g_ctx* ctx, double* ms, int32_t n);
/* ------------------------------------------- learned TOI proposal (MLP) --
 * No counterpart in the reference.  A 20-128-128-2 MLP with SiLU, BF16
 * weights and activations and FP32 accumulation, trained and run by this
 * library's own tensor-core kernels.  Input: the 20 FP32 features of a CCD
 * pair query (B's pose in A's frame: rotation 3x3 row major and translation;
 * relative linear and angular velocity in A's frame; the two bodies' bounding
 * radii), standardised with d2g_mlp_set_normalization.  Output per query:
 * (normalised time of impact, hit logit).  Loss: squared TOI error plus the
 * hit's binary cross-entropy, averaged over the batch.  Parameters (FP32
 * master copy, D2G_MLP_PARAMS floats): W1 [128][20], b1 [128], W2 [128][128],
 * b2 [128], W3 [2][128], b3 [2].  Training is Adam (0.9, 0.999, 1e-8) over
 * shuffled mini-batches. */
#define D2G_MLP_PARAMS 19458
/* A network belongs to the context it was created on.  Destroying the context
 * first is allowed: the network then keeps only its device memory (freed by
 * d2g_mlp_destroy) and its other calls return D2G_ERR_STATE. */
int d2g_mlp_create(d2g_ctx* ctx, uint64_t seed, d2g_mlp** out);
void d2g_mlp_destroy(d2g_mlp* mlp);
int d2g_mlp_params(d2g_mlp* mlp, float* params, int32_t n);
int d2g_mlp_set_params(d2g_mlp* mlp, const float* params, int32_t n);
int d2g_mlp_set_normalization(d2g_mlp* mlp, const float* mean20, const float* std20);
int d2g_mlp_predict(d2g_mlp* mlp, const float* features, int32_t n, float* out);
/* Gradient of the mean loss over n samples (targets [n][2]: TOI, hit). */
int d2g_mlp_gradient(d2g_mlp* mlp, const float* features, const float* targets, int32_t n, float* grad, float* loss);
int d2g_mlp_train(d2g_mlp* mlp, const float* features, const float* targets, int32_t n, int32_t epochs, int32_t batch,
                  float lr, uint64_t seed, float* epoch_loss);
/* ------------------------------------ allocation-free discrete narrow phase
 * No counterpart in the reference.  The same compareTreesFull traversal and
 * contacts as d2g_compare_trees_full, for callers that may not allocate
 * device memory during the call: hosts with a fixed up-front memory budget
 * (real-time game or robotics loops where an allocation can stall or fail
 * mid-frame), or embedding runtimes that own every allocation.  It calls no
 * cudaMalloc, cudaFree or allocating library routine and needs no context:
 * the caller passes the scene, pairs and output buffers in device memory, and
 * a stream.  Intermediate buffers live in one file-scope device array of
 * 24 MiB that every GPU loading this library holds until the process exits.
 * Limits per call (larger requests fail with D2G_ERR_INVALID, before the
 * traversal or at the tree level that would pass them): */
#define D2G_NOALLOC_MAX_PAIRS 2048       /* body pairs (each puts one root node pair in the first level) */
#define D2G_NOALLOC_MAX_NODE_PAIRS 2048  /* node pairs in one tree level */
#define D2G_NOALLOC_MAX_CONTACTS 32768   /* contacts found */
/* All calls share that array: counters are cleared on every call, and calls
 * whose GPU work overlaps (other streams or threads) race on it.  The call
 * reads each tree level's sizes back to the host, so it synchronizes the
 * stream once per level and once at the end.  The first call on a device
 * looks up the array's address (cudaGetSymbolAddress) and caches it: make
 * that first call before any stream capture.  Returns D2G_CAPACITY when the
 * contacts exceed `capacity` (offsets and *n_contacts are still written;
 * contacts are not). */
typedef struct d2g_device_scene {
    int32_t n_meshes;
    int32_t n_nodes;
    const int32_t* mesh_node_off; /* device pointers, layout as d2g_trees / d2g_bodies */
    const int32_t* nodes;
    const int32_t* ntris;
    const double* tris;
    const double* eps;
    const double* inner_eps;
    int32_t n_bodies;
    const int32_t* mesh;
    const double* fut; /* [n_bodies][14] future states used as the poses */
    const double* geo_eps;
} d2g_device_scene;
int d2g_compare_trees_full_noalloc(const d2g_device_scene* scene, const int32_t* d_pairs, int32_t n_pairs,
                                   double* d_contacts, int32_t capacity, int32_t* d_offsets, int32_t* n_contacts,
                                   void* stream);

#ifdef __cplusplus
}
#endif

#endif /* D2G_H */
