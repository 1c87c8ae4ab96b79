/*
 * cosmosim_abi.h — the binary interface that libcosmosim_gb300.so shares with
 * cosmosim's C callers (main.c, tests/test_physics.c, the Unreal plugin).
 *
 * The three structs below are ABI: their field order, types and therefore
 * their sizes and offsets are those of the reference headers, so a caller that
 * was compiled against cosmosim's own headers can link this library instead of
 * cosmosim's octree.c / integrator.c / sph.c / cosmosim_api.c unchanged.
 *   Body          — reference src/body.h:13-27   (168 bytes on LP64)
 *   OctreeNode    — reference src/octree.h:6-14  (104 bytes on LP64)
 *   CosmosimConfig— reference src/cosmosim_api.h:16-27 (72 bytes on LP64)
 * The static assertions at the end of this header pin those sizes.
 *
 * Every entry point declared here keeps the reference signature; the file:line
 * next to each one names the declaration it replaces.
 */
#ifndef COSMOSIM_ABI_H
#define COSMOSIM_ABI_H

#ifdef __cplusplus
extern "C" {
#endif

/* Body kinds (reference src/body.h:4-11). Only STAR and GAS matter to the
   gravity/SPH path: every kind attracts; SPH acts between GAS bodies. */
typedef enum {
    BODY_STAR = 0,
    BODY_GAS = 1,
    BODY_SMBH = 2,
    BODY_JET = 3,
    BODY_DUST = 4,
    BODY_LOBE = 5
} BodyType;

/* One particle, array-of-structs as the callers hold it (reference
   src/body.h:13-27). mass <= 0 marks a dead body: it is left out of the tree,
   receives zero acceleration and is neither kicked nor drifted. */
typedef struct {
    double x, y, z;
    double vx, vy, vz;
    double ax, ay, az;
    double mass;
    BodyType type;
    double spin_x, spin_y, spin_z;
    double accretion_rate;
    double luminosity;
    double lifetime;
    double density;
    double pressure;
    double internal_energy;
    double smoothing_h;
} Body;

/* One octree cell in the caller-owned pool (reference src/octree.h:6-14).
   (cx,cy,cz,total_mass) is the cell's centre of mass and mass; center_* and
   half_size its geometric cube; body_index >= 0 marks a leaf; children[q] is
   the cell of octant q (bit0: x >= centre, bit1: y < centre, bit2: z < centre)
   or -1. The root is pool[0]. */
typedef struct {
    double cx, cy, cz;
    double total_mass;
    double center_x, center_y, center_z;
    double half_size;
    int body_index;
    int children[8];
} OctreeNode;

/* Simulation set-up for the handle API (reference src/cosmosim_api.h:16-27). */
typedef struct {
    int n_bodies;
    int merger;
    int quasar;
    double dt;
    double theta;
    double smbh_mass_frac;
    double accretion_radius;
    double jet_speed;
    double feedback_strength;
    int substeps;
} CosmosimConfig;

typedef void *SimHandle;

/* Quasar-mode settings of the reference's CPU quasar step (src/quasar.h:6-22).
   The quasar step itself stays on the caller's CPU path; this library only
   calls it, between substeps, when the application links it. */
typedef struct {
    double accretion_radius;
    double swallow_radius;
    double isco_radius;
    double viscosity_alpha;
    double jet_speed;
    double jet_mass;
    double jet_lifetime;
    double feedback_strength;
    double eta_eff;
    double eddington_k;
    double accretion_smoothing;
    int jet_cap;
    int jet_count;
    int max_bodies;
    int jet_ring_count;
} QuasarConfig;

#if defined(_WIN32)
#define CSG_EXPORT __declspec(dllexport)
#else
#define CSG_EXPORT __attribute__((visibility("default")))
#endif

/* SPH constants of the reference (src/sph.h:7-9). */
#define CSG_SPH_GAMMA (5.0 / 3.0)
#define CSG_SPH_TARGET_NEIGHBORS 32
#define CSG_SPH_MAX_NEIGHBORS 128

/* ---- octree.h (reference src/octree.h:16-36) ---------------------------- */

/* Builds the octree of the alive bodies into pool[0..*pool_size). pool must
   hold at least 8*n nodes, as for the reference (src/octree.c:114-169). */
CSG_EXPORT void octree_build(OctreeNode *pool, int *pool_size, const Body *bodies, int n);

/* Sets a of every body to the Barnes-Hut monopole acceleration from the tree
   in pool, with Plummer softening and opening angle theta
   (src/octree.c:220-234). */
CSG_EXPORT void octree_compute_forces(const OctreeNode *pool, int root, Body *bodies, int n,
                                      double G, double softening, double theta);

/* Writes into neighbor_buf the first buf_capacity alive bodies within radius
   of (cx,cy,cz), in depth-first octant order, and returns how many
   (src/octree.c:293-318). */
CSG_EXPORT int octree_find_neighbors(const OctreeNode *pool, int root, const Body *bodies,
                                     int n, double cx, double cy, double cz, double radius,
                                     int *neighbor_buf, int buf_capacity);

/* ---- integrator.h (reference src/integrator.h:7-17) --------------------- */

/* One kick-drift-kick leapfrog step (src/integrator.c:12-57); pool is scratch
   of at least 8*n nodes and holds the rebuilt tree on return. */
CSG_EXPORT void integrator_step(Body *bodies, int n, double dt, double G, double softening,
                                double theta, OctreeNode *pool, int sph_enabled);

/* Builds the tree and sets the accelerations once (src/integrator.c:4-10). */
CSG_EXPORT void integrator_init_accelerations(Body *bodies, int n, double G, double softening,
                                              double theta, OctreeNode *pool);

/* ---- sph.h (reference src/sph.h:12-19) ---------------------------------- */

CSG_EXPORT void sph_compute_density(Body *bodies, int n, const OctreeNode *tree);
CSG_EXPORT void sph_compute_forces(Body *bodies, int n, const OctreeNode *tree);
CSG_EXPORT void sph_apply_cooling(Body *bodies, int n, double dt);

/* ---- cosmosim_api.h (reference src/cosmosim_api.h:35-42) ---------------- */

CSG_EXPORT CosmosimConfig cosmosim_default_config(void);
CSG_EXPORT SimHandle cosmosim_create(CosmosimConfig config);
CSG_EXPORT void cosmosim_step(SimHandle handle);
CSG_EXPORT const Body *cosmosim_get_bodies(SimHandle handle);
CSG_EXPORT int cosmosim_get_count(SimHandle handle);
CSG_EXPORT int cosmosim_get_active_count(SimHandle handle);
CSG_EXPORT double cosmosim_get_sim_time(SimHandle handle);
CSG_EXPORT void cosmosim_destroy(SimHandle handle);

#ifdef __cplusplus
}
#endif

/* Layout pins (LP64: Linux x86_64 and aarch64). */
#ifdef __cplusplus
static_assert(sizeof(Body) == 168, "Body must be 168 bytes");
static_assert(sizeof(OctreeNode) == 104, "OctreeNode must be 104 bytes");
static_assert(sizeof(CosmosimConfig) == 72, "CosmosimConfig must be 72 bytes");
static_assert(sizeof(QuasarConfig) == 104, "QuasarConfig must be 104 bytes");
#else
_Static_assert(sizeof(Body) == 168, "Body must be 168 bytes");
_Static_assert(sizeof(OctreeNode) == 104, "OctreeNode must be 104 bytes");
_Static_assert(sizeof(CosmosimConfig) == 72, "CosmosimConfig must be 72 bytes");
#endif

#endif /* COSMOSIM_ABI_H */
