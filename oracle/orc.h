/*
 * orc.h — CPU oracle for the gravity/SPH hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C (C11 + OpenMP) restatement of
 * cosmosim's double-precision CPU algorithm, used as the oracle for the CUDA
 * path and as the timed CPU baseline. Only tests/, __graft_entry__.smoke() and
 * bench.py (its cpu_baseline leg and its --impl reference arm) may load it.
 * The product library never links or calls it.
 *
 * Every function follows the reference file:line given beside it step for
 * step, including the order of floating-point operations, so that with
 * -ffp-contract=off it reproduces the reference bit for bit; this is checked
 * against the reference's own compiled sources and golden fixtures in tests/.
 * Symbols are prefixed orc_ so the oracle can share a process with the library.
 */
#ifndef CSG_ORACLE_H
#define CSG_ORACLE_H

#include <stdint.h>
#include "../include/cosmosim_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- octree (reference src/octree.c) ---- */
void orc_octree_build(OctreeNode *pool, int *pool_size, const Body *bodies, int n);
void orc_octree_compute_forces(const OctreeNode *pool, int root, Body *bodies, int n, double G,
                               double softening, double theta);
int orc_octree_find_neighbors(const OctreeNode *pool, int root, const Body *bodies, int n,
                              double cx, double cy, double cz, double radius, int *buf,
                              int capacity);

/* Interaction counts of the reference walk: per body (may be NULL) and total.
   An interaction is one accepted cell or one leaf other than the body itself
   (reference src/octree.c:191-209). */
int64_t orc_octree_count_interactions(const OctreeNode *pool, int root, const Body *bodies,
                                      int n, double theta, int32_t *per_body);

/* ---- SPH (reference src/sph.c) ---- */
void orc_sph_compute_density(Body *bodies, int n, const OctreeNode *tree);
void orc_sph_compute_forces(Body *bodies, int n, const OctreeNode *tree);
void orc_sph_apply_cooling(Body *bodies, int n, double dt);

/* ---- integrator (reference src/integrator.c) ---- */
void orc_integrator_step(Body *bodies, int n, double dt, double G, double softening,
                         double theta, OctreeNode *pool, int sph_enabled);
void orc_integrator_init_accelerations(Body *bodies, int n, double G, double softening,
                                       double theta, OctreeNode *pool);

/* ---- checks (reference tests/test_physics.c:34-71) ---- */
/* Direct-sum accelerations of the bodies listed in idx (all n if idx NULL),
   written to acc[3*k..]. Same pair formula as the reference test helper. */
void orc_direct_forces(const Body *bodies, int n, const int32_t *idx, int m, double G,
                       double softening, double *acc);
/* Kinetic + softened potential energy, O(n^2). */
double orc_total_energy(const Body *bodies, int n, double G, double softening);

/* Seeded benchmark initial conditions (orc_ics.c): the kinds of the
   library's csg_generate_ics, byte for byte, so that CPU-only runs need not
   load the library. Returns n, or -1 for a bad kind or count. */
int orc_generate_ics(int kind, int n, uint64_t seed, Body *out);

/* Threads the OpenMP loops use (0 = runtime default). Returns the count in use. */
int orc_set_threads(int nthreads);

/* Quasar step, reference src/quasar.c:477-509 (single-threaded, as the
   reference). The generator state and knot phase persist between calls
   (src/quasar.c:11, :224); orc_quasar_seed sets them. */
void orc_quasar_step(Body *bodies, int *n, int n_alloc, QuasarConfig *cfg, double dt);
void orc_quasar_seed(uint64_t rng_state, int knot_phase);

#ifdef __cplusplus
}
#endif
#endif
