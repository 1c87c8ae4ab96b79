/*
 * csg_device.h — the thin C-ABI between the C11 host layer and the CUDA
 * kernels. Everything here is plain C: opaque handles, pointers and sizes.
 *
 * A csgd_t holds one simulation's device state on one CUDA stream:
 *   - bodies as FP64 structure-of-arrays in the caller's index order
 *     (x,y,z, vx,vy,vz, ax,ay,az, mass, type, density, pressure, u, h),
 *   - the octree in depth-first (preorder) layout, built every substep from
 *     63-bit octant keys (see dev_tree.cu),
 *   - scratch for the key sort, the tree and the Body array-of-structs staging.
 * All calls are asynchronous on the state's stream unless they say otherwise;
 * csgd_sync() waits and reports the first error.
 */
#ifndef CSG_DEVICE_H
#define CSG_DEVICE_H

#include <stdint.h>
#include "../../../include/cosmosim_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct csgd csgd_t;

/* Error codes and precisions: CSG_OK, CSG_ERR_*, CSG_PREC_* (cosmosim_gb300.h). */

typedef struct {
    double G, softening, theta;
    int precision; /* CSG_PREC_* */
} csgd_force_params;

csgd_t *csgd_create(void);
void csgd_destroy(csgd_t *d);

/* Uses the given cudaStream_t (NULL = the state's own stream). */
void csgd_set_stream(csgd_t *d, void *stream);
void *csgd_stream(csgd_t *d);
/* The device Body staging array (capacity >= the reserved body count). */
Body *csgd_aos(csgd_t *d);

/* Tree builds also record what a reference-order pool export needs (on for
   states that export after most builds; export works either way). */
void csgd_set_export_order(csgd_t *d, int on);

/* Makes room for n bodies (grow-only). */
int csgd_reserve(csgd_t *d, int n);

/* The build's key sort on host keys (csg_sort_keys, cosmosim_gb300.h); uses
   the state's key buffers. */
int csgd_sort_keys(csgd_t *d, const unsigned long long *keys, int n, int bits,
                   unsigned long long *out_keys, int *out_index);
int csgd_count(const csgd_t *d);

/* Forest: the n bodies form n_sys independent systems, system g holding the
   host_counts[g] bodies that follow those of systems 0..g-1 (caller order;
   counts sum to n). Every system gets its own root cube and tree; walks never
   cross systems. n_sys = 1 (the default, counts ignored) is one simulation.
   SPH, pool export/import and neighbour queries need n_sys = 1. A later
   csgd_reserve with another n returns to one system. */
int csgd_set_systems(csgd_t *d, int n_sys, const int *host_counts);
int csgd_system_count(const csgd_t *d);

/* Walk launch shape (CsgWalkShape, cosmosim_gb300.h). */
int csgd_set_walk_shape(csgd_t *d, const CsgWalkShape *w);
void csgd_get_walk_shape(const csgd_t *d, CsgWalkShape *w);
/* Times every candidate shape on the current tree (reps walks each, median)
   and keeps the fastest; *out gets it, all[0..all_cap) every candidate with
   its time, *n_all their number. Blocks; not inside a stream capture. */
int csgd_autotune_walk(csgd_t *d, const csgd_force_params *p, int reps, CsgWalkShape *out,
                       CsgWalkShape *all, int all_cap, int *n_all);

/* Body array-of-structs <-> device SoA (host buffers may be pageable). */
int csgd_upload_bodies(csgd_t *d, const Body *host, int n);
int csgd_download_bodies(csgd_t *d, Body *host, int n);
/* Download of what a leapfrog step changes (x..az, and with sph != 0 density,
   pressure, internal energy, smoothing length): into a mapped (pinned) host
   array those fields are written directly and the caller's other fields are
   left alone; any other host array gets csgd_download_bodies. */
int csgd_download_step_fields(csgd_t *d, Body *host, int n, int sph);
/* Refreshes the device Body staging from the SoA fields (no copy to the host),
   and the SoA fields from the staging. */
int csgd_pack_aos(csgd_t *d);
int csgd_unpack_aos(csgd_t *d);

/* Alive bodies (mass <= 0 skipped) as packed float records, in index order,
   at most max_bodies: CSG_SNAPSHOT_UE (16 floats) or CSG_SNAPSHOT_RENDER (10).
   out is a device pointer when out_is_device, else host memory. Blocks. */
int csgd_snapshot_f32(csgd_t *d, int format, float *out, int out_is_device, int max_bodies,
                      int *count_out);

/* Exponential-disk initial conditions generated on the device (the recipe of
   csg_generate_ics kinds 0, 3, 5, 6): system g gets counts[g] bodies from
   plans[g], written to out (device Body array) one system after another.
   The seeded xorshift64 stream is jumped ahead per run of bodies, so body i
   draws the same numbers as the host generator's body i. Blocks. */
typedef struct {
    double mass, rd, zh, smbh, gas_frac, bulge_mass, bulge_a;
    uint64_t seed;   /* generator state before the disk's first draw */
    int pad;
} csgd_disk_plan;
int csgd_generate_disks(void *stream, const csgd_disk_plan *plans, const int *counts, int n_sys,
                        Body *out);
/* Replaces the bodies by a device Body array of n bodies (D2D). */
int csgd_upload_device_bodies(csgd_t *d, const Body *device_bodies, int n);

/* Quasar step on the device (reference src/quasar.c:477-509): may append
   bodies up to n_alloc (<= the reserved capacity); *jet_count is read and
   updated (the reference's cfg->jet_count); *n_out gets the new body count.
   The generator state and knot phase persist in the state between steps;
   csgd_quasar_state sets them (defaults 1 and 0, as the reference starts).
   Blocks (the host needs the new count). */
int csgd_quasar_step(csgd_t *d, const QuasarConfig *cfg, int n_alloc, double dt,
                     int *jet_count, int *n_out);
int csgd_quasar_state(csgd_t *d, unsigned long long rng, int knot_phase);
/* Phase timing: on = 1 makes every later substep run as direct launches with
   CUDA events between its phases (and NVTX ranges around them), waiting for
   each substep's events; the phase times add up in ms[7] (kick+drift, tree
   build, gravity walk, SPH, second kick, cooling, whole substep), then in
   ms[7..11] the build's parts (keys, sort, cells, moments, the rest). Turning
   it on resets the sums; turning it off keeps them for reading. */
int csgd_set_phase_timing(csgd_t *d, int on);
int csgd_phase_times(const csgd_t *d, double ms[12], long long *substeps);
/* 1 when a CUDA device is visible (tells allocation failures from a missing GPU). */
int csgd_has_device(void);
/* Limit of the walks' bounded producer/consumer waits, in polls (<= 0: the
   default 2^22). Drops the captured substep. */
void csgd_set_wait_limit(csgd_t *d, int polls);
/* Runs the radix sort's look-back wait on a status word that nothing
   publishes, with the given poll limit: *status receives the error the wait
   reported (CSG_ERR_DEVICE_WAIT when it gave up, as it must). */
int csgd_check_device_wait(csgd_t *d, int polls, int *status);
/* Frees the quasar step's device scratch (state destruction). */
void csgd_quasar_free(csgd_t *d);

/* Drops bodies whose mass is not > 0, keeping the order of the rest
   (reference src/quasar.c:511-523); *new_n is the new count. Blocks. */
int csgd_compact(csgd_t *d, int *new_n);

/* Tree build over the current positions/masses. With geometry != 0 it also
   computes every cell's geometric centre (needed by SPH and pool export). */
int csgd_build_tree(csgd_t *d, int geometry);

/* Accelerations a = Barnes-Hut gravity (overwrites a; dead bodies get 0).
   exact != 0 uses the reference's own FP64 operation sequence. */
int csgd_gravity(csgd_t *d, const csgd_force_params *p);
int csgd_gravity_ex(csgd_t *d, const csgd_force_params *p, int exact);

/* Interaction lists of the current tree (built here): with fill = 0 writes
   counts[i] (cells body i interacts with; untouched for dead bodies); with
   fill = 1 writes the cell ids, in the reference's depth-first order, to
   ids[offs[i] ..], at most cap entries in all. Device pointers. */
int csgd_walk_lists(csgd_t *d, const csgd_force_params *p, int *counts, const int *offs,
                    int *ids, int cap, int fill);

/* SPH on the current tree (needs geometry). csgd_sph_forces =
   csgd_sph_force_terms (pair terms; touches no acceleration) then
   csgd_sph_force_sums (adds them to the accelerations). reuse_lists = 1 is
   for a force pass right after csgd_sph_density on the same tree and bodies:
   only the gas bodies whose smoothing length that pass changed search the
   tree again; the others keep the density pass's list, which is the list a
   new search would find (same tree, position and radius). */
int csgd_sph_density(csgd_t *d);
int csgd_sph_forces(csgd_t *d, int reuse_lists);
int csgd_sph_force_terms(csgd_t *d, int reuse_lists);
int csgd_sph_force_sums(csgd_t *d);
int csgd_sph_cooling(csgd_t *d, double dt);

/* Leapfrog pieces: v += a*dt/2 and x += v*dt; and v += a*dt/2. */
int csgd_kick_drift(csgd_t *d, double dt);
int csgd_kick(csgd_t *d, double dt);

/* One full KDK substep, all on the device (reference src/integrator.c:12-57). */
int csgd_substep(csgd_t *d, double dt, const csgd_force_params *p, int sph);

/* k substeps; with graphs enabled (default) one substep is captured once as a
   CUDA graph and replayed (re-captured when dt/G/softening/theta/precision/
   sph/n or the stream change). */
int csgd_substeps(csgd_t *d, int k, double dt, const csgd_force_params *p, int sph);
void csgd_enable_graphs(csgd_t *d, int on);

/* Allocates the SPH neighbour lists now (they are otherwise allocated on the
   first SPH pass, which must not happen inside a stream capture). */
int csgd_prepare_sph(csgd_t *d);

/* The tree as a reference-layout pool, in the reference's allocation order.
   Blocks until done. pool must hold *pool_size_out <= capacity nodes; a
   mapped (pinned) host pool is written by the export kernel directly. */
int csgd_export_pool(csgd_t *d, OctreeNode *pool, int capacity, int *pool_size_out);

/* The same export enqueued on the state's stream without a host round trip:
   dst is device-accessible (device memory or the device view of a mapped
   host array) with room for capacity cells; a larger tree records
   CSG_ERR_NODE_CAPACITY for the next csgd_sync and writes nothing. Needs a
   tree built with the export order (csgd_set_export_order). */
int csgd_export_to(csgd_t *d, OctreeNode *dst, int capacity);

/* Device view of a mapped (pinned) host pointer, or NULL for any other
   memory. */
void *csgd_host_view(const void *p);

/* While set (dst != NULL), every substep also exports the tree it builds to
   dst (as csgd_export_to), on a third stream beside the walk. Returns 1 when
   set, 0 when this state cannot (no third stream, no export order, several
   systems): the caller then exports after the substep. */
int csgd_set_substep_export(csgd_t *d, OctreeNode *dst, int capacity);

/* Replaces the device tree by the caller's pool (nodes reachable from root;
   n_nodes = highest reachable index + 1). */
int csgd_import_pool(csgd_t *d, const OctreeNode *pool, int n_nodes, int root);

/* Neighbour query on the current tree, reference semantics (first cap alive
   bodies within radius in depth-first order). Blocks until done. */
int csgd_find_neighbors(csgd_t *d, double cx, double cy, double cz, double radius, int *buf,
                        int cap, int *count_out);

/* Node count of the current tree (blocks). */
int csgd_node_count(csgd_t *d, int *n_nodes);

/* Interaction count summed over gravity walks since the last reset (only
   while stats are enabled). */
void csgd_enable_stats(csgd_t *d, int on);
int csgd_reset_stats(csgd_t *d);
int csgd_interactions(csgd_t *d, int64_t *total);
/* ... with the walks' warp steps and the lane-steps of lanes still walking. */
int csgd_walk_stats(csgd_t *d, int64_t *interactions, int64_t *warp_steps,
                    int64_t *active_lane_steps);

/* Alive bodies (mass > 0 or NaN, as the reference's mass <= 0 test). Blocks. */
int csgd_alive_count(csgd_t *d, int *count);

/* FP64 diagnostics on the current bodies: direct-sum accelerations of the
   ns bodies in host_idx (host_out: 3*ns doubles), and KE / softened PE. Block. */
int csgd_direct_forces(csgd_t *d, const int *host_idx, int ns, double G, double softening,
                       double *host_out);
int csgd_energy(csgd_t *d, double G, double softening, double *ke, double *pe);

/* Kernels launched on this state so far. */
unsigned long long csgd_launch_count(const csgd_t *d);

/* Waits for the stream; returns CSG_OK or the first error (CUDA or device). */
int csgd_sync(csgd_t *d);
const char *csgd_error_string(int code);

#ifdef __cplusplus
}
#endif
#endif
