/*
 * capi_internal.h — shared state of the C11 host layer.
 *
 * The free functions of the reference API (octree_*, integrator_*, sph_*)
 * take host Body/OctreeNode arrays on every call. Each calling thread gets its
 * own device state (csgd_t, created on first use, grown as needed) so calls
 * from different threads never share buffers or streams.
 */
#ifndef CSG_CAPI_INTERNAL_H
#define CSG_CAPI_INTERNAL_H

#include "../../../include/cosmosim_gb300.h"
#include "../device/csg_device.h"

/* Thread's device state, or NULL when no CUDA device is usable (then the
   thread's last error is CSG_ERR_NO_DEVICE). */
csgd_t *csg_thread_dev(void);
void csg_thread_set_error(int code);
int csg_thread_precision(void);

/* Node count (highest reachable index + 1) of the tree reachable from root,
   found by a depth-first scan. Returns 0, or CSG_ERR_BAD_POOL when the
   cells do not form a tree. */
int csg_pool_extent(const OctreeNode *pool, int root, int *n_nodes);

/* Seeded initial conditions (ics.c). */
int csg_generate_ics_impl(int kind, int n, uint64_t seed, Body *out);
void csg_ref_spiral(Body *bodies, int n, double cx, double cy, double galaxy_mass,
                    double disk_radius, double vx_bulk, double vy_bulk, uint64_t seed);
void csg_ref_merger(Body *bodies, int n, double separation, double approach_vel, uint64_t seed);
void csg_ref_quasar_galaxy(Body *bodies, int n, double cx, double cy, double galaxy_mass,
                           double disk_radius, double vx_bulk, double vy_bulk,
                           double smbh_mass_frac, uint64_t seed);
void csg_ref_quasar_merger(Body *bodies, int n, double separation, double approach_vel,
                           double smbh_mass_frac, uint64_t seed);
void csg_ref_merger_dust(Body *bodies, int start_idx, int n_dust, double separation,
                         uint64_t seed);
int csg_disk_plan(int kind, uint64_t seed, csgd_disk_plan *plan);
/* Copies a device state's phase sums into the C-ABI record. */
int csg_fill_phase_times(const csgd_t *d, CsgPhaseTimes *out);

#endif
