/*
 * cosmosim_gb300.h — additive entry points of libcosmosim_gb300.so.
 *
 * Nothing here replaces a reference symbol; these are the extensions a caller
 * may use beside the drop-in API of cosmosim_abi.h. None has a counterpart in
 * the reference unless its comment names one.
 *
 * Error convention (as the reference's API): no call aborts or traps. Free
 * functions record their status per calling thread (csg_last_error); handle
 * calls record it per handle (cosmosim_last_error).
 */
#ifndef COSMOSIM_GB300_H
#define COSMOSIM_GB300_H

#include <stdint.h>
#include "cosmosim_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Error codes. */
#define CSG_OK 0
#define CSG_ERR_CUDA 1
#define CSG_ERR_NOMEM 2
#define CSG_ERR_NODE_CAPACITY 3
#define CSG_ERR_BAD_ARG 4
#define CSG_ERR_BAD_POOL 5
#define CSG_ERR_WALK_LIMIT 6
#define CSG_ERR_NO_DEVICE 7
#define CSG_ERR_UNSUPPORTED 8
#define CSG_ERR_DEVICE_WAIT 9 /* a bounded device-side wait expired */

/* Walk precision. FP64 is the drop-in default. FP32_MIXED evaluates pair
   accelerations in FP32 (positions as float hi/lo pairs, Kahan-compensated
   per-body sums) with FP64 tree moments, drift and opening ties. */
#define CSG_PREC_FP64 0
#define CSG_PREC_FP32_MIXED 1

/* Most independent systems one handle may hold (cosmosim_create_ensemble). */
#define CSG_MAX_SYSTEMS 65536

/* Launch shape of the gravity walk. A walk task is up to 32 consecutive
   key-ordered bodies of one system, walked by one warp. Until a shape is
   set (cosmosim_set_walk_shape, cosmosim_autotune_walk) a handle uses
   {4, 0, 0}.
     warps_per_block  4 or 8
     task_group       0: one warp per task (grid covers every task);
                      g > 0: persistent launch, each warp takes g tasks at a
                      time from a device counter until none are left
     blocks_per_sm    persistent launch only: blocks per SM (1..32)
     ms               filled by the autotuner: median walk time, ms
   The shape applies to the FP32-mixed walk; the FP64 walk always runs one
   producer/consumer warp pair per task (or, for systems of up to 12 x 32
   bodies per SM, pairs per child subtree of the root). Results do not depend
   on the shape; only the time does. */
typedef struct {
    int warps_per_block;
    int task_group;
    int blocks_per_sm;
    float ms;
} CsgWalkShape;

/* Status of the calling thread's last free-function call (octree_*,
   integrator_*, sph_*); 0 = success. Reset by every call. */
CSG_EXPORT int csg_last_error(void);
CSG_EXPORT const char *csg_error_string(int code);

/* Precision the calling thread's free functions use (default FP64). */
CSG_EXPORT void csg_set_precision(int precision);

/* Frees the calling thread's device state (the free functions create one per
   thread on first use; a thread pool can release it before a thread ends).
   The next free-function call on the thread creates a new one. */
CSG_EXPORT void csg_release_thread_state(void);

/* ---- Failure handling and fault injection ----------------------------------
   No counterpart in the reference (its API has no error channel). Every device
   wait in the library is bounded; the walks' producer/consumer waits give up
   after `polls` polls (default 2^22, about 0.3 s) and report
   CSG_ERR_DEVICE_WAIT at the next sync, with the context still usable.
   cosmosim_set_wait_limit / csg_set_wait_limit lower that limit for a handle /
   the calling thread's free functions (polls <= 0 restores the default) — for
   tests that make a wait run out. */
CSG_EXPORT int cosmosim_set_wait_limit(SimHandle handle, int polls);
CSG_EXPORT void csg_set_wait_limit(int polls);

/* Self-check of the tree sort's look-back wait: runs it, on the calling
   thread's GPU state, on a status word that nothing publishes, with the given
   poll limit (>= 1). *status receives what the wait reported:
   CSG_ERR_DEVICE_WAIT when it gave up, as it must. Returns CSG_OK when the
   check ran. */
CSG_EXPORT int csg_check_device_wait(int polls, int *status);

/* Allocation-failure injection: the next `allow` device or pinned-host
   allocations of the library succeed and every later one fails, as on a GPU
   out of memory, until csg_inject_alloc_failure(-1). Calls that need memory
   then fail with CSG_ERR_NOMEM (cosmosim_create* return NULL) and leave the
   caller's arrays unchanged. Process-wide; for tests. */
CSG_EXPORT void csg_inject_alloc_failure(long long allow);

/* Status of the handle's last call; 0 = success. The reference API has no
   error channel; this is an additive one. */
CSG_EXPORT int cosmosim_last_error(SimHandle handle);

/* Run-time physics parameters for a handle. */
typedef struct {
    double G;          /* gravitational constant (reference api: 1.0) */
    double softening;  /* Plummer softening (reference api: 1.5) */
    double theta;      /* opening angle */
    double dt;         /* step */
    int substeps;      /* substeps per cosmosim_step */
    int sph;           /* 1: SPH density/forces/cooling every substep */
    int precision;     /* CSG_PREC_* */
} CsgSimParams;

/* A handle over caller-supplied bodies (copied), usable with every
   cosmosim_* call. The initial accelerations are computed as in
   cosmosim_create (tree + gravity). Returns NULL on failure. */
CSG_EXPORT SimHandle cosmosim_create_from_bodies(const Body *bodies, int n,
                                                 const CsgSimParams *params);

/* Batched ensemble: n_sys independent systems in one handle — no
   counterpart in the reference, which runs one system per process. System g
   is the counts[g] bodies that follow those of systems 0..g-1 in `bodies`
   (counts sum to n). Every system gets its own root cube and octree (the
   cells the reference would build for that system alone); one walk launch
   covers all systems and never crosses between them, so each system's
   accelerations equal those of a handle created over it alone. Substeps run
   as one captured CUDA graph for the whole ensemble. params->sph must be 0
   (CSG_ERR_UNSUPPORTED otherwise). Returns NULL on failure. */
CSG_EXPORT SimHandle cosmosim_create_ensemble(const Body *bodies, int n, int n_sys,
                                              const int *counts, const CsgSimParams *params);
CSG_EXPORT int cosmosim_system_count(SimHandle handle);

/* Walk launch shape of a handle (see CsgWalkShape). */
CSG_EXPORT int cosmosim_set_walk_shape(SimHandle handle, const CsgWalkShape *shape);
CSG_EXPORT int cosmosim_get_walk_shape(SimHandle handle, CsgWalkShape *shape);

/* Autotuner: builds the tree of the handle's current bodies, times the walk
   (at the handle's precision) with every candidate shape — warps per block
   {4, 8} x {one warp per task, persistent with task groups {1, 2, 4} and
   8, 16 or 24 resident warps per SM} — `reps` times each, keeps the fastest on the
   handle and writes it to *best. all (may be NULL) receives up to all_cap
   candidates with their times, *n_all (may be NULL) their number. Blocking;
   changes no body. */
CSG_EXPORT int cosmosim_autotune_walk(SimHandle handle, int reps, CsgWalkShape *best,
                                      CsgWalkShape *all, int all_cap, int *n_all);

/* cosmosim_create with run-time G, softening and precision. */
CSG_EXPORT SimHandle cosmosim_create_ex(CosmosimConfig config, double G, double softening,
                                        int precision);

/* Device-resident stepping: k substeps, asynchronous on the handle's stream
   (no host copy). cosmosim_step calls this, then marks the host copy stale. */
CSG_EXPORT int cosmosim_substeps_async(SimHandle handle, int k);
CSG_EXPORT int cosmosim_sync(SimHandle handle);

/* Substeps of a handle replay one captured CUDA graph per substep (default
   on); off runs them as individual launches. */
CSG_EXPORT int cosmosim_enable_graphs(SimHandle handle, int on);

/* Runs the handle's work on the given cudaStream_t (NULL: its own stream). */
CSG_EXPORT int cosmosim_set_stream(SimHandle handle, void *cuda_stream);

/* Snapshot of the alive bodies as packed float records, built on the GPU —
   no counterpart in the reference, whose consumers convert the Body array
   on the host:
     CSG_SNAPSHOT_UE      16 floats per body, the Unreal plugin's
                          FCosmosimBodyGPU (pos, mass, vel, type, internal
                          energy, density, lifetime, luminosity, spin, 0);
     CSG_SNAPSHOT_RENDER  10 floats per body, the renderer's vertex record
                          (pos, mass, vel, type, internal energy, density).
   Bodies with mass <= 0 are skipped; index order; at most max_bodies.
   out_is_device: out is a device pointer (e.g. a graphics-interop buffer),
   else host memory. Returns the number of records written, or -1 (see
   cosmosim_last_error). Blocking. */
#define CSG_SNAPSHOT_UE 0
#define CSG_SNAPSHOT_RENDER 1
CSG_EXPORT int cosmosim_snapshot_f32(SimHandle handle, int format, float *out, int out_is_device,
                                     int max_bodies);

/* Drops the dead bodies (mass not > 0) of a handle on the GPU, keeping the
   order of the others (the reference's quasar_compact, src/quasar.c:511-523).
   Returns the new count, or -1. Blocking. */
CSG_EXPORT int cosmosim_compact(SimHandle handle);

/* Copies the bodies out (n must equal cosmosim_get_count). */
CSG_EXPORT int cosmosim_copy_bodies(SimHandle handle, Body *out, int n);

/* Replaces the handle's bodies by the caller's (n must equal
   cosmosim_get_count; every field is taken, the accelerations too, as the
   next substep's first kick uses them). Asynchronous on the handle's stream:
   the caller keeps `bodies` unchanged until cosmosim_sync. The system layout
   of an ensemble is kept. */
CSG_EXPORT int cosmosim_set_bodies(SimHandle handle, const Body *bodies, int n);

/* Phase-level calls for measurement: rebuild the tree from the current
   positions; run only the gravity walk on the current tree. Asynchronous. */
CSG_EXPORT int cosmosim_build_tree_async(SimHandle handle);
CSG_EXPORT int cosmosim_gravity_async(SimHandle handle);

/* Per-phase timing of the real substep — no counterpart in the reference,
   which has no tracing. With timing on, a handle's substeps run as direct
   launches (not the captured graph) with CUDA events between their phases
   and NVTX ranges ("csg.kick_drift", "csg.build", "csg.gravity", "csg.sph",
   "csg.kick", "csg.cooling") around them; each substep waits for its events,
   and the phase times add up until read. SPH that overlaps the gravity walk
   on its own stream counts its own span plus its sums after the walk; the
   substep total is the elapsed time of the whole substep. Enabling resets
   the sums; disabling keeps them for reading and returns to graph replays. */
typedef struct {
    double kick_drift_ms; /* first half kick + drift */
    double build_ms;      /* bounding box, keys, sort, cells, moments */
    double gravity_ms;    /* the Barnes-Hut walk */
    double sph_ms;        /* neighbour lists, density, pressure and viscosity forces */
    double kick_ms;       /* second half kick */
    double cooling_ms;    /* SPH cooling */
    double substep_ms;    /* whole substeps */
    long long substeps;   /* substeps timed */
    /* the build's parts (sum to build_ms): */
    double build_keys_ms;    /* bounding box, root cube, keys */
    double build_sort_ms;    /* radix sort of the keys */
    double build_cells_ms;   /* shared keys, cell counts and scan, cells, links */
    double build_moments_ms; /* masses and centres of mass */
    double build_rest_ms;    /* walk tasks; SPH cell geometry */
} CsgPhaseTimes;
CSG_EXPORT int cosmosim_enable_phase_timing(SimHandle handle, int on);
CSG_EXPORT int cosmosim_phase_times(SimHandle handle, CsgPhaseTimes *out);
/* The same for the calling thread's free functions (integrator_step). */
CSG_EXPORT int csg_enable_phase_timing(int on);
CSG_EXPORT int csg_phase_times(CsgPhaseTimes *out);

/* Interaction counting (accepted cells + leaves, the reference walk's unit). */
CSG_EXPORT int cosmosim_enable_stats(SimHandle handle, int on);
CSG_EXPORT int cosmosim_interactions(SimHandle handle, int64_t *total);
/* The same counters with the walks' warp steps (one cell visited by a warp)
   and the lane-steps of lanes that had not finished: active / (32 steps) is
   the walk's lane utilisation. */
CSG_EXPORT int cosmosim_walk_stats(SimHandle handle, int64_t *interactions, int64_t *warp_steps,
                                   int64_t *active_lane_steps);
CSG_EXPORT int cosmosim_node_count(SimHandle handle, int *n_nodes);
CSG_EXPORT int cosmosim_set_precision(SimHandle handle, int precision);

/* FP64 diagnostics on the handle's current bodies (blocking): direct-sum
   accelerations of the m bodies listed in idx into out[3*m] (the formula of
   the reference's test helper, tests/test_physics.c:54-71; in an ensemble
   only bodies of the same system attract; every idx must lie in [0, count),
   else CSG_ERR_BAD_ARG), and kinetic / softened potential energy
   (tests/test_physics.c:34-52, O(n^2)). */
CSG_EXPORT int cosmosim_direct_forces(SimHandle handle, const int *idx, int m, double *out);
CSG_EXPORT int cosmosim_energy(SimHandle handle, double *kinetic, double *potential);

/* Kernels this handle has launched so far (for launch accounting). */
CSG_EXPORT int64_t cosmosim_launch_count(SimHandle handle);

/* FP32 and FP64 FMA throughput of the current GPU in TFLOP/s, measured by
   timing independent FMA chains: the pipe peaks the gravity walks are
   bound by. */
CSG_EXPORT int csg_measure_fp_peaks(double *fp32_tflops, double *fp64_tflops);

/* Self-check of the integer-pipe double division and square root the SPH
   passes use (correctly rounded, so they must equal the compiler's operators
   bit for bit): n seeded operand pairs of several kinds on the current GPU;
   the mismatch counts are returned (0 and 0 when correct). */
CSG_EXPORT int csg_check_div_sqrt(int64_t n, uint64_t seed, int64_t *div_mismatches,
                                  int64_t *sqrt_mismatches);

/* The tree build's key sort on caller keys: an LSD radix sort, 8 bits a pass,
   ceil(bits/8) passes (bits 1..64), stable. out_keys = keys in ascending order
   of their low 8*ceil(bits/8) bits; out_index = the input position of each
   sorted key (equal keys keep their input order). Host arrays of n entries
   (n >= 0). Uses the calling thread's device state; returns CSG_OK or an
   error code. */
CSG_EXPORT int csg_sort_keys(const uint64_t *keys, int n, int bits, uint64_t *out_keys,
                             int *out_index);

/* FP64 direct-sum accelerations without any allocation — has no counterpart
   in the reference. For callers that cannot allocate device memory (an
   engine or renderer with a fixed GPU budget and its own allocator, a
   real-time thread that must not block on cudaMalloc/cudaFree): all pointers
   are device pointers the caller already owns — x, y, z, mass (n bodies, SoA),
   sys (n system ids, or NULL when all n bodies form one system), idx (m
   sample indices) and out (3*m doubles); the work is queued on the given
   cudaStream_t and not waited for. Body i is attracted by every other body j
   with sys[j] == sys[i] (all bodies when sys is NULL), mass <= 0 counting as
   0: the formula and system rule of cosmosim_direct_forces. A sample index
   outside [0, n) reads no body; its row of out is NaN. Scratch is a fixed
   1.5 MiB array inside the library, so m may be at most 4096 (larger m:
   CSG_ERR_BAD_ARG). The first call on each device looks up that array's
   address, so make it before any stream capture on that device; the address
   is cached per device and does not survive a cudaDeviceReset. Calls share
   the array: calls that overlap on the GPU race. */
CSG_EXPORT int csg_direct_forces_noalloc(const double *x, const double *y, const double *z,
                                         const double *mass, const int *sys, int n,
                                         const int *idx, int m, double G, double softening,
                                         double *out, void *stream);

/* ---- Adjoint of the kick-drift-kick leapfrog -------------------------------
   No counterpart in the reference. Differentiates a T-substep FP64 run
   (src/integrator.c:4-57: initial forces, then kick/drift/forces/kick) with
   respect to the initial positions and velocities, for the loss
   L = mean over alive bodies of |x_T - target|^2.
     CSG_ADJ_TREE    Barnes-Hut forces; each substep's interaction lists (the
                     reference walk's cells, depth-first order) are frozen:
                     the gradient is that of the run with those lists fixed;
     CSG_ADJ_DIRECT  FP64 direct-sum forces (every pair).
   The backward pass contracts the softened tidal tensor with the adjoint
   vector over the lists; memory is bounded by keeping positions and
   velocities every checkpoint_every substeps and recomputing each segment
   (bit-identically) before reversing it. */
typedef struct csg_adjoint csg_adjoint;
#define CSG_ADJ_TREE 0
#define CSG_ADJ_DIRECT 1

/* params: G, softening, theta, dt and substeps (= T) are used; sph must be 0.
   NULL on failure (csg_last_error). */
CSG_EXPORT csg_adjoint *csg_adjoint_create(int n, const CsgSimParams *params,
                                           int checkpoint_every, int mode);
CSG_EXPORT void csg_adjoint_destroy(csg_adjoint *adj);

/* Runs T substeps from bodies (their accelerations are recomputed), returns
   the loss against target (3n doubles, x y z per body) and, if final_out is
   not NULL, the final bodies. record = 1 also keeps every substep's tree and
   lists (T+1 sets) for csg_adjoint_forward_frozen. Blocking. */
CSG_EXPORT int csg_adjoint_forward(csg_adjoint *adj, const Body *bodies, const double *target,
                                   int record, double *loss, Body *final_out);

/* dL/dx_0 and dL/dv_0 of the last csg_adjoint_forward (3n doubles each, x y z
   per body). Blocking. */
CSG_EXPORT int csg_adjoint_backward(csg_adjoint *adj, double *grad_x, double *grad_v);

/* The loss of a run from other initial positions/velocities (same masses)
   with the recorded run's trees and interaction lists — the map whose
   gradient csg_adjoint_backward returns (for finite-difference checks).
   Needs a forward with record = 1; does not change what backward refers to. */
CSG_EXPORT int csg_adjoint_forward_frozen(csg_adjoint *adj, const Body *bodies,
                                          const double *target, double *loss);

/* Device memory held, the list entries (interactions) of the last forward,
   and the kernels launched so far. */
CSG_EXPORT int csg_adjoint_stats(csg_adjoint *adj, int64_t *device_bytes, int64_t *interactions,
                                 int64_t *launches);

/* ---- Quasar step on the GPU ---------------------------------------------------
   csg_quasar_step has the signature and semantics of the reference's
   quasar_step (src/quasar.h:29-34, src/quasar.c:477-509): accretion onto
   SMBHs, accretion rate / luminosity, radiation feedback, jet decay into
   lobes, recycling of distant jets, jet spawning; bodies may be appended up to
   n_alloc, *n and cfg->jet_count are updated. It runs on the calling thread's
   GPU state. The random generator state and the jet knot phase persist
   between calls as the reference's file statics do (src/quasar.c:11, :224);
   csg_quasar_seed sets them (the reference starts at 1 and 0). Handles in
   quasar mode run the same step on their resident bodies after every
   substep. */
CSG_EXPORT void csg_quasar_step(Body *bodies, int *n, int n_alloc, QuasarConfig *cfg, double dt);
CSG_EXPORT void csg_quasar_seed(uint64_t rng_state, int knot_phase);
/* The reference's defaults (src/quasar.c:37-57). */
CSG_EXPORT QuasarConfig csg_quasar_default_config(void);

/* Free-function parity mode: gravity with the reference's exact operation
   sequence (no fused multiply-add, 1/(r2*sqrt(r2))). Same signature as
   octree_compute_forces. */
CSG_EXPORT void csg_octree_compute_forces_exact(const OctreeNode *pool, int root, Body *bodies,
                                                int n, double G, double softening,
                                                double theta);

/* Seeded initial conditions following the reference generators
   (src/initial_conditions.c) with the benchmark configurations' parameters.
     kind 0: exponential-disk spiral, 20k default, disk mass 1, SMBH 0.01
     kind 1: two-disk merger, mass ratio 1:1.2, 50 deg tilt, 10% gas, SPH fields
     kind 2: Plummer bulge (30%, a = 0.5) + exponential disk (70%), total mass 1
     kind 3: one ensemble galaxy (scale length, SMBH fraction from seed)
     kind 4: two-disk merger, stars only
     kind 5: the merger's first disk alone (mass 1, R_d 1, SMBH 0.005), own frame
     kind 6: the merger's second disk alone (mass 1.2, R_d 1.3, SMBH 0.006),
             untilted, own frame (kinds 5 and 6 let a caller set the orbit)
   Returns the number of bodies written (n). */
CSG_EXPORT int csg_generate_ics(int kind, int n, uint64_t seed, Body *out);

/* The same initial conditions generated on the GPU into a device Body array
   (kinds 0, 3, 5 and 6: the single exponential disks). Each body draws the
   same random numbers as on the host (the generator is jumped ahead per run
   of bodies); log/exp/sin/cos are CUDA's, so positions and velocities agree
   to a few ulp, masses and types exactly. Returns n, or -1. Blocking. */
CSG_EXPORT int csg_generate_ics_device(int kind, int n, uint64_t seed, Body *device_out,
                                       void *stream);

/* An ensemble handle whose systems are generated on the GPU: system g has
   counts[g] bodies of csg_generate_ics kind `kind` (0, 3, 5 or 6) with seed
   seed0 + g. Otherwise as cosmosim_create_ensemble. */
CSG_EXPORT SimHandle cosmosim_create_ensemble_ics(int kind, int n_sys, const int *counts,
                                                  uint64_t seed0, const CsgSimParams *params);

#ifdef __cplusplus
}
#endif
#endif
