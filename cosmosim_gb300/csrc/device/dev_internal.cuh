// dev_internal.cuh — device state and node layouts shared by the .cu files.
//
// Tree layout (all arrays indexed by node id; ids are depth-first preorder):
//   a node's first child is id+1 and the node after its subtree is `next`, so
//   a walk that either descends (id+1) or skips (next) visits cells in the
//   reference's depth-first octant order 0..7 (src/octree.c:213-217) with no
//   stack at all.
//   NodeW64  — FP64 walk record: centre of mass, mass, opening size s^2, next, body
//   NodeW32  — FP32 walk record: the same in FP32 (mass-weighted centre rounded)
//   geo      — geometric centre and half size (SPH neighbour search, export)
//   link     — parent, level, first sorted body, body count
//   child    — 8 child ids per node in octant order (export, moments)
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "csg_device.h"

#define CSG_WARP 32
#define CSG_MAX_LEVEL 64  // reference src/octree.c:5 (MAX_DEPTH)
#define CSG_KEY_LEVELS 21 // levels held by the 63-bit primary key
#define CSG_DEAD_KEY 0xFFFFFFFFFFFFFFFFull

struct __align__(16) NodeW64 {
    double cx, cy, cz, m;
    double s2;      // (2 * half_size)^2, the reference's s*s (src/octree.c:202-203)
    int next;       // id after this subtree
    int body;       // caller body index for a leaf, -1 for an internal cell
};

// FP32 walk record: the centre of mass is held as a float hi/lo pair so that
// body-to-cell differences keep ~48 bits; everything after the difference is
// FP32 (rsqrt, products, compensated sums).
struct __align__(16) NodeW32 {
    float cx, cy, cz, m;    // hi parts of the centre of mass, mass
    float lx, ly, lz, s2;   // lo parts (centre - hi), s^2
    int next;
    int body;
    float s;                // 2 * half_size
    float pad;
};

// FP32 neighbour-search record: the cell cube, and for a leaf its body
// position and index (body -1 for internal cells, -2 for a leaf whose body is
// dead, -3 for a leaf that names no body). cmax = max |centre| + half size bounds the FP32
// rounding of box tests.
struct __align__(16) NodeS32 {
    float cx, cy, cz, hs;
    float bx, by, bz;
    int body;
    int next;
    float cmax;
    int pad0, pad1;
};

struct __align__(16) NodeLink {
    int parent;
    int level;
    int first;  // first sorted position of the cell's bodies
    int count;  // number of bodies in the cell
};

// One system of the forest (a single simulation is a forest of one): its
// alive-body bounding box, root cube, key parameters, where its bodies sit in
// the sorted order and where its cells sit in the preorder node array.
struct DevRoot {
    unsigned long long omin[3], omax[3]; // order-preserving bbox encodings
    double c0[3];                        // root centre
    double hs0;                          // root half size
    double key_scale;                    // 2^52 / hs0: key grid units x 2^32 (fast key path)
    double key_off[3];                   // (2^20 - c0 * 2^20 / hs0) x 2^32
    long long key_tol;                   // fast-path guard, in units of 2^-32 grid cells
    int fast_keys;                       // 1 when the fast key path is safe
    int n_alive;                         // alive bodies of this system
    int first;                           // their first sorted position
    int root;                            // preorder id of the root cell
    int end;                             // one past the system's last cell
    int pad;
};

// A walk task: up to 32 consecutive sorted bodies of one system (one warp).
struct WalkTask {
    int gal, pos0, count, pad;
};

// Per-build scalars kept on the device so that no step needs a host round trip.
struct DevScalars {
    int n_tasks;       // walk tasks of the current tree
    int task_next;     // persistent walks: next task to take
    int n_alive;
    int n_nodes;
    int deep;                            // positions that share a 63-bit key
    int err;                             // first device error code (0 = none)
    int n_gas;
    int pad0;
    unsigned long long interactions;     // walk statistics (when enabled)
    unsigned long long walk_steps;       // warp traversal steps
    unsigned long long walk_active;      // lane-steps of lanes still walking
    unsigned long long key_slow;         // bodies that took the exact key path
    int alive_count;                     // csgd_alive_count result
};

// Quasar step state kept on the device between steps (the reference keeps
// the generator state and the knot phase in file statics, src/quasar.c:11
// and :224; the live jet count in its QuasarConfig), and the counters one
// step passes between its stages.
struct QuasarState {
    unsigned long long rng;
    int knot_phase;
    int jet_count;
    int n;      // bodies in use (the step appends jets and lobes)
    int n_smbh; // bodies of type SMBH found by the current step
    double swallowed; // mass accreted this step, summed in accretion order
    int expired;      // jets whose lifetime ran out this step
    int n_events;     // accretion events of the current SMBH
    int spawns;       // jet spawns that happen this step
    int spawned;      // bodies they add
    int err;          // CSG_* code; the step changed nothing when set
};

// ---- xorshift64 jump-ahead ----------------------------------------------------
// The generator (Marsaglia xorshift, shifts 13/7/17) is linear over GF(2): one
// step is a 64x64 bit matrix M, so the state k draws ahead is M^k s. The table
// holds M^(2^b) by columns (col[b][j] = M^(2^b) e_j); a jump applies one
// column sum per set bit of k.
constexpr int XS_JUMP_LEVELS = 40;
struct XsJumpTable {
    unsigned long long col[XS_JUMP_LEVELS][64];
};
const XsJumpTable &xs_jump_table_host(); // built once per process (dev_ics.cu)

__host__ __device__ inline unsigned long long xs_apply(const unsigned long long *col,
                                                       unsigned long long s)
{
    unsigned long long r = 0;
    for (int j = 0; j < 64; j++)
        if ((s >> j) & 1ull)
            r ^= col[j];
    return r;
}

__device__ inline unsigned long long xs_jump(const XsJumpTable *t, unsigned long long s,
                                             unsigned long long k)
{
    for (int lv = 0; k; lv++, k >>= 1)
        if (k & 1ull)
            s = xs_apply(t->col[lv], s);
    return s;
}

struct csgd {
    cudaStream_t stream;
    cudaStream_t own_stream;
    cudaStream_t aux;             // SPH runs here beside the gravity walk
    cudaEvent_t ev_fork, ev_join; // (timing disabled)
    cudaStream_t aux2;            // pool export beside the walk (free functions)
    cudaEvent_t ev_fork2, ev_join2;
    OctreeNode *export_dst; // set: substeps also export their tree here (device view)
    int export_cap;         // capacity of export_dst, cells
    int n;        // bodies in use
    int cap;      // body capacity
    int node_cap; // node capacity (8*cap + 64)
    int stats;
    int host_err; // first error seen on the host side (launch, allocation)
    int wait_polls; // limit of the bounded device waits (0: the default, 2^22 polls)
    // phase timing (csgd_set_phase_timing): events between the phases of a
    // substep on the main stream (tev); around SPH on its stream and at the
    // main stream's rejoin (taux); sums of the phase times so far
    int timing;
    cudaEvent_t tev[7], taux[3];
    double phase_ms[7]; // kick+drift, build, gravity, SPH, kick, cooling, substep
    long long timed_substeps;
    // the build's own parts (keys, sort, cells, moments, the rest), between
    // events bev[0..5] recorded by csgd_build_tree while timing
    cudaEvent_t bev[6];
    double build_ms[5];
    unsigned long long launches; // kernels launched on this state (measurement)

    // bodies, caller index order
    double *x, *y, *z, *vx, *vy, *vz, *ax, *ay, *az, *m;
    double *rho, *P, *u, *h;
    int *type;
    Body *aos;        // Body staging for host I/O
    OctreeNode *pool; // reference-layout staging for export/import

    // forest: system id of every body (caller order) and of every sorted
    // position; per-system roots; walk tasks
    int n_gal;
    int gal_cap;
    int *gid, *sgid;
    DevRoot *roots;
    // bodies per system of an ensemble (device, gal_cap ints) and their
    // least and largest count; a single system has d->n bodies
    int *sys_n;
    int sys_min_n, sys_max_n;
    WalkTask *tasks;
    int task_cap;
    // walk launch shape: warps per block (4 or 8), task group (0 = one warp
    // per task, else tasks taken from an atomic counter this many at a time)
    // and, for the persistent form, blocks per SM
    int walk_warps, walk_group, walk_bps;
    int num_sms;
    int export_order; // builds also keep what pool export needs (two lowest indices per cell)
    int minidx_valid; // the current tree has them

    // keys and sort
    unsigned long long *key, *key_alt;
    int *perm, *perm_alt;
    unsigned long long *ext; // 3 words per sorted position (deep cells only)
    unsigned int *sort_hist;
    int sort_hist_cap;

    // per sorted position
    signed char *lcp;  // lcp with the next position, in levels (-1 at the end)
    int *cnt, *base;   // node counts and their exclusive scan (cap+1)
    int *scan_tmp;
    int scan_tmp_cap;
    int *gas;          // gas bodies in key order (caller indices)
    int *nb;           // SPH neighbour lists, 128 slots x cap (slot-major)
    int *nb_count;
    double *pr2, *cs; // SPH per-body force terms
    double *sph_term; // SPH pair terms, 3 x 128 x cap (slot-major)
    int *sph_relist;  // per gas slot: 1 when the density pass changed h
    int nb_cap;

    // nodes
    NodeW64 *w64;
    NodeW32 *w32;
    NodeLink *link;
    double4_32a *geo;
    NodeS32 *s32;
    int *child;   // 8 per node
    int *nchild;
    int *ticket;
    int2 *minidx; // two smallest caller indices below each cell (export order)
    unsigned long long *ord_key, *ord_key_alt;
    int *ord_id, *ord_id_alt, *rank;

    DevScalars *sc;      // device
    DevScalars *sc_host; // pinned mirror
    int *h_int;          // pinned scratch for single values read back (4 ints)
    QuasarState *qs;     // device, allocated by the first quasar step
    double *wpart;       // FP32 walk units' partial sums, 24 x wpart_cap doubles
    int wpart_cap;
    void *q_scratch;     // device scratch of the quasar step (dev_quasar.cu)
    int q_scratch_cap;   // bodies it is sized for
    int geometry_valid;
    // captured substep (cosmosim_substeps_async path)
    cudaGraphExec_t graph;
    unsigned long long graph_launches; // kernels in one replay
    double graph_key[4];               // dt, G, softening, theta it was captured for
    int graph_prec, graph_sph, graph_n;
    cudaStream_t graph_stream;
    OctreeNode *graph_export;
    int graph_export_cap;
    int use_graphs;
    int imported;  // the tree came from a caller pool (no sorted order)
    int gas_valid; // d->gas / n_gas match the current tree
};

// ---- helpers shared by the .cu files ----
// Event k of the build's parts (timing only; see csgd::bev).
void csgd_build_mark(csgd_t *d, int k);
// Every device and pinned-host allocation of the library goes through these
// two. Fault injection (csg_inject_alloc_failure) can make them fail: the
// next `k` allocations succeed, every later one returns
// cudaErrorMemoryAllocation until the injection is cleared.
cudaError_t csgd_malloc(void **p, size_t bytes);
cudaError_t csgd_malloc_host(void **p, size_t bytes);
int csgd_check(csgd_t *d, cudaError_t e);
void csgd_drop_graph(csgd_t *d); // destroys the captured substep (after a sync)
// allocates the cell geometry (geo, s32) and/or the pool staging on first use
extern "C" int csgd_ensure_tree_extras(csgd_t *d, int geometry, int pool);
void csgd_set_err(csgd_t *d, int code);
int csgd_grid(long long n, int block);

// ---- programmatic dependent launch ----
// csgd_launch queues a kernel whose blocks may be scheduled while the kernel
// before it in the stream still runs, so a chain of short kernels does not
// pay each launch after the previous kernel's end. Every kernel queued this
// way begins with pdl_wait(), which returns once the previous kernel has
// completed and its writes are visible, before any global memory access;
// pdl_release() then lets the next kernel's blocks be scheduled. Both are
// no-ops in a kernel launched without the attribute. The tree build and its
// sort and scans launch this way; the walks, kicks and SPH passes do not (the
// 100k merger substep, SPH on its own stream beside the walk, went from 1.11
// to 1.14 ms when they did, likely because blocks scheduled early and waiting
// hold SM slots the other stream's kernels could use).
__device__ __forceinline__ void pdl_wait()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
}
__device__ __forceinline__ void pdl_release()
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_enter()
{
    pdl_wait();
    pdl_release();
}
template <typename... P, typename... A>
inline void csgd_launch(csgd_t *d, void (*k)(P...), int grid, int block, cudaStream_t s,
                        A &&...args)
{
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k, static_cast<A &&>(args)...);
    d->launches++;
}

// ---- sort / scan utilities (dev_sort.cu) ----
// Stable LSD radix sort of (key, value) over n items, on key bits [0, bits).
// Result in (key, val); alt buffers are scratch of the same size. With n_dev
// the item count is min(n, *n_dev), read on the device (no host round trip;
// the launches are sized for n).
int csg_radix_sort(csgd_t *d, unsigned long long *key, int *val, unsigned long long *key_alt,
                   int *val_alt, int n, int bits, const int *n_dev = nullptr);
// Exclusive scan of in[0..n) into out[0..n], out[n] = total. count_limit, when
// non-NULL, is a device int: items at positions >= *count_limit count as 0.
int csg_scan_exclusive(csgd_t *d, const int *in, int *out, int n, const int *count_limit);

// Polls a bounded device wait makes before it gives up (csgd::wait_polls).
constexpr int CSG_WAIT_POLLS_DEFAULT = 1 << 22;
// The walks split each task by the root's children when there are few tasks
// for the GPU: up to 12 per SM (about 58k bodies on 152 SMs). Above that the
// whole-task walk already fills the SMs and the split only adds root-level
// work. The FP32 walk decides per launch (both forms give the same bits); the
// FP64 walk per system, by its body count (the forms sum differently, and a
// system must come out the same alone and in an ensemble).
inline bool csgd_walk_split(const csgd_t *d)
{
    return (long long)d->n / 32 + d->n_gal + 1 <= 12LL * d->num_sms;
}
inline long long csgd_split_max_bodies(const csgd_t *d) { return 12LL * 32 * d->num_sms; }
inline int csgd_sys_min_n(const csgd_t *d) { return d->n_gal > 1 ? d->sys_min_n : d->n; }
inline int csgd_sys_max_n(const csgd_t *d) { return d->n_gal > 1 ? d->sys_max_n : d->n; }
// Scratch of the split walks, allocated on first use outside any capture
// when `precision` and the size call for it; CSG_OK or CSG_ERR_NOMEM.
int csgd_prepare_walk(csgd_t *d, int precision);
inline int csgd_wait_polls(const csgd_t *d)
{
    return d->wait_polls > 0 ? d->wait_polls : CSG_WAIT_POLLS_DEFAULT;
}

// ---- device error codes written to DevScalars::err ----
__device__ __forceinline__ void dev_fail(DevScalars *sc, int code) { atomicCAS(&sc->err, 0, code); }

// FP32 value of a positive double whose exponent lies in FP32's normal range,
// from its bits alone (exponent rebased from 1023 to 127, mantissa truncated
// to 23 bits: relative error < 2^-23). Integer operations only: conversion
// instructions would run on the FP64 pipe, the bottleneck of the FP64 force
// kernels on this GPU.
__device__ __forceinline__ float f32_from_f64_bits(long long b)
{
    return __int_as_float((int)((b >> 29) - (896LL << 23)));
}

// y^2 (exact: 48 significant bits) and y^3 (rounded to nearest, < 2^-53
// relative error) as doubles, for a positive normal float 2^-60 < y < 2^60,
// by integer multiplies of y's 24-bit significand Y (y = Y 2^(ey-150)):
// no FP64 operations. Y^2 lies in [2^46, 2^48): shifted so its leading bit
// sits at bit 52, added to (biased exponent - 1) << 52 (the leading bit
// supplies the missing 1). Y^3 / 2^8 (the high word of (Y 2^40)(Y^2 2^16))
// lies in [2^61, 2^64): rounded to 53 bits the same way (a carry out of the
// significand moves into the exponent, as it should).
__device__ __forceinline__ void pow23_from_f32(float y, double &y2, double &y3)
{
    const unsigned yb = __float_as_uint(y);
    const unsigned Y = (yb & 0x7fffffu) | 0x800000u;
    const long long ey = (long long)(yb >> 23);
    const unsigned long long S = (unsigned long long)Y * Y;
    const unsigned t = (unsigned)(S >> 47); // 1: leading bit at 47
    y2 = __longlong_as_double(((2 * ey + 768 + t) << 52) + (long long)(S << (6 - t)));
    const unsigned long long hi = __umul64hi((unsigned long long)Y << 40, S << 16);
    const int lz = __clz((unsigned)(hi >> 32)); // 0..2
    const int sh = 11 - lz;
    const unsigned long long M = (hi + (1ull << (sh - 1))) >> sh;
    y3 = __longlong_as_double(((3 * ey + 643 - lz) << 52) + (long long)M);
}

// m r^-3 by integer arithmetic only, for r2 = r^2 in [2^-99, 2^100) and m a
// positive normal double with biased exponent in [160, 1887] (then every
// step below stays in range and the result is a normal double), from the
// FP32 seed y0 of r^-1 (|1 - r2 y0^2| < 2^-20). With y0 = Y 2^(ey-150)
// (Y its 24-bit significand), S = Y^2 and r2 = Mr 2^(er-1075):
//   e = 1 - r2 y0^2 = 1 - Mr S / 2^K, K = 1375 - er - 2 ey in [98, 101]:
//       Mr S is one 53 x 48-bit product (128 bits); e 2^64 is the
//       difference 2^K - Mr S shifted right by K - 64 (|e 2^64| < 2^45);
//   c = (1-e)^-3/2 = 1 + 3/2 e + 15/8 e^2 (next term < 2^-58) in 62-bit
//       fixed point;
//   m y0^3 c = Mm Y^3 C 2^(em + 3 ey - 1587): Y^3 2^-8 (the high word of
//       (Y 2^40)(S 2^16)), times 2C, times Mm 2^11, each keeping the high
//       64 bits, leaves Q in [2^58, 2^63.1), rounded to 53 bits and packed
//       with its exponent (a carry out of the significand moves into the
//       exponent).
// Relative error < 1.01 x 2^-53 (one rounding; the truncated high words and
// series add < 2^-57).
__device__ __forceinline__ double m_r3_from_seed(long long rb, long long mb, float y0)
{
    const unsigned long long MANT = 0xfffffffffffffull, HID = 1ull << 52;
    const unsigned yb = __float_as_uint(y0);
    const unsigned Y = (yb & 0x7fffffu) | 0x800000u;
    const long long ey = (long long)(yb >> 23);
    const unsigned long long S = (unsigned long long)Y * Y;
    const unsigned long long Mr = ((unsigned long long)rb & MANT) | HID;
    const unsigned long long L = Mr * S, H = __umul64hi(Mr, S);
    const int sh = (int)(1375 - 64 - (rb >> 52) - 2 * ey); // K - 64, 34..37
    const long long Dhi = (1LL << sh) - (long long)H - (L != 0ull);
    const unsigned long long Dlo = 0ull - L;
    const long long E64 = (long long)(((unsigned long long)Dhi << (64 - sh)) | (Dlo >> sh));
    const unsigned long long aE = (unsigned long long)(E64 < 0 ? -E64 : E64);
    const long long C = (1LL << 62) + ((3 * E64) >> 3) + (long long)((15ull * __umul64hi(aE, aE)) >> 5);
    const unsigned long long hi3 = __umul64hi((unsigned long long)Y << 40, S << 16);
    const unsigned long long Z = __umul64hi(hi3, (unsigned long long)C << 1);
    const unsigned long long Q = __umul64hi((((unsigned long long)mb & MANT) | HID) << 11, Z);
    const int lz = __clz((unsigned)(Q >> 32)); // 0..5
    const int s = 11 - lz;
    const unsigned long long M = (Q + (1ull << (s - 1))) >> s;
    return __longlong_as_double((((mb >> 52) + 3 * ey - 378 - lz) << 52) + (long long)M);
}

// w = 3/2 e + 15/8 e^2 = e c, c = 3/2 + 15/8 e, the series term of
// (1-e)^-3/2 - 1, for |e| < 2^-7 (the seeds give |e| < 2^-20), by integer
// arithmetic: c in 62-bit fixed point (C in [2^62, 2^63)), times e's 53-bit
// significand by one 64 x 64 -> high-64 multiply, rounded to 53 bits (w
// within 2^-53 relative, plus < 2^-60 from truncations). For |e| < 2^-63,
// w = 0 (then w < 2^-62: below the result's rounding). Keeps the series off
// the FP64 pipe.
__device__ __forceinline__ double r3_series_w(double e)
{
    const long long eb = __double_as_longlong(e);
    const long long ee = (eb >> 52) & 0x7ff;
    const unsigned long long Em = ((unsigned long long)eb & 0xfffffffffffffull) | (1ull << 52);
    const int s = (int)min(max(1016 - ee, 0LL), 63LL);
    const unsigned long long T = (15ull * Em) >> s; // 15/8 |e| 2^62, < 2^57
    const unsigned long long C = eb < 0 ? (3ull << 61) - T : (3ull << 61) + T;
    const unsigned long long R = __umul64hi(Em << 11, C << 1); // [2^62, 2^64)
    const int lz = __clz((unsigned)(R >> 32));                 // 0 or 1
    const int sh = 11 - lz;
    const unsigned long long M = (R + (1ull << (sh - 1))) >> sh;
    const long long w = (eb & (1LL << 63)) | (((ee - lz) << 52) + (long long)M);
    return ee < 960 ? 0.0 : __longlong_as_double(w);
}

// r^-3 and r^-5 for r2 = r^2 without divisions: y0 = FP32 rsqrt seed (rel.
// error < 2^-21; y0^2 and y0^3 by pow23_from_f32), e = 1 - r2 y0^2 (one
// fused multiply-add), then r^-2 = y0^2 (1 + e + e^2) and
// r^-3 = y0^3 (1 + 3/2 e + 15/8 e^2) (the binomial series; the first omitted
// terms are < 2^-60). Outside 2^-99 <= r2 < 2^100 the plain expressions.
__device__ __forceinline__ void inv_r3_r5(double r2, double &inv3, double &inv5)
{
    const long long bits = __double_as_longlong(r2);
    if ((unsigned long long)((bits >> 52) - 924) <= 198ull) {
        double y0sq, y3;
        pow23_from_f32(rsqrtf(f32_from_f64_bits(bits)), y0sq, y3);
        const double e = fma(-r2, y0sq, 1.0);
        inv3 = fma(y3, r3_series_w(e), y3);
        const double inv2 = fma(y0sq, fma(e, e, e), y0sq);
        inv5 = inv3 * inv2;
        return;
    }
    inv3 = 1.0 / (r2 * sqrt(r2));
    inv5 = inv3 / r2;
}
