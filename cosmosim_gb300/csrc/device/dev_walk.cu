// dev_walk.cu — Barnes-Hut gravity walks (reference src/octree.c:171-234).
//
// Both walks give every body exactly the reference's interaction set: the
// cells it accepts by the monopole test (s*s)/d^2 < theta^2 with d^2 > 0, or
// reaches as leaves other than itself, in depth-first octant order.
//
// Traversal: one warp walks the preorder tree for 32 bodies that are
// neighbours in key order. The warp keeps one cursor; each lane keeps a single
// index `skip` below which it sleeps (it accepted an ancestor or the cell's
// subtree does not concern it). At a cell, active lanes take leaves, accept or
// ask to open; the cursor moves to id+1 (first child) if any active lane
// opens, else to the cell's `next`. Lanes that accepted the cell sleep until
// `next`. No stack, no divergent descent, per-lane depth-first order kept.
// The next 32 cells in preorder are staged per warp in shared memory with one
// coalesced load, and re-staged only when the cursor leaves that window.
//
// FP64 walk: the drop-in precision (k_walk64q). Openings decided as in the
//   FP32 walk (equal to the reference's FP64 rounding); interactions queued
//   and evaluated densely in FP64, 1/r^3 from an FP32 rsqrt seed refined to
//   full FP64 accuracy. k_walk64<EXACT=true> instead uses the reference's own
//   operation sequence per step (1/(r2*sqrt(r2)), no fused multiply-add) —
//   bit-identical results on the reference's own tree; used by parity tests.
// FP32-mixed walk: positions and centres as float hi/lo pairs (differences
//   keep ~48 bits), rsqrt/products in FP32, Kahan-compensated FP32 sums per
//   body. Openings within the FP32 error band of the threshold are decided in
//   FP64, so the interaction set equals the FP64 walk's.
#include "dev_internal.cuh"

namespace {

constexpr int WALK_THREADS = 256;
constexpr int WALK_WARPS = WALK_THREADS / CSG_WARP;

struct WalkArgs {
    const int *perm;
    const double *x, *y, *z;
    const NodeW64 *w64;
    const NodeW32 *w32;
    DevScalars *sc;
    double *ax, *ay, *az;
    double G, eps2, theta2, t2lo, t2hi;
    float Gf, eps2f, theta2f, guard_abs, guard_rel;
    int node_cap;
};

// Reference opening decision fl(s2/d2) < theta2 (src/octree.c:202-203),
// without a division unless s2 is within 2^-50 of theta2*d2.
__device__ __forceinline__ bool accept64(double s2, double d2, const WalkArgs &a)
{
    if (!(d2 > 0.0))
        return false;
    if (s2 < a.t2lo * d2)
        return true;
    if (s2 > a.t2hi * d2)
        return false;
    return __ddiv_rn(s2, d2) < a.theta2;
}

__device__ __forceinline__ double inv_r3_fast(double r2)
{
    if (r2 >= 1e-30 && r2 <= 1e30) {
        double y = (double)rsqrtf((float)r2);
        // Newton steps on y^-2 = r2: y += y/2 * (1 - r2*y*y)
        double e = fma(-r2 * y, y, 1.0);
        y = fma(0.5 * y, e, y);
        e = fma(-r2 * y, y, 1.0);
        y = fma(0.5 * y, e, y);
        return y * y * y;
    }
    return 1.0 / (r2 * sqrt(r2));
}

template <bool EXACT, bool STATS>
__global__ void __launch_bounds__(WALK_THREADS) k_walk64(WalkArgs a)
{
    __shared__ NodeW64 win_all[WALK_WARPS][CSG_WARP];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    NodeW64 *win = win_all[warp];
    const int n_alive = a.sc->n_alive;
    const long long p = (long long)blockIdx.x * WALK_THREADS + threadIdx.x;
    const long long warp0 = p - lane;
    if (warp0 >= n_alive)
        return;
    if (a.sc->n_nodes > a.node_cap || a.sc->n_nodes < 1)
        return; // no valid tree (capacity error already recorded)
    const int nn = a.sc->n_nodes;
    const bool valid = p < n_alive;
    const int me = valid ? a.perm[p] : -1;
    const double px = valid ? a.x[me] : 0.0, py = valid ? a.y[me] : 0.0,
                 pz = valid ? a.z[me] : 0.0;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    unsigned long long hits = 0;
    int skip = valid ? 0 : INT_MAX;
    int cur = 0, wbase = INT_MIN / 2;
    while (cur < nn) {
        if (cur - wbase >= CSG_WARP) {
            wbase = cur;
            __syncwarp();
            if (wbase + lane < nn)
                win[lane] = a.w64[wbase + lane];
            __syncwarp();
        }
        const NodeW64 c = win[cur - wbase];
        bool open = false;
        if (cur >= skip) {
            if (c.m == 0.0) { // empty cell: reference returns at once (src/octree.c:181-182)
                skip = c.next;
            } else {
                double dx, dy, dz, d2;
                if (EXACT) {
                    dx = __dsub_rn(c.cx, px);
                    dy = __dsub_rn(c.cy, py);
                    dz = __dsub_rn(c.cz, pz);
                    d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)),
                                   __dmul_rn(dz, dz));
                } else {
                    dx = c.cx - px;
                    dy = c.cy - py;
                    dz = c.cz - pz;
                    d2 = dx * dx + dy * dy + dz * dz;
                }
                bool take;
                if (c.body >= 0) {
                    take = (c.body != me);
                } else {
                    take = EXACT ? (d2 > 0.0 && __ddiv_rn(c.s2, d2) < a.theta2) : accept64(c.s2, d2, a);
                    if (take)
                        skip = c.next;
                    else
                        open = true;
                }
                if (take) {
                    if (EXACT) {
                        double r2 = __dadd_rn(d2, a.eps2);
                        double inv = __ddiv_rn(1.0, __dmul_rn(r2, __dsqrt_rn(r2)));
                        double gm = __dmul_rn(a.G, c.m);
                        sx = __dadd_rn(sx, __dmul_rn(__dmul_rn(gm, dx), inv));
                        sy = __dadd_rn(sy, __dmul_rn(__dmul_rn(gm, dy), inv));
                        sz = __dadd_rn(sz, __dmul_rn(__dmul_rn(gm, dz), inv));
                    } else {
                        double f = a.G * c.m * inv_r3_fast(d2 + a.eps2);
                        sx = fma(f, dx, sx);
                        sy = fma(f, dy, sy);
                        sz = fma(f, dz, sz);
                    }
                    if (STATS)
                        hits++;
                }
            }
        }
        const int nxt = __any_sync(0xffffffffu, open) ? cur + 1 : c.next;
        if (nxt <= cur) { // a malformed tree must not loop
            dev_fail(a.sc, CSG_ERR_WALK_LIMIT);
            break;
        }
        cur = nxt;
    }
    if (valid) {
        a.ax[me] = sx;
        a.ay[me] = sy;
        a.az[me] = sz;
    }
    if (STATS) {
        unsigned int h = __reduce_add_sync(0xffffffffu, (unsigned int)hits);
        if (lane == 0)
            atomicAdd(&a.sc->interactions, (unsigned long long)h);
    }
}

// 1/r^3 for the queued FP64 walk: FP32 rsqrt seed y0 (rel. error < 2^-21),
// e = 1 - r2*y0^2 exactly enough in FP64, then y = y0 (1 + e/2 + 3e^2/8)
// (the Taylor series of (1-e)^-1/2 to second order; residual < 2^-60).
__device__ __forceinline__ double inv_r3_q(double r2)
{
    if (r2 >= 1e-30 && r2 <= 1e30) {
        const double y0 = (double)rsqrtf((float)r2);
        const double e = fma(-r2 * y0, y0, 1.0);
        const double y = fma(y0 * e, fma(0.375, e, 0.5), y0);
        return y * y * y;
    }
    return 1.0 / (r2 * sqrt(r2));
}

// FP64 walk with dense evaluation. The traversal is the FP32 one below (its
// decisions equal the FP64 reference's, see k_walk32); accepted cells are
// pushed into per-lane FIFO queues in shared memory and evaluated in FP64 in
// batches where every lane has work, in the order they were accepted (the
// reference's depth-first order). The FP64 pipe then does useful work on
// (almost) every lane instead of once per traversal step for the few lanes
// that interact at that step.
constexpr int Q64 = 32; // queue slots per lane
constexpr int F64 = 8;  // entries per lane per dense batch

// Evaluates the lane's next `count` queued cells (count >= 0; lanes without a
// body pass 0 and never read their queue).
__device__ __forceinline__ void q64_eval(const WalkArgs &a, const int *q, int lane, int &head,
                                         int count, double px, double py, double pz,
                                         double &sx, double &sy, double &sz)
{
    count = max(count, 0);
    const int kmax = (int)__reduce_max_sync(0xffffffffu, (unsigned)count);
    for (int s = 0; s < kmax; s++) {
        if (s < count) {
            const int node = q[((head + s) & (Q64 - 1)) * CSG_WARP + lane];
            const double2 c01 = __ldg((const double2 *)&a.w64[node]);     // cx, cy
            const double2 c23 = __ldg((const double2 *)&a.w64[node] + 1); // cz, m
            const double4 c = make_double4(c01.x, c01.y, c23.x, c23.y);
            const double dx = c.x - px, dy = c.y - py, dz = c.z - pz;
            const double r2 = fma(dx, dx, fma(dy, dy, fma(dz, dz, a.eps2)));
            const double f = a.G * c.w * inv_r3_q(r2);
            sx = fma(f, dx, sx);
            sy = fma(f, dy, sy);
            sz = fma(f, dz, sz);
        }
    }
    head += count;
}

template <bool STATS>
__global__ void __launch_bounds__(WALK_THREADS) k_walk64q(WalkArgs a)
{
    __shared__ NodeW32 win_all[WALK_WARPS][CSG_WARP];
    __shared__ int q_all[WALK_WARPS][Q64 * CSG_WARP];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    NodeW32 *win = win_all[warp];
    int *q = q_all[warp];
    const int n_alive = a.sc->n_alive;
    const long long p = (long long)blockIdx.x * WALK_THREADS + threadIdx.x;
    const long long warp0 = p - lane;
    if (warp0 >= n_alive)
        return;
    if (a.sc->n_nodes > a.node_cap || a.sc->n_nodes < 1)
        return;
    const int nn = a.sc->n_nodes;
    const bool valid = p < n_alive;
    const int me = valid ? a.perm[p] : -1;
    const double px = valid ? a.x[me] : 0.0, py = valid ? a.y[me] : 0.0,
                 pz = valid ? a.z[me] : 0.0;
    const float hx = (float)px, hy = (float)py, hz = (float)pz;
    const float lx = (float)(px - (double)hx), ly = (float)(py - (double)hy),
                lz = (float)(pz - (double)hz);
    double sx = 0.0, sy = 0.0, sz = 0.0;
    int head = 0, tail = 0;
    unsigned long long hits = 0;
    int skip = valid ? 0 : INT_MAX;
    int cur = 0, wbase = INT_MIN / 2;
    while (cur < nn) {
        if (cur - wbase >= CSG_WARP) {
            wbase = cur;
            __syncwarp();
            if (wbase + lane < nn)
                win[lane] = a.w32[wbase + lane];
            __syncwarp();
        }
        const NodeW32 c = win[cur - wbase];
        bool open = false;
        if (cur >= skip) {
            if (c.m == 0.0f && a.w64[cur].m == 0.0) {
                skip = c.next;
            } else {
                bool take;
                if (c.body >= 0) {
                    take = (c.body != me);
                } else {
                    const float dx = (c.cx - hx) + (c.lx - lx);
                    const float dy = (c.cy - hy) + (c.ly - ly);
                    const float dz = (c.cz - hz) + (c.lz - lz);
                    const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    const float lhs = a.theta2f * d2;
                    const float band = c.s2 * a.guard_rel;
                    if (c.s2 < lhs - band && d2 > 0.f) {
                        take = true;
                    } else if (c.s2 > lhs + band) {
                        take = false;
                    } else {
                        const NodeW64 e = a.w64[cur];
                        const double ex = e.cx - px, ey = e.cy - py, ez = e.cz - pz;
                        take = accept64(e.s2, ex * ex + ey * ey + ez * ez, a);
                    }
                    if (take)
                        skip = c.next;
                    else
                        open = true;
                }
                if (take) {
                    q[(tail & (Q64 - 1)) * CSG_WARP + lane] = cur;
                    tail++;
                    if (STATS)
                        hits++;
                }
            }
        }
        const int cnt = tail - head; // 0..Q64-1; always 0 for a lane without a body
        const int cmin = (int)__reduce_min_sync(0xffffffffu, (unsigned)(valid ? cnt : INT_MAX));
        const int cmax = (int)__reduce_max_sync(0xffffffffu, (unsigned)cnt);
        if (cmin >= F64)
            q64_eval(a, q, lane, head, valid ? F64 : 0, px, py, pz, sx, sy, sz);
        else if (cmax >= Q64 - 1) // a lane is about to overflow: drain what is there
            q64_eval(a, q, lane, head, min(cnt, F64), px, py, pz, sx, sy, sz);
        const int nxt = __any_sync(0xffffffffu, open) ? cur + 1 : c.next;
        if (nxt <= cur) {
            dev_fail(a.sc, CSG_ERR_WALK_LIMIT);
            break;
        }
        cur = nxt;
    }
    while (__any_sync(0xffffffffu, tail - head > 0))
        q64_eval(a, q, lane, head, min(tail - head, F64), px, py, pz, sx, sy, sz);
    if (valid) {
        a.ax[me] = sx;
        a.ay[me] = sy;
        a.az[me] = sz;
    }
    if (STATS) {
        unsigned int hsum = __reduce_add_sync(0xffffffffu, (unsigned int)hits);
        if (lane == 0)
            atomicAdd(&a.sc->interactions, (unsigned long long)hsum);
    }
}

__device__ __forceinline__ void kahan_add(float &s, float &c, float v)
{
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}

template <bool STATS>
__global__ void __launch_bounds__(WALK_THREADS) k_walk32(WalkArgs a)
{
    __shared__ NodeW32 win_all[WALK_WARPS][CSG_WARP];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    NodeW32 *win = win_all[warp];
    const int n_alive = a.sc->n_alive;
    const long long p = (long long)blockIdx.x * WALK_THREADS + threadIdx.x;
    const long long warp0 = p - lane;
    if (warp0 >= n_alive)
        return;
    if (a.sc->n_nodes > a.node_cap || a.sc->n_nodes < 1)
        return; // no valid tree (capacity error already recorded)
    const int nn = a.sc->n_nodes;
    const bool valid = p < n_alive;
    const int me = valid ? a.perm[p] : -1;
    const double px = valid ? a.x[me] : 0.0, py = valid ? a.y[me] : 0.0,
                 pz = valid ? a.z[me] : 0.0;
    const float hx = (float)px, hy = (float)py, hz = (float)pz;
    const float lx = (float)(px - (double)hx), ly = (float)(py - (double)hy),
                lz = (float)(pz - (double)hz);
    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    unsigned long long hits = 0;
    int skip = valid ? 0 : INT_MAX;
    int cur = 0, wbase = INT_MIN / 2;
    while (cur < nn) {
        if (cur - wbase >= CSG_WARP) {
            wbase = cur;
            __syncwarp();
            if (wbase + lane < nn)
                win[lane] = a.w32[wbase + lane];
            __syncwarp();
        }
        const NodeW32 c = win[cur - wbase];
        bool open = false;
        if (cur >= skip) {
            if (c.m == 0.0f && a.w64[cur].m == 0.0) {
                skip = c.next;
            } else {
                const float dx = (c.cx - hx) + (c.lx - lx);
                const float dy = (c.cy - hy) + (c.ly - ly);
                const float dz = (c.cz - hz) + (c.lz - lz);
                const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                bool take;
                if (c.body >= 0) {
                    take = (c.body != me);
                } else {
                    // |theta^2 d^2 - s^2| inside the FP32 error band -> decide in FP64
                    const float lhs = a.theta2f * d2;
                    const float band = c.s * a.guard_abs + c.s2 * a.guard_rel;
                    if (c.s2 < lhs - band && d2 > 0.f) {
                        take = true;
                    } else if (c.s2 > lhs + band) {
                        take = false;
                    } else {
                        const NodeW64 e = a.w64[cur];
                        const double ex = e.cx - px, ey = e.cy - py, ez = e.cz - pz;
                        take = accept64(e.s2, ex * ex + ey * ey + ez * ez, a);
                    }
                    if (take)
                        skip = c.next;
                    else
                        open = true;
                }
                if (take) {
                    const float y = rsqrtf(d2 + a.eps2f);
                    const float f = a.Gf * c.m * (y * y * y);
                    kahan_add(sx, cx, f * dx);
                    kahan_add(sy, cy, f * dy);
                    kahan_add(sz, cz, f * dz);
                    if (STATS)
                        hits++;
                }
            }
        }
        const int nxt = __any_sync(0xffffffffu, open) ? cur + 1 : c.next;
        if (nxt <= cur) {
            dev_fail(a.sc, CSG_ERR_WALK_LIMIT);
            break;
        }
        cur = nxt;
    }
    if (valid) {
        a.ax[me] = (double)sx + (double)(-cx);
        a.ay[me] = (double)sy + (double)(-cy);
        a.az[me] = (double)sz + (double)(-cz);
    }
    if (STATS) {
        unsigned int h = __reduce_add_sync(0xffffffffu, (unsigned int)hits);
        if (lane == 0)
            atomicAdd(&a.sc->interactions, (unsigned long long)h);
    }
}

// Dead bodies get a = 0 (src/octree.c:226-230); alive ones are overwritten by
// the walk.
__global__ void k_zero_acc(const double *__restrict__ m, double *ax, double *ay, double *az, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    if (m[i] <= 0.0) {
        ax[i] = 0.0;
        ay[i] = 0.0;
        az[i] = 0.0;
    }
}

} // namespace

// Host mirror of the scalars needed to size the FP32 error band.
extern "C" int csgd_gravity_ex(csgd_t *d, const csgd_force_params *p, int exact)
{
    const int n = d->n;
    if (n <= 0)
        return CSG_OK;
    WalkArgs a;
    a.perm = d->perm;
    a.x = d->x;
    a.y = d->y;
    a.z = d->z;
    a.w64 = d->w64;
    a.w32 = d->w32;
    a.sc = d->sc;
    a.ax = d->ax;
    a.ay = d->ay;
    a.az = d->az;
    a.G = p->G;
    a.eps2 = p->softening * p->softening;
    a.theta2 = p->theta * p->theta;
    a.t2lo = a.theta2 * (1.0 - 0x1p-50);
    a.t2hi = a.theta2 * (1.0 + 0x1p-50);
    a.Gf = (float)p->G;
    a.eps2f = (float)a.eps2;
    a.theta2f = (float)a.theta2;
    // FP32 error band: |d| is exact to ~2^-46 |coordinates| (hi/lo pairs), d^2
    // to a few FP32 ulps; 2^-19 relative covers both with a wide margin.
    a.guard_abs = 0.0f;
    a.guard_rel = 0x1p-19f * (1.0f + a.theta2f);
    a.node_cap = d->node_cap;
    cudaStream_t s = d->stream;
    { k_zero_acc<<<csgd_grid(n, 256), 256, 0, s>>>(d->m, d->ax, d->ay, d->az, n); d->launches++; }
    const int g = csgd_grid(n, WALK_THREADS);
    if (p->precision == CSG_PREC_FP32_MIXED && !exact) {
        if (d->stats)
            { k_walk32<true><<<g, WALK_THREADS, 0, s>>>(a); d->launches++; }
        else
            { k_walk32<false><<<g, WALK_THREADS, 0, s>>>(a); d->launches++; }
    } else if (exact) {
        if (d->stats)
            { k_walk64<true, true><<<g, WALK_THREADS, 0, s>>>(a); d->launches++; }
        else
            { k_walk64<true, false><<<g, WALK_THREADS, 0, s>>>(a); d->launches++; }
    } else {
        if (d->stats)
            { k_walk64q<true><<<g, WALK_THREADS, 0, s>>>(a); d->launches++; }
        else
            { k_walk64q<false><<<g, WALK_THREADS, 0, s>>>(a); d->launches++; }
    }
    return csgd_check(d, cudaGetLastError());
}

extern "C" int csgd_gravity(csgd_t *d, const csgd_force_params *p)
{
    return csgd_gravity_ex(d, p, 0);
}
