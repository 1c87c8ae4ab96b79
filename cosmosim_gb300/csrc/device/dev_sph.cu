// dev_sph.cu — SPH density/pressure and forces on the shared octree
// (reference src/sph.c:45-196) and the neighbour query of
// src/octree.c:236-318.
//
// Neighbour order matters: the reference keeps the first 128 bodies within
// the radius in depth-first octant order (src/octree.c:260-277, sph.h:9), and
// the cap binds often. Walking the preorder tree with per-lane subtree skips
// (as in dev_walk.cu) meets the leaves in exactly that order. Each pass runs in
// two kernels: the walk records every gas body's capped list, then a pair
// kernel sums over the lists in that order — the FP64 pair arithmetic then
// runs densely, one lane per gas body, instead of once per walk step for
// whichever lanes found a neighbour. Lanes are the gas bodies in key order.
// Its divisions and square roots (about ten FP64 operations each with the
// compiler's operators, on a GPU whose FP64 rate is 1/64 of FP32) run on the
// integer pipes (div_rn, sqrt_rn): correctly rounded, so bit-identical.
//
// Compiled with -fmad=false, with the reference's operation order, so for the
// same inputs every sum rounds as the reference's does.
#include "dev_fpint.cuh"
#include "dev_internal.cuh"

namespace {

constexpr int SPH_THREADS = 128;
constexpr int SPH_WARPS = SPH_THREADS / CSG_WARP;
constexpr double GAMMA = 5.0 / 3.0;
constexpr double PI_D = 3.14159265358979323846;

// M4 cubic spline W(r, h), src/sph.c:11-25, with its normalisation 8/(pi h^3)
// computed by the caller once per gas body (the same expression, so the same
// value): one division fewer per pair.
__device__ __forceinline__ double kernel_W_norm(double r, double h, double norm)
{
    if (h < 1e-10)
        return 0.0;
    double q = div_rn(r, h);
    if (q > 1.0)
        return 0.0;
    if (q <= 0.5)
        return norm * (1.0 - 6.0 * q * q + 6.0 * q * q * q);
    double t = 1.0 - q;
    return norm * 2.0 * t * t * t;
}

__device__ __forceinline__ double kernel_norm(double h) { return div_rn(8.0, PI_D * h * h * h); }

// the kernel's radial derivative dW/dr(r, h), src/sph.c:27-41
__device__ __forceinline__ double kernel_dWdr(double r, double h)
{
    if (h < 1e-10)
        return 0.0;
    double q = div_rn(r, h);
    if (q > 1.0 || r < 1e-15)
        return 0.0;
    double norm = div_rn(8.0, PI_D * h * h * h);
    if (q <= 0.5)
        return div_rn(norm * (-12.0 * q + 18.0 * q * q), h);
    double t = 1.0 - q;
    return div_rn(norm * (-6.0 * t * t), h);
}

struct SphArgs {
    const int *gas;
    const double *x, *y, *z, *vx, *vy, *vz, *m;
    const int *type;
    double *h, *rho, *P, *u;
    double *ax, *ay, *az;
    const double4_32a *geo;
    const NodeS32 *s32;
    const NodeW64 *w64;
    DevScalars *sc;
    int *nb;       // neighbour lists, slot-major
    int *nb_count; // neighbours per gas body
    int *relist;   // per gas body: the density pass changed h (search again)
    int reuse;     // force pass: keep the density lists of bodies with relist 0
    int density;   // density pass (the lists also store 8/(pi h^3) in pr2)
    double *pr2, *cs; // per-body force terms (k_sph_body_terms)
    double *term;     // pair terms, 3 planes of 128 slots x stride (slot-major)
    int n, node_cap, stride;
};

// ---- neighbour lists: one warp per query ----------------------------------
//
// The warp scans the preorder cells 32 at a time. Lane k tests cell cur+k
// against the query sphere (the reference's box test, src/octree.c:250-256).
// A cell is reached only if no ancestor failed; inside the window an
// ancestor u of v satisfies u < v < next(u), so "v lies under a failed cell"
// is an exclusive prefix-max over lanes of next(u) of failed cells, compared
// with v. Reached leaves whose body lies within the radius are neighbours,
// taken in lane (= depth-first) order up to the cap. The cursor then moves
// past the window and past every failed cell's subtree.
//
// Tests run in FP32 with a bound on their rounding: a decision is taken in
// FP32 only when the FP32 value clears the threshold by more than that bound
// (position errors <= 8 ulp of the largest magnitude involved per axis, plus
// 2^-18 relative on the squared sums); otherwise the reference's own FP64
// expression decides. So every decision equals the reference's.

constexpr float FP32_EPS_POS = 0x1p-21f; // 8 x 2^-24 per axis
constexpr float FP32_EPS_SUM = 0x1p-18f;

// Box test of src/octree.c:250-256: true when the cell may hold neighbours.
__device__ __forceinline__ bool box_reaches(const NodeS32 &c, float qx, float qy, float qz,
                                            float mq, float r2f, const SphArgs &a, int cell,
                                            double px, double py, double pz, double r2)
{
    const float e = (mq + c.cmax) * FP32_EPS_POS;
    const float dx = fmaxf(0.0f, fabsf(qx - c.cx) - c.hs);
    const float dy = fmaxf(0.0f, fabsf(qy - c.cy) - c.hs);
    const float dz = fmaxf(0.0f, fabsf(qz - c.cz) - c.hs);
    const float lx = fmaxf(0.0f, dx - e), ly = fmaxf(0.0f, dy - e), lz = fmaxf(0.0f, dz - e);
    const float lo = lx * lx + ly * ly + lz * lz;
    if (lo > r2f * (1.0f + FP32_EPS_SUM))
        return false;
    const float hx = dx + e, hy = dy + e, hz = dz + e;
    const float hi = hx * hx + hy * hy + hz * hz;
    if (hi < r2f * (1.0f - FP32_EPS_SUM))
        return true;
    const double4_32a g = a.geo[cell]; // too close to call in FP32
    double gx = fmax(0.0, fabs(px - g.x) - g.w);
    double gy = fmax(0.0, fabs(py - g.y) - g.w);
    double gz = fmax(0.0, fabs(pz - g.z) - g.w);
    return !(gx * gx + gy * gy + gz * gz > r2);
}

// Leaf test of src/octree.c:262-272: body within the radius.
__device__ __forceinline__ bool leaf_within(const NodeS32 &c, float qx, float qy, float qz,
                                            float mq, float r2f, const SphArgs &a, double px,
                                            double py, double pz, double r2)
{
    const float mb = fmaxf(fabsf(c.bx), fmaxf(fabsf(c.by), fabsf(c.bz)));
    const float e = (mq + mb) * FP32_EPS_POS;
    const float dx = fabsf(c.bx - qx), dy = fabsf(c.by - qy), dz = fabsf(c.bz - qz);
    const float hx = dx + e, hy = dy + e, hz = dz + e;
    const float hi = hx * hx + hy * hy + hz * hz;
    if (hi < r2f * (1.0f - FP32_EPS_SUM))
        return true;
    const float lx = fmaxf(0.0f, dx - e), ly = fmaxf(0.0f, dy - e), lz = fmaxf(0.0f, dz - e);
    const float lo = lx * lx + ly * ly + lz * lz;
    if (lo > r2f * (1.0f + FP32_EPS_SUM))
        return false;
    const int j = c.body;
    double bx = a.x[j] - px;
    double by = a.y[j] - py;
    double bz = a.z[j] - pz;
    return bx * bx + by * by + bz * bz <= r2;
}

__device__ __forceinline__ int warp_excl_max(int v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o)
            v = max(v, t);
    }
    int ex = __shfl_up_sync(0xffffffffu, v, 1);
    return lane == 0 ? INT_MIN : ex;
}

// Lists: gas body gas[k] gets its first CSG_SPH_MAX_NEIGHBORS neighbours within
// its current smoothing length, in depth-first order, slot-major
// (nb[slot * stride + k]) for coalesced reads in the pair kernels. The density
// pass uses h before its update (src/sph.c:53-63), the force pass after it
// (src/sph.c:112-126): each pass builds its list from the h it sees.
__device__ __forceinline__ void list_one(const SphArgs &a, int k, int lane)
{
    const int nnodes = (a.sc->n_nodes > a.node_cap) ? 0 : a.sc->n_nodes;
    const int i = a.gas[k];
    const double px = a.x[i], py = a.y[i], pz = a.z[i];
    const double h = a.h[i];
    const double r2 = h * h;
    const float qx = (float)px, qy = (float)py, qz = (float)pz;
    const float mq = fmaxf(fabsf(qx), fmaxf(fabsf(qy), fabsf(qz)));
    const float r2f = (float)r2;
    const unsigned lt = (1u << lane) - 1u;
    const size_t stride = (size_t)a.stride;
    int found = 0;
    int cur = 0;
    while (cur < nnodes && found < CSG_SPH_MAX_NEIGHBORS) {
        const int v = cur + lane;
        const bool valid = v < nnodes;
        NodeS32 c;
        bool reach = false;
        int fail_next = 0;
        if (valid) {
            c = a.s32[v];
            reach = box_reaches(c, qx, qy, qz, mq, r2f, a, v, px, py, pz, r2);
            if (!reach)
                fail_next = c.next;
            if (c.next <= v)
                dev_fail(a.sc, CSG_ERR_WALK_LIMIT);
        }
        const int above = warp_excl_max(fail_next);
        bool cand = false;
        if (valid && reach && above <= v && c.body != -1) {
            if (c.body == -3)
                dev_fail(a.sc, CSG_ERR_BAD_POOL);
            else if (c.body >= 0)
                cand = leaf_within(c, qx, qy, qz, mq, r2f, a, px, py, pz, r2);
        }
        const unsigned m = __ballot_sync(0xffffffffu, cand);
        if (cand) {
            const int slot = found + __popc(m & lt);
            if (slot < CSG_SPH_MAX_NEIGHBORS)
                a.nb[stride * slot + k] = c.body;
        }
        found = min(CSG_SPH_MAX_NEIGHBORS, found + __popc(m));
        // skip past the window and past every failed subtree
        const int jump = __reduce_max_sync(0xffffffffu, (unsigned)max(fail_next, 0));
        cur = max(cur + CSG_WARP, jump); // strictly increases: the loop ends
    }
    if (lane == 0) {
        a.nb_count[k] = found;
        if (a.density) // its pairs need 8/(pi h^3) of this body
            a.pr2[i] = h < 1e-10 ? 0.0 : kernel_norm(h);
    }
}

__global__ void __launch_bounds__(SPH_THREADS) k_sph_lists(SphArgs a)
{
    const int lane = threadIdx.x & 31;
    const int n_gas = a.sc->n_gas;
    const int nwarps = (int)((gridDim.x * (long long)SPH_THREADS) >> 5);
    for (int k = (int)(((long long)blockIdx.x * SPH_THREADS + threadIdx.x) >> 5); k < n_gas;
         k += nwarps) // warp-uniform
        if (!a.reuse || a.relist[k])
            list_one(a, k, lane);
}

// Pair kernels. Each pass runs in two kernels so that the FP64 pair
// arithmetic (sqrt, divisions) keeps every SM busy even when gas bodies are
// few: one thread per (list slot, gas body) writes the pair's term, then one
// thread per gas body adds its terms in list order — the reference's order,
// with the same operations, so the sums are the reference's bit for bit
// (a skipped pair stores 0, and x - 0 == x for every x).
__device__ __forceinline__ bool pair_slot(const SphArgs &a, long long t, int n_gas, int &s,
                                          int &k)
{
    s = (int)(t / n_gas);
    k = (int)(t - (long long)s * n_gas);
    return s < a.nb_count[k];
}

// Density terms m_j W(r, h_i), src/sph.c:53-63.
__global__ void __launch_bounds__(SPH_THREADS) k_sph_density_terms(SphArgs a)
{
    const int n_gas = a.sc->n_gas;
    const long long total = (long long)CSG_SPH_MAX_NEIGHBORS * n_gas;
    const size_t stride = (size_t)a.stride;
    for (long long t = (long long)blockIdx.x * SPH_THREADS + threadIdx.x; t < total;
         t += (long long)gridDim.x * SPH_THREADS) {
        int s, k;
        if (!pair_slot(a, t, n_gas, s, k))
            continue;
        const int i = a.gas[k];
        const int j = a.nb[stride * s + k];
        double dx = a.x[i] - a.x[j];
        double dy = a.y[i] - a.y[j];
        double dz = a.z[i] - a.z[j];
        double r = sqrt_rn(dx * dx + dy * dy + dz * dz);
        a.term[stride * s + k] = a.m[j] * kernel_W_norm(r, a.h[i], a.pr2[i]);
    }
}

// The per-body sums run one thread per gas body in small blocks (the gas
// bodies are ~10% of all: 64-thread blocks spread them over every SM) and
// load SUM_BATCH slots ahead of the additions, which stay in list order.
constexpr int SUM_THREADS = 64;
constexpr int SUM_BATCH = 8;

// Density, adaptive h and pressure, src/sph.c:45-97.
__global__ void __launch_bounds__(SUM_THREADS) k_sph_density_sums(SphArgs a)
{
    const int k = blockIdx.x * SUM_THREADS + threadIdx.x;
    if (k >= a.sc->n_gas)
        return;
    const int i = a.gas[k];
    const double h = a.h[i];
    const int nn = a.nb_count[k];
    const size_t stride = (size_t)a.stride;
    const double *__restrict__ term = a.term;
    double rho = 0.0;
    int s = 0;
    for (; s + SUM_BATCH <= nn; s += SUM_BATCH) {
        double t[SUM_BATCH];
#pragma unroll
        for (int u = 0; u < SUM_BATCH; u++)
            t[u] = __ldg(&term[stride * (s + u) + k]);
#pragma unroll
        for (int u = 0; u < SUM_BATCH; u++)
            rho += t[u];
    }
    for (; s < nn; s++)
        rho += __ldg(&term[stride * s + k]);
    int relist = 1;
    if (nn < 20 && h < 50.0)
        a.h[i] = h * 1.2;
    else if (nn > 48 && h > 0.1)
        a.h[i] = h * 0.8;
    else
        relist = 0;
    a.relist[k] = relist;
    if (rho < 1e-15 || isnan(rho))
        rho = 1e-15;
    a.rho[i] = rho;
    double u = a.u[i];
    if (u < 1e-15)
        u = 1e-15;
    a.P[i] = (GAMMA - 1.0) * rho * u;
}

// Per-body terms of the force pass: P/(rho^2 + 1e-15) and the sound speed
// sqrt(gamma P/(rho + 1e-15)) (src/sph.c:112, :153-154, :170-171). The pair
// terms need them for both bodies of every pair; computing them once per body
// gives the same values as the reference's per-pair evaluation.
__global__ void __launch_bounds__(SUM_THREADS) k_sph_body_terms(SphArgs a)
{
    const int k = blockIdx.x * SUM_THREADS + threadIdx.x;
    if (k >= a.sc->n_gas)
        return;
    const int j = a.gas[k];
    const double rho = a.rho[j], P = a.P[j];
    a.pr2[j] = div_rn(P, rho * rho + 1e-15);
    a.cs[j] = sqrt_rn(div_rn(GAMMA * P, rho + 1e-15));
}

// Pressure gradient + Monaghan viscosity terms, src/sph.c:126-186.
__global__ void __launch_bounds__(SPH_THREADS) k_sph_force_terms(SphArgs a)
{
    const int n_gas = a.sc->n_gas;
    const long long total = (long long)CSG_SPH_MAX_NEIGHBORS * n_gas;
    const size_t stride = (size_t)a.stride;
    const size_t plane = stride * CSG_SPH_MAX_NEIGHBORS;
    for (long long t = (long long)blockIdx.x * SPH_THREADS + threadIdx.x; t < total;
         t += (long long)gridDim.x * SPH_THREADS) {
        int s, k;
        if (!pair_slot(a, t, n_gas, s, k))
            continue;
        const size_t o = stride * s + k;
        const int i = a.gas[k];
        const int j = a.nb[o];
        double tx = 0.0, ty = 0.0, tz = 0.0;
        if (j != i && a.type[j] == BODY_GAS) {
            double dx = a.x[i] - a.x[j];
            double dy = a.y[i] - a.y[j];
            double dz = a.z[i] - a.z[j];
            double r = sqrt_rn(dx * dx + dy * dy + dz * dz);
            if (!(r < 1e-15)) {
                const double h_i = a.h[i], rho_i = a.rho[i];
                double h_avg = 0.5 * (h_i + a.h[j]);
                double rho_j = a.rho[j];
                double dvx = a.vx[i] - a.vx[j];
                double dvy = a.vy[i] - a.vy[j];
                double dvz = a.vz[i] - a.vz[j];
                double vr = dvx * dx + dvy * dy + dvz * dz;
                double visc = 0.0;
                if (vr < 0.0) {
                    double mu = div_rn(h_avg * vr, r * r + 0.01 * h_avg * h_avg);
                    double c_avg = 0.5 * (a.cs[i] + a.cs[j]);
                    double rho_avg = 0.5 * (rho_i + rho_j);
                    visc = div_rn(-1.0 * c_avg * mu + 2.0 * mu * mu, rho_avg + 1e-15);
                }
                double g = kernel_dWdr(r, h_avg);
                double gx = div_rn(g * dx, r);
                double gy = div_rn(g * dy, r);
                double gz = div_rn(g * dz, r);
                double f = a.m[j] * (a.pr2[i] + a.pr2[j] + visc);
                tx = f * gx;
                ty = f * gy;
                tz = f * gz;
            }
        }
        a.term[o] = tx;
        a.term[plane + o] = ty;
        a.term[2 * plane + o] = tz;
    }
}

// Sums of the force terms in list order, src/sph.c:187-196.
__global__ void __launch_bounds__(SUM_THREADS) k_sph_force_sums(SphArgs a)
{
    const int k = blockIdx.x * SUM_THREADS + threadIdx.x;
    if (k >= a.sc->n_gas)
        return;
    const int i = a.gas[k];
    const int nn = a.nb_count[k];
    const size_t stride = (size_t)a.stride;
    const size_t plane = stride * CSG_SPH_MAX_NEIGHBORS;
    const double *__restrict__ term = a.term;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    int s = 0;
    for (; s + SUM_BATCH <= nn; s += SUM_BATCH) {
        double tx[SUM_BATCH], ty[SUM_BATCH], tz[SUM_BATCH];
#pragma unroll
        for (int u = 0; u < SUM_BATCH; u++) {
            const size_t o = stride * (s + u) + k;
            tx[u] = __ldg(&term[o]);
            ty[u] = __ldg(&term[plane + o]);
            tz[u] = __ldg(&term[2 * plane + o]);
        }
#pragma unroll
        for (int u = 0; u < SUM_BATCH; u++) {
            sx -= tx[u];
            sy -= ty[u];
            sz -= tz[u];
        }
    }
    for (; s < nn; s++) {
        const size_t o = stride * s + k;
        sx -= __ldg(&term[o]);
        sy -= __ldg(&term[plane + o]);
        sz -= __ldg(&term[2 * plane + o]);
    }
    if (isnan(sx))
        sx = 0.0;
    if (isnan(sy))
        sy = 0.0;
    if (isnan(sz))
        sz = 0.0;
    a.ax[i] += sx * 0.1;
    a.ay[i] += sy * 0.1;
    a.az[i] += sz * 0.1;
}

__global__ void k_gas_flags(DevScalars *sc, const int *__restrict__ perm,
                            const int *__restrict__ type, int *__restrict__ flag)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= sc->n_alive)
        return;
    flag[p] = (type[perm[p]] == BODY_GAS) ? 1 : 0;
}

__global__ void k_gas_scatter(DevScalars *sc, const int *__restrict__ perm,
                              const int *__restrict__ flag, const int *__restrict__ base,
                              int *__restrict__ gas)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int na = sc->n_alive;
    if (p == 0)
        sc->n_gas = base[na];
    if (p >= na)
        return;
    if (flag[p])
        gas[base[p]] = perm[p];
}

// One query, one thread: src/octree.c:293-318.
__global__ void k_find_one(SphArgs a, double cx, double cy, double cz, double radius, int cap,
                           int *__restrict__ buf, int *__restrict__ count)
{
    const int nn = (a.sc->n_nodes > a.node_cap) ? 0 : a.sc->n_nodes;
    const double r2 = radius * radius;
    int c = 0, cur = 0;
    while (cur < nn && c < cap) {
        const double4_32a g = a.geo[cur];
        const int next = a.w64[cur].next, body = a.w64[cur].body;
        if (next <= cur) {
            dev_fail(a.sc, CSG_ERR_WALK_LIMIT);
            break;
        }
        double gx = fmax(0.0, fabs(cx - g.x) - g.w);
        double gy = fmax(0.0, fabs(cy - g.y) - g.w);
        double gz = fmax(0.0, fabs(cz - g.z) - g.w);
        if (gx * gx + gy * gy + gz * gz > r2) {
            cur = next;
            continue;
        }
        if (body >= 0) {
            if (body >= a.n) {
                dev_fail(a.sc, CSG_ERR_BAD_POOL);
            } else if (!(a.m[body] <= 0.0)) {
                double bx = a.x[body] - cx;
                double by = a.y[body] - cy;
                double bz = a.z[body] - cz;
                if (bx * bx + by * by + bz * bz <= r2)
                    buf[c++] = body;
            }
        }
        cur = cur + 1;
    }
    *count = c;
}

SphArgs make_args(csgd_t *d)
{
    SphArgs a;
    a.gas = d->gas;
    a.x = d->x;
    a.y = d->y;
    a.z = d->z;
    a.vx = d->vx;
    a.vy = d->vy;
    a.vz = d->vz;
    a.m = d->m;
    a.type = d->type;
    a.h = d->h;
    a.rho = d->rho;
    a.P = d->P;
    a.u = d->u;
    a.ax = d->ax;
    a.ay = d->ay;
    a.az = d->az;
    a.geo = d->geo;
    a.s32 = d->s32;
    a.w64 = d->w64;
    a.sc = d->sc;
    a.nb = d->nb;
    a.nb_count = d->nb_count;
    a.relist = d->sph_relist;
    a.reuse = 0;
    a.density = 0;
    a.pr2 = d->pr2;
    a.cs = d->cs;
    a.term = d->sph_term;
    a.n = d->n;
    a.node_cap = d->node_cap;
    a.stride = d->cap;
    return a;
}

// Caller-index order, for trees imported from a caller pool (no key order).
__global__ void k_gas_flags_idx(int n, const double *__restrict__ m, const int *__restrict__ type,
                                int *__restrict__ flag)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    flag[i] = (type[i] == BODY_GAS && !(m[i] <= 0.0)) ? 1 : 0;
}

__global__ void k_gas_scatter_idx(DevScalars *sc, int n, const int *__restrict__ flag,
                                  const int *__restrict__ base, int *__restrict__ gas)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0)
        sc->n_gas = base[n];
    if (i < n && flag[i])
        gas[base[i]] = i;
}

int gas_list(csgd_t *d)
{
    if (d->gas_valid)
        return CSG_OK;
    const int n = d->n;
    const int g = csgd_grid(n, 256);
    if (!d->imported) {
        { k_gas_flags<<<g, 256, 0, d->stream>>>(d->sc, d->perm, d->type, d->cnt); d->launches++; }
        int rc = csg_scan_exclusive(d, d->cnt, d->base, n, &d->sc->n_alive);
        if (rc)
            return rc;
        { k_gas_scatter<<<g, 256, 0, d->stream>>>(d->sc, d->perm, d->cnt, d->base, d->gas); d->launches++; }
    } else {
        { k_gas_flags_idx<<<g, 256, 0, d->stream>>>(n, d->m, d->type, d->cnt); d->launches++; }
        int rc = csg_scan_exclusive(d, d->cnt, d->base, n, nullptr);
        if (rc)
            return rc;
        { k_gas_scatter_idx<<<g, 256, 0, d->stream>>>(d->sc, n, d->cnt, d->base, d->gas); d->launches++; }
    }
    d->gas_valid = 1;
    return csgd_check(d, cudaGetLastError());
}

} // namespace

// Lists live in device memory sized for every body being gas (128 ints each),
// allocated on first SPH use.
static int ensure_lists(csgd_t *d)
{
    int rc = csgd_ensure_tree_extras(d, 1, 0); // SPH walks the cell geometry
    if (rc)
        return rc;
    if (d->nb && d->nb_cap >= d->cap)
        return CSG_OK;
    if (d->nb)
        cudaFree(d->nb);
    if (d->nb_count)
        cudaFree(d->nb_count);
    if (d->pr2)
        cudaFree(d->pr2);
    if (d->cs)
        cudaFree(d->cs);
    if (d->sph_term)
        cudaFree(d->sph_term);
    if (d->sph_relist)
        cudaFree(d->sph_relist);
    d->nb = nullptr;
    d->nb_count = d->sph_relist = nullptr;
    d->pr2 = d->cs = d->sph_term = nullptr;
    size_t c = (size_t)(d->cap > 0 ? d->cap : 1);
    if (csgd_malloc((void **)&d->nb, sizeof(int) * CSG_SPH_MAX_NEIGHBORS * c) != cudaSuccess ||
        csgd_malloc((void **)&d->nb_count, sizeof(int) * c) != cudaSuccess ||
        csgd_malloc((void **)&d->sph_relist, sizeof(int) * c) != cudaSuccess ||
        csgd_malloc((void **)&d->pr2, sizeof(double) * c) != cudaSuccess ||
        csgd_malloc((void **)&d->cs, sizeof(double) * c) != cudaSuccess ||
        csgd_malloc((void **)&d->sph_term, sizeof(double) * 3 * CSG_SPH_MAX_NEIGHBORS * c) !=
            cudaSuccess) {
        cudaGetLastError();
        csgd_set_err(d, CSG_ERR_NOMEM);
        return CSG_ERR_NOMEM;
    }
    d->nb_cap = d->cap;
    return CSG_OK;
}

static int sph_pass(csgd_t *d, int forces, bool sums = true, bool reuse = false)
{
    if (d->n_gal > 1) { // one system only (see csgd_set_systems)
        return CSG_ERR_UNSUPPORTED;
    }
    if (d->n <= 0)
        return CSG_OK;
    if (!d->geometry_valid) {
        return CSG_ERR_BAD_ARG;
    }
    int rc = ensure_lists(d);
    if (!rc)
        rc = gas_list(d);
    if (rc)
        return rc;
    SphArgs a = make_args(d);
    a.reuse = (forces && reuse) ? 1 : 0;
    a.density = forces ? 0 : 1;
    const int g = csgd_grid(d->n, SUM_THREADS);
    // one warp per gas body for the lists, warps striding over the gas bodies
    int gl = csgd_grid((long long)d->n * CSG_WARP, SPH_THREADS);
    if (gl > d->num_sms * 16)
        gl = d->num_sms * 16;
    { k_sph_lists<<<gl, SPH_THREADS, 0, d->stream>>>(a); d->launches++; }
    // pair terms: a grid-stride pass over (slot, gas body), sized for 32 warps
    // per SM (the gas count is known on the device only)
    const int gp = d->num_sms * (2048 / SPH_THREADS);
    if (forces) {
        { k_sph_body_terms<<<g, SUM_THREADS, 0, d->stream>>>(a); d->launches++; }
        { k_sph_force_terms<<<gp, SPH_THREADS, 0, d->stream>>>(a); d->launches++; }
        if (sums)
            { k_sph_force_sums<<<g, SUM_THREADS, 0, d->stream>>>(a); d->launches++; }
    } else {
        { k_sph_density_terms<<<gp, SPH_THREADS, 0, d->stream>>>(a); d->launches++; }
        { k_sph_density_sums<<<g, SUM_THREADS, 0, d->stream>>>(a); d->launches++; }
    }
    return csgd_check(d, cudaGetLastError());
}

extern "C" int csgd_sph_density(csgd_t *d) { return sph_pass(d, 0); }

extern "C" int csgd_prepare_sph(csgd_t *d) { return ensure_lists(d); }

extern "C" int csgd_sph_forces(csgd_t *d, int reuse_lists)
{
    return sph_pass(d, 1, true, reuse_lists != 0);
}

extern "C" int csgd_sph_force_terms(csgd_t *d, int reuse_lists)
{
    return sph_pass(d, 1, false, reuse_lists != 0);
}

extern "C" int csgd_sph_force_sums(csgd_t *d)
{
    if (d->n <= 0)
        return CSG_OK;
    SphArgs a = make_args(d);
    { k_sph_force_sums<<<csgd_grid(d->n, SUM_THREADS), SUM_THREADS, 0, d->stream>>>(a); d->launches++; }
    return csgd_check(d, cudaGetLastError());
}

extern "C" int csgd_find_neighbors(csgd_t *d, double cx, double cy, double cz, double radius,
                                   int *buf, int cap, int *count_out)
{
    if (d->n_gal > 1) { // one system only (see csgd_set_systems)
        return CSG_ERR_UNSUPPORTED;
    }
    *count_out = 0;
    if (cap <= 0)
        return CSG_OK;
    if (!d->geometry_valid) {
        return CSG_ERR_BAD_ARG;
    }
    // scratch: the export rank buffer holds the result (node_cap >= cap is not
    // guaranteed, so cap is clamped to the buffer)
    if (cap > d->node_cap)
        cap = d->node_cap;
    int *dbuf = d->rank;
    int *dcount = d->ord_id;
    SphArgs a = make_args(d);
    { k_find_one<<<1, 1, 0, d->stream>>>(a, cx, cy, cz, radius, cap, dbuf, dcount); d->launches++; }
    int c = 0;
    cudaMemcpyAsync(&c, dcount, sizeof(int), cudaMemcpyDeviceToHost, d->stream);
    int rc = csgd_sync(d);
    if (rc)
        return rc;
    if (c > 0) {
        cudaMemcpyAsync(buf, dbuf, sizeof(int) * (size_t)c, cudaMemcpyDeviceToHost, d->stream);
        rc = csgd_sync(d);
    }
    *count_out = c;
    return rc;
}
