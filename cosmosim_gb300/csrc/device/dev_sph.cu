// dev_sph.cu — SPH density/pressure and forces on the shared octree
// (reference src/sph.c:45-196) and the neighbour query of
// src/octree.c:236-318.
//
// Neighbour order matters: the reference keeps the first 128 bodies within
// the radius in depth-first octant order (src/octree.c:260-277, sph.h:9), and
// the cap binds often. Walking the preorder tree with per-lane subtree skips
// (as in dev_walk.cu) meets the leaves in exactly that order, so each lane can
// sum its density/force terms on the fly, in the reference's order, without a
// neighbour list. Lanes are the gas bodies in key order.
//
// Compiled with -fmad=false, with the reference's operation order, so for the
// same inputs every sum rounds as the reference's does.
#include "dev_internal.cuh"

namespace {

constexpr int SPH_THREADS = 128;
constexpr int SPH_WARPS = SPH_THREADS / CSG_WARP;
constexpr double GAMMA = 5.0 / 3.0;
constexpr double PI_D = 3.14159265358979323846;

// M4 cubic spline, src/sph.c:11-25
__device__ __forceinline__ double kernel_W(double r, double h)
{
    if (h < 1e-10)
        return 0.0;
    double q = r / h;
    if (q > 1.0)
        return 0.0;
    double norm = 8.0 / (PI_D * h * h * h);
    if (q <= 0.5)
        return norm * (1.0 - 6.0 * q * q + 6.0 * q * q * q);
    double t = 1.0 - q;
    return norm * 2.0 * t * t * t;
}

// its radial derivative, src/sph.c:27-41
__device__ __forceinline__ double kernel_dWdr(double r, double h)
{
    if (h < 1e-10)
        return 0.0;
    double q = r / h;
    if (q > 1.0 || r < 1e-15)
        return 0.0;
    double norm = 8.0 / (PI_D * h * h * h);
    if (q <= 0.5)
        return norm * (-12.0 * q + 18.0 * q * q) / h;
    double t = 1.0 - q;
    return norm * (-6.0 * t * t) / h;
}

struct SphArgs {
    const int *gas;
    const double *x, *y, *z, *vx, *vy, *vz, *m;
    const int *type;
    double *h, *rho, *P, *u;
    double *ax, *ay, *az;
    const double4 *geo;
    const NodeW64 *w64;
    DevScalars *sc;
    int n, node_cap;
};

struct NbStep {
    int next, body;
};

// Shared traversal: calls visit(j) for each neighbour j of the lane in
// depth-first order until the lane has `cap` neighbours.
template <typename Visit>
__device__ __forceinline__ void neighbour_walk(const SphArgs &a, bool valid, double qx, double qy,
                                               double qz, double r2, double4 *wgeo, NbStep *wnb,
                                               Visit visit)
{
    const int lane = threadIdx.x & 31;
    const int nn = (a.sc->n_nodes > a.node_cap) ? 0 : a.sc->n_nodes;
    int skip = valid ? 0 : INT_MAX;
    int found = 0;
    int cur = 0, wbase = INT_MIN / 2;
    while (cur < nn) {
        if (__all_sync(0xffffffffu, skip == INT_MAX))
            break;
        if (cur - wbase >= CSG_WARP) {
            wbase = cur;
            __syncwarp();
            if (wbase + lane < nn) {
                wgeo[lane] = a.geo[wbase + lane];
                wnb[lane] = NbStep{a.w64[wbase + lane].next, a.w64[wbase + lane].body};
            }
            __syncwarp();
        }
        const double4 g = wgeo[cur - wbase];
        const NbStep s = wnb[cur - wbase];
        bool descend = false;
        if (cur >= skip) {
            double gx = fmax(0.0, fabs(qx - g.x) - g.w);
            double gy = fmax(0.0, fabs(qy - g.y) - g.w);
            double gz = fmax(0.0, fabs(qz - g.z) - g.w);
            if (gx * gx + gy * gy + gz * gz > r2) {
                skip = s.next;
            } else if (s.body >= 0) {
                const int j = s.body;
                if (j >= a.n) {
                    dev_fail(a.sc, CSG_ERR_BAD_POOL);
                } else if (!(a.m[j] <= 0.0)) {
                    double bx = a.x[j] - qx;
                    double by = a.y[j] - qy;
                    double bz = a.z[j] - qz;
                    if (bx * bx + by * by + bz * bz <= r2) {
                        visit(j);
                        if (++found >= CSG_SPH_MAX_NEIGHBORS)
                            skip = INT_MAX;
                    }
                }
            } else {
                descend = true;
            }
        }
        const int nxt = __any_sync(0xffffffffu, descend) ? cur + 1 : s.next;
        if (nxt <= cur) {
            dev_fail(a.sc, CSG_ERR_WALK_LIMIT);
            break;
        }
        cur = nxt;
    }
    // the count is returned through visit's captured state
    (void)found;
}

// src/sph.c:45-97
__global__ void __launch_bounds__(SPH_THREADS) k_sph_density(SphArgs a)
{
    __shared__ double4 wgeo_all[SPH_WARPS][CSG_WARP];
    __shared__ NbStep wnb_all[SPH_WARPS][CSG_WARP];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n_gas = a.sc->n_gas;
    const long long k = (long long)blockIdx.x * SPH_THREADS + threadIdx.x;
    if (k - lane >= n_gas)
        return;
    const bool valid = k < n_gas;
    const int i = valid ? a.gas[k] : 0;
    const double qx = a.x[i], qy = a.y[i], qz = a.z[i];
    const double h = a.h[i];
    double rho = 0.0;
    int nn = 0;
    neighbour_walk(a, valid, qx, qy, qz, h * h, wgeo_all[warp], wnb_all[warp], [&](int j) {
        nn++;
        double dx = qx - a.x[j];
        double dy = qy - a.y[j];
        double dz = qz - a.z[j];
        double r = sqrt(dx * dx + dy * dy + dz * dz);
        rho += a.m[j] * kernel_W(r, h);
    });
    if (!valid)
        return;
    if (nn < 20 && h < 50.0)
        a.h[i] = h * 1.2;
    else if (nn > 48 && h > 0.1)
        a.h[i] = h * 0.8;
    if (rho < 1e-15 || isnan(rho))
        rho = 1e-15;
    a.rho[i] = rho;
    double u = a.u[i];
    if (u < 1e-15)
        u = 1e-15;
    a.P[i] = (GAMMA - 1.0) * rho * u;
}

// src/sph.c:101-196
__global__ void __launch_bounds__(SPH_THREADS) k_sph_forces(SphArgs a)
{
    __shared__ double4 wgeo_all[SPH_WARPS][CSG_WARP];
    __shared__ NbStep wnb_all[SPH_WARPS][CSG_WARP];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n_gas = a.sc->n_gas;
    const long long k = (long long)blockIdx.x * SPH_THREADS + threadIdx.x;
    if (k - lane >= n_gas)
        return;
    const bool valid = k < n_gas;
    const int i = valid ? a.gas[k] : 0;
    const double qx = a.x[i], qy = a.y[i], qz = a.z[i];
    const double h_i = a.h[i];
    const double rho_i = a.rho[i];
    const double P_i = a.P[i];
    const double c_i = sqrt(GAMMA * P_i / (rho_i + 1e-15));
    const double vxi = a.vx[i], vyi = a.vy[i], vzi = a.vz[i];
    double sx = 0.0, sy = 0.0, sz = 0.0;
    neighbour_walk(a, valid, qx, qy, qz, h_i * h_i, wgeo_all[warp], wnb_all[warp], [&](int j) {
        if (j == i || a.type[j] != BODY_GAS)
            return;
        double dx = qx - a.x[j];
        double dy = qy - a.y[j];
        double dz = qz - a.z[j];
        double r = sqrt(dx * dx + dy * dy + dz * dz);
        if (r < 1e-15)
            return;
        double h_avg = 0.5 * (h_i + a.h[j]);
        double rho_j = a.rho[j];
        double P_j = a.P[j];
        double dvx = vxi - a.vx[j];
        double dvy = vyi - a.vy[j];
        double dvz = vzi - a.vz[j];
        double vr = dvx * dx + dvy * dy + dvz * dz;
        double visc = 0.0;
        if (vr < 0.0) {
            double mu = h_avg * vr / (r * r + 0.01 * h_avg * h_avg);
            double c_j = sqrt(GAMMA * P_j / (rho_j + 1e-15));
            double c_avg = 0.5 * (c_i + c_j);
            double rho_avg = 0.5 * (rho_i + rho_j);
            visc = (-1.0 * c_avg * mu + 2.0 * mu * mu) / (rho_avg + 1e-15);
        }
        double g = kernel_dWdr(r, h_avg);
        double gx = g * dx / r;
        double gy = g * dy / r;
        double gz = g * dz / r;
        double f = a.m[j] * (P_i / (rho_i * rho_i + 1e-15) + P_j / (rho_j * rho_j + 1e-15) + visc);
        sx -= f * gx;
        sy -= f * gy;
        sz -= f * gz;
    });
    if (!valid)
        return;
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
        const double4 g = a.geo[cur];
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
    a.w64 = d->w64;
    a.sc = d->sc;
    a.n = d->n;
    a.node_cap = d->node_cap;
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

extern "C" int csgd_sph_density(csgd_t *d)
{
    if (d->n <= 0)
        return CSG_OK;
    if (!d->geometry_valid) {
        csgd_set_err(d, CSG_ERR_BAD_ARG);
        return CSG_ERR_BAD_ARG;
    }
    int rc = gas_list(d);
    if (rc)
        return rc;
    SphArgs a = make_args(d);
    { k_sph_density<<<csgd_grid(d->n, SPH_THREADS), SPH_THREADS, 0, d->stream>>>(a); d->launches++; }
    return csgd_check(d, cudaGetLastError());
}

extern "C" int csgd_sph_forces(csgd_t *d)
{
    if (d->n <= 0)
        return CSG_OK;
    if (!d->geometry_valid) {
        csgd_set_err(d, CSG_ERR_BAD_ARG);
        return CSG_ERR_BAD_ARG;
    }
    int rc = gas_list(d);
    if (rc)
        return rc;
    SphArgs a = make_args(d);
    { k_sph_forces<<<csgd_grid(d->n, SPH_THREADS), SPH_THREADS, 0, d->stream>>>(a); d->launches++; }
    return csgd_check(d, cudaGetLastError());
}

extern "C" int csgd_find_neighbors(csgd_t *d, double cx, double cy, double cz, double radius,
                                   int *buf, int cap, int *count_out)
{
    *count_out = 0;
    if (cap <= 0)
        return CSG_OK;
    if (!d->geometry_valid) {
        csgd_set_err(d, CSG_ERR_BAD_ARG);
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
