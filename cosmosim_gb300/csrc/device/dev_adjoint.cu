// dev_adjoint.cu — adjoint of the kick-drift-kick leapfrog
// (reference src/integrator.c:4-57) over Barnes-Hut gravity with frozen
// interaction lists, or over FP64 direct-sum gravity.
//
// Forward model (FP64). a(x)_i = sum over the cells c in body i's list L_i
// of G M_c (X_c - x_i) / (|X_c - x_i|^2 + eps^2)^(3/2), where L_i is the
// reference walk's interaction set on the tree of x (the same cells, in the
// same depth-first order) and X_c, M_c the centre of mass and mass of the
// bodies in c. The lists change only where an opening decision flips; the
// adjoint differentiates with them frozen, as is usual for tree codes, and
// forward_frozen replays a recorded run's lists so that finite differences
// see the same map.
//
// Jacobian-transpose product (J^T mu)_j of a = a(x), with the softened tidal
// tensor T(d) = G M (I/r^3 - 3 d d^T / r^5), r^2 = |d|^2 + eps^2:
//   self term      -sum_{c in L_j} T(X_c - x_j) mu_j
//   through X_c    m_j sum_{c containing j} g_c / M_c,
//                  g_c = sum_{i : c in L_i} T(X_c - x_i) mu_i
// (dX_c/dx_j = m_j/M_c for j in c). k_adj_jt forms the self term and scatters
// g_c per interaction; k_adj_push walks each body's ancestors.
// Direct sum: (J^T mu)_j = G sum_{i != j} T1(x_i - x_j) (m_j mu_i - m_i mu_j),
// T1 the tensor with unit mass.
//
// Reverse sweep (lambda_x, lambda_v: adjoints of x_n, v_n; start at n = T
// with lambda_x = dLoss/dx_T, lambda_v = 0):
//   for n = T-1 .. 0:  lambda_v += dt lambda_x              (drift)
//                      lambda_x += J(x_n)^T (c_n dt lambda_v) (both half kicks
//                      that use a(x_n): c_n = 1, or 1/2 at n = 0)
// Memory: positions and velocities are kept every K substeps; a segment's
// trees and lists are rebuilt from its checkpoint (bit-identical: every
// forward kernel is deterministic) before it is reversed.
#include "dev_internal.cuh"

#include <stdlib.h>
#include <string.h>

#include <vector>

extern "C" void csg_thread_set_error(int code); // capi_context.c

namespace {

constexpr int AT = 256;

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sorted position -> the leaf cell holding it.
__global__ void k_adj_leaf_of(const NodeLink *__restrict__ link, const NodeW64 *__restrict__ w64,
                              int nn, int *__restrict__ leaf_of)
{
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nn || w64[id].body < 0)
        return;
    const NodeLink l = link[id];
    for (int q = 0; q < l.count; q++)
        leaf_of[l.first + q] = id;
}

// Position and mass of every sorted position (the member ranges of the cells
// then read contiguous memory).
__global__ void k_adj_gather(const int *__restrict__ perm, int n, const double *__restrict__ x,
                             const double *__restrict__ y, const double *__restrict__ z,
                             const double *__restrict__ m, double4_32a *__restrict__ sb)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n)
        return;
    const int j = perm[q];
    sb[q] = make_double4_32a(x[j], y[j], z[j], m[j]);
}

// Centre of mass and mass of every cell from the current positions of its
// member bodies (sorted range [first, first+count) of sb); one warp per cell,
// the lanes' partial sums combined by a fixed butterfly (deterministic).
__global__ void k_adj_moments(const NodeLink *__restrict__ link, int nn,
                              const double4_32a *__restrict__ sb, double4_32a *__restrict__ xm)
{
    const int w = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= nn)
        return;
    const NodeLink l = link[w];
    double M = 0.0, sx = 0.0, sy = 0.0, sz = 0.0;
    for (int q = l.first + lane; q < l.first + l.count; q += CSG_WARP) {
        const double4_32a b = sb[q];
        M += b.w;
        sx += b.w * b.x;
        sy += b.w * b.y;
        sz += b.w * b.z;
    }
    M = warp_sum(M);
    sx = warp_sum(sx);
    sy = warp_sum(sy);
    sz = warp_sum(sz);
    if (lane == 0)
        xm[w] = make_double4_32a(sx / M, sy / M, sz / M, M);
}

// a_i from the body's list; one warp per body (lanes stride the list).
__global__ void k_adj_forces(const int *__restrict__ offs, const int *__restrict__ ids,
                             const double4_32a *__restrict__ xm, const double *__restrict__ x,
                             const double *__restrict__ y, const double *__restrict__ z,
                             const double *__restrict__ m, int n, double G, double eps2,
                             double *__restrict__ ax, double *__restrict__ ay,
                             double *__restrict__ az)
{
    const int i = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= n)
        return;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    if (m[i] > 0.0) {
        const double px = x[i], py = y[i], pz = z[i];
        for (int k = offs[i] + lane; k < offs[i + 1]; k += CSG_WARP) {
            const double4_32a c = xm[ids[k]];
            const double dx = c.x - px, dy = c.y - py, dz = c.z - pz;
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            double inv3, inv5;
            inv_r3_r5(r2, inv3, inv5);
            const double f = G * c.w * inv3;
            sx += f * dx;
            sy += f * dy;
            sz += f * dz;
        }
    }
    sx = warp_sum(sx);
    sy = warp_sum(sy);
    sz = warp_sum(sz);
    if (lane == 0) {
        ax[i] = sx;
        ay[i] = sy;
        az[i] = sz;
    }
}

// Self term of (J^T mu)_i and the scatter of T mu_i into the cells' g.
__global__ void k_adj_jt(const int *__restrict__ offs, const int *__restrict__ ids,
                         const double4_32a *__restrict__ xm, const double *__restrict__ x,
                         const double *__restrict__ y, const double *__restrict__ z,
                         const double *__restrict__ m, const double *__restrict__ mux,
                         const double *__restrict__ muy, const double *__restrict__ muz, int n,
                         double G, double eps2, double *__restrict__ g, double *__restrict__ jx,
                         double *__restrict__ jy, double *__restrict__ jz)
{
    const int i = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= n)
        return;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    if (m[i] > 0.0) {
        const double px = x[i], py = y[i], pz = z[i];
        const double ux = mux[i], uy = muy[i], uz = muz[i];
        for (int k = offs[i] + lane; k < offs[i + 1]; k += CSG_WARP) {
            const int c = ids[k];
            const double4_32a q = xm[c];
            const double dx = q.x - px, dy = q.y - py, dz = q.z - pz;
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            double inv3, inv5;
            inv_r3_r5(r2, inv3, inv5);
            const double gm = G * q.w;
            const double dm = 3.0 * (dx * ux + dy * uy + dz * uz) * inv5;
            const double wx = gm * (ux * inv3 - dm * dx);
            const double wy = gm * (uy * inv3 - dm * dy);
            const double wz = gm * (uz * inv3 - dm * dz);
            sx += wx;
            sy += wy;
            sz += wz;
            atomicAdd(&g[3 * (size_t)c + 0], wx);
            atomicAdd(&g[3 * (size_t)c + 1], wy);
            atomicAdd(&g[3 * (size_t)c + 2], wz);
        }
    }
    sx = warp_sum(sx);
    sy = warp_sum(sy);
    sz = warp_sum(sz);
    if (lane == 0) {
        jx[i] = -sx;
        jy[i] = -sy;
        jz[i] = -sz;
    }
}

// (J^T mu)_j += m_j * sum over the cells containing j of g_c / M_c.
__global__ void k_adj_push(const int *__restrict__ perm, const int *__restrict__ leaf_of,
                           const NodeLink *__restrict__ link, const double4_32a *__restrict__ xm,
                           const double *__restrict__ g, const double *__restrict__ m, int n_alive,
                           int nn, double *__restrict__ jx, double *__restrict__ jy,
                           double *__restrict__ jz, DevScalars *sc)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_alive)
        return;
    const int j = perm[p];
    double sx = 0.0, sy = 0.0, sz = 0.0;
    int c = leaf_of[p], steps = 0;
    while (c >= 0 && c < nn) {
        if (++steps > CSG_MAX_LEVEL + 1) { // deeper than any tree built here
            dev_fail(sc, CSG_ERR_WALK_LIMIT);
            break;
        }
        const double inv = 1.0 / xm[c].w;
        sx += g[3 * (size_t)c + 0] * inv;
        sy += g[3 * (size_t)c + 1] * inv;
        sz += g[3 * (size_t)c + 2] * inv;
        c = link[c].parent;
    }
    const double mj = m[j];
    jx[j] += mj * sx;
    jy[j] += mj * sy;
    jz[j] += mj * sz;
}

constexpr int DT2 = 128;

__global__ void __launch_bounds__(DT2) k_adj_direct_forces(const double *__restrict__ x,
                                                           const double *__restrict__ y,
                                                           const double *__restrict__ z,
                                                           const double *__restrict__ m, int n,
                                                           double G, double eps2,
                                                           double *__restrict__ ax,
                                                           double *__restrict__ ay,
                                                           double *__restrict__ az)
{
    __shared__ double4_32a sj[DT2];
    const int i = blockIdx.x * DT2 + threadIdx.x;
    const bool live = i < n && m[i] > 0.0;
    const double px = i < n ? x[i] : 0.0, py = i < n ? y[i] : 0.0, pz = i < n ? z[i] : 0.0;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int t = 0; t < n; t += DT2) {
        __syncthreads();
        const int j = t + threadIdx.x;
        sj[threadIdx.x] = (j < n) ? make_double4_32a(x[j], y[j], z[j], m[j] > 0.0 ? m[j] : 0.0)
                                  : make_double4_32a(0.0, 0.0, 0.0, 0.0);
        __syncthreads();
        const int cnt = min(DT2, n - t);
        if (live) {
            for (int q = 0; q < cnt; q++) {
                if (t + q == i)
                    continue;
                const double4_32a b = sj[q];
                const double dx = b.x - px, dy = b.y - py, dz = b.z - pz;
                const double r2 = dx * dx + dy * dy + dz * dz + eps2;
                const double f = G * b.w / (r2 * sqrt(r2));
                sx += f * dx;
                sy += f * dy;
                sz += f * dz;
            }
        }
    }
    if (i < n) {
        ax[i] = sx;
        ay[i] = sy;
        az[i] = sz;
    }
}

__global__ void __launch_bounds__(DT2) k_adj_direct_jt(const double *__restrict__ x,
                                                       const double *__restrict__ y,
                                                       const double *__restrict__ z,
                                                       const double *__restrict__ m,
                                                       const double *__restrict__ mux,
                                                       const double *__restrict__ muy,
                                                       const double *__restrict__ muz, int n,
                                                       double G, double eps2,
                                                       double *__restrict__ jx,
                                                       double *__restrict__ jy,
                                                       double *__restrict__ jz)
{
    __shared__ double4_32a sp[DT2];
    __shared__ double3 su[DT2];
    const int j = blockIdx.x * DT2 + threadIdx.x;
    const bool live = j < n && m[j] > 0.0;
    const double px = j < n ? x[j] : 0.0, py = j < n ? y[j] : 0.0, pz = j < n ? z[j] : 0.0;
    const double mj = live ? m[j] : 0.0;
    const double ux = live ? mux[j] : 0.0, uy = live ? muy[j] : 0.0, uz = live ? muz[j] : 0.0;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int t = 0; t < n; t += DT2) {
        __syncthreads();
        const int i = t + threadIdx.x;
        const bool li = i < n && m[i] > 0.0;
        sp[threadIdx.x] = li ? make_double4_32a(x[i], y[i], z[i], m[i]) : make_double4_32a(0, 0, 0, 0);
        su[threadIdx.x] = li ? make_double3(mux[i], muy[i], muz[i]) : make_double3(0, 0, 0);
        __syncthreads();
        const int cnt = min(DT2, n - t);
        if (live) {
            for (int q = 0; q < cnt; q++) {
                const double4_32a b = sp[q];
                if (t + q == j || b.w == 0.0)
                    continue;
                const double3 u = su[q];
                // v = m_j mu_i - m_i mu_j, T1(d) v = v/r^3 - 3 d (d.v)/r^5
                const double vx = mj * u.x - b.w * ux, vy = mj * u.y - b.w * uy,
                             vz = mj * u.z - b.w * uz;
                const double dx = b.x - px, dy = b.y - py, dz = b.z - pz;
                const double r2 = dx * dx + dy * dy + dz * dz + eps2;
                const double inv3 = 1.0 / (r2 * sqrt(r2));
                const double dv = 3.0 * (dx * vx + dy * vy + dz * vz) * inv3 / r2;
                sx += vx * inv3 - dv * dx;
                sy += vy * inv3 - dv * dy;
                sz += vz * inv3 - dv * dz;
            }
        }
    }
    if (j < n) {
        jx[j] = G * sx;
        jy[j] = G * sy;
        jz[j] = G * sz;
    }
}

// lambda_v += dt lambda_x, mu = scale * lambda_v (dead bodies: all zero).
__global__ void k_adj_drift(int n, const double *__restrict__ m, double dt, double scale,
                            double *lx, double *ly, double *lz, double *lvx, double *lvy,
                            double *lvz, double *mux, double *muy, double *muz)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    if (!(m[i] > 0.0)) {
        lx[i] = ly[i] = lz[i] = lvx[i] = lvy[i] = lvz[i] = 0.0;
        mux[i] = muy[i] = muz[i] = 0.0;
        return;
    }
    lvx[i] += dt * lx[i];
    lvy[i] += dt * ly[i];
    lvz[i] += dt * lz[i];
    mux[i] = scale * lvx[i];
    muy[i] = scale * lvy[i];
    muz[i] = scale * lvz[i];
}

__global__ void k_adj_add(int n, const double *__restrict__ m, const double *__restrict__ jx,
                          const double *__restrict__ jy, const double *__restrict__ jz, double *lx,
                          double *ly, double *lz)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !(m[i] > 0.0))
        return;
    lx[i] += jx[i];
    ly[i] += jy[i];
    lz[i] += jz[i];
}

// One substep's frozen tree and interaction lists.
struct Slot {
    double *x = nullptr, *y = nullptr, *z = nullptr; // positions (caller order)
    int *perm = nullptr;                             // sorted alive bodies
    int *leaf_of = nullptr;                          // sorted position -> leaf cell
    NodeLink *link = nullptr;                        // cells
    int *offs = nullptr;                             // n+1 list offsets (caller order)
    int *ids = nullptr;                              // list entries (cell ids)
    int nn = 0, n_alive = 0;
    long long total = 0, cap_ids = 0;
};

template <typename T>
cudaError_t alloc(T **p, size_t count)
{
    *p = nullptr;
    return csgd_malloc((void **)p, sizeof(T) * (count ? count : 1));
}

} // namespace

struct csg_adjoint {
    csgd_t *d = nullptr;
    int n = 0, T = 0, K = 0, mode = 0;
    double G = 1.0, eps = 0.0, theta = 0.5, dt = 0.0;
    std::vector<Slot> slots;
    int recorded = 0;     // slots hold every substep of the last forward
    int have_forward = 0;
    std::vector<double *> ckpt; // 6n doubles per checkpoint (x y z vx vy vz)
    double *lam = nullptr;      // 6n: lambda x y z, lambda v x y z
    double *mu = nullptr;       // 3n
    double *jt = nullptr;       // 3n
    double *g = nullptr;        // 3 per cell
    double4_32a *xm = nullptr;      // per cell
    double4_32a *sb = nullptr;      // per sorted position: x y z m (moment pass)
    int *counts = nullptr;      // n
    int *h_total = nullptr;     // pinned: list entries of the current substep
    std::vector<double> host_m, final_x, target;
    double loss = 0.0;
    int n_alive = 0;
    long long interactions = 0; // list entries over the last forward
    size_t bytes = 0;
};

namespace {

csgd_force_params walk_params(const csg_adjoint *a)
{
    csgd_force_params p;
    p.G = a->G;
    p.softening = a->eps;
    p.theta = a->theta;
    p.precision = CSG_PREC_FP64;
    return p;
}

int cuda_rc(csg_adjoint *a, cudaError_t e)
{
    if (e == cudaSuccess)
        return CSG_OK;
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? CSG_ERR_NOMEM : CSG_ERR_CUDA;
}

void free_slot(Slot &s)
{
    void *p[] = {s.x, s.y, s.z, s.perm, s.leaf_of, s.link, s.offs, s.ids};
    for (void *q : p)
        if (q)
            cudaFree(q);
    s = Slot();
}

int ensure_slots(csg_adjoint *a, int count)
{
    const int n = a->n, ncap = 8 * n + 64;
    while ((int)a->slots.size() < count) {
        Slot s;
        cudaError_t e = alloc(&s.x, n);
        if (e == cudaSuccess) e = alloc(&s.y, n);
        if (e == cudaSuccess) e = alloc(&s.z, n);
        if (e == cudaSuccess && a->mode == CSG_ADJ_TREE) {
            e = alloc(&s.perm, n);
            if (e == cudaSuccess) e = alloc(&s.leaf_of, n);
            if (e == cudaSuccess) e = alloc(&s.link, ncap);
            if (e == cudaSuccess) e = alloc(&s.offs, (size_t)n + 1);
        }
        if (e != cudaSuccess) {
            free_slot(s);
            return cuda_rc(a, e);
        }
        a->bytes += sizeof(double) * 3 * (size_t)n;
        if (a->mode == CSG_ADJ_TREE)
            a->bytes += sizeof(int) * (3 * (size_t)n + 1) + sizeof(NodeLink) * (size_t)ncap;
        a->slots.push_back(s);
    }
    return CSG_OK;
}

// Forces of the current positions (d->x..) into d->ax.., recording the tree
// and lists into slot s (tree mode) or the positions only (direct mode).
int eval(csg_adjoint *a, Slot &s)
{
    csgd_t *d = a->d;
    cudaStream_t st = d->stream;
    const int n = a->n;
    cudaMemcpyAsync(s.x, d->x, sizeof(double) * n, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(s.y, d->y, sizeof(double) * n, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(s.z, d->z, sizeof(double) * n, cudaMemcpyDeviceToDevice, st);
    if (a->mode == CSG_ADJ_DIRECT) {
        { k_adj_direct_forces<<<csgd_grid(n, DT2), DT2, 0, st>>>(d->x, d->y, d->z, d->m, n, a->G, a->eps * a->eps, d->ax, d->ay, d->az); d->launches++; }
        return csgd_check(d, cudaGetLastError());
    }
    int rc = csgd_build_tree(d, 0);
    int nn = 0;
    if (!rc)
        rc = csgd_node_count(d, &nn); // syncs; also reports build errors
    if (rc)
        return rc;
    s.nn = nn;
    s.n_alive = d->sc_host->n_alive;
    cudaMemcpyAsync(s.perm, d->perm, sizeof(int) * n, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(s.link, d->link, sizeof(NodeLink) * (size_t)nn, cudaMemcpyDeviceToDevice, st);
    { k_adj_leaf_of<<<csgd_grid(nn, AT), AT, 0, st>>>(d->link, d->w64, nn, s.leaf_of); d->launches++; }
    const csgd_force_params p = walk_params(a);
    cudaMemsetAsync(a->counts, 0, sizeof(int) * n, st);
    rc = csgd_walk_lists(d, &p, a->counts, nullptr, nullptr, 0, 0);
    if (!rc)
        rc = csg_scan_exclusive(d, a->counts, s.offs, n, nullptr);
    int total = 0;
    if (!rc) {
        cudaMemcpyAsync(a->h_total, s.offs + n, sizeof(int), cudaMemcpyDeviceToHost, st);
        rc = csgd_sync(d);
        total = *a->h_total;
    }
    if (rc)
        return rc;
    if (total < 0) { // more entries than an int offset holds
        csgd_set_err(d, CSG_ERR_NODE_CAPACITY);
        return CSG_ERR_NODE_CAPACITY;
    }
    if (total > s.cap_ids) {
        if (s.ids)
            cudaFree(s.ids);
        a->bytes -= sizeof(int) * (size_t)s.cap_ids;
        s.cap_ids = total + total / 4 + 1024;
        cudaError_t e = alloc(&s.ids, (size_t)s.cap_ids);
        if (e != cudaSuccess) {
            s.cap_ids = 0;
            return cuda_rc(a, e);
        }
        a->bytes += sizeof(int) * (size_t)s.cap_ids;
    }
    s.total = total;
    a->interactions += total;
    rc = csgd_walk_lists(d, &p, a->counts, s.offs, s.ids, total, 1);
    if (rc)
        return rc;
    const int wb = AT / CSG_WARP;
    { k_adj_gather<<<csgd_grid(n, AT), AT, 0, st>>>(s.perm, n, d->x, d->y, d->z, d->m, a->sb); d->launches++; }
    { k_adj_moments<<<csgd_grid(nn, wb), AT, 0, st>>>(s.link, nn, a->sb, a->xm); d->launches++; }
    { k_adj_forces<<<csgd_grid(n, wb), AT, 0, st>>>(s.offs, s.ids, a->xm, d->x, d->y, d->z, d->m, n, a->G, a->eps * a->eps, d->ax, d->ay, d->az); d->launches++; }
    return csgd_check(d, cudaGetLastError());
}

// Forces of the current positions with slot s's frozen cells and lists.
int eval_frozen(csg_adjoint *a, const Slot &s)
{
    csgd_t *d = a->d;
    cudaStream_t st = d->stream;
    const int n = a->n;
    if (a->mode == CSG_ADJ_DIRECT) {
        { k_adj_direct_forces<<<csgd_grid(n, DT2), DT2, 0, st>>>(d->x, d->y, d->z, d->m, n, a->G, a->eps * a->eps, d->ax, d->ay, d->az); d->launches++; }
        return csgd_check(d, cudaGetLastError());
    }
    const int wb = AT / CSG_WARP;
    { k_adj_gather<<<csgd_grid(n, AT), AT, 0, st>>>(s.perm, n, d->x, d->y, d->z, d->m, a->sb); d->launches++; }
    { k_adj_moments<<<csgd_grid(s.nn, wb), AT, 0, st>>>(s.link, s.nn, a->sb, a->xm); d->launches++; }
    { k_adj_forces<<<csgd_grid(n, wb), AT, 0, st>>>(s.offs, s.ids, a->xm, d->x, d->y, d->z, d->m, n, a->G, a->eps * a->eps, d->ax, d->ay, d->az); d->launches++; }
    return csgd_check(d, cudaGetLastError());
}

// jt = J(x_s)^T mu.
int jt_product(csg_adjoint *a, const Slot &s)
{
    csgd_t *d = a->d;
    cudaStream_t st = d->stream;
    const int n = a->n;
    const double *mux = a->mu, *muy = a->mu + n, *muz = a->mu + 2 * (size_t)n;
    double *jx = a->jt, *jy = a->jt + n, *jz = a->jt + 2 * (size_t)n;
    if (a->mode == CSG_ADJ_DIRECT) {
        { k_adj_direct_jt<<<csgd_grid(n, DT2), DT2, 0, st>>>(s.x, s.y, s.z, d->m, mux, muy, muz, n, a->G, a->eps * a->eps, jx, jy, jz); d->launches++; }
        return csgd_check(d, cudaGetLastError());
    }
    const int wb = AT / CSG_WARP;
    cudaMemsetAsync(a->g, 0, sizeof(double) * 3 * (size_t)s.nn, st);
    { k_adj_gather<<<csgd_grid(n, AT), AT, 0, st>>>(s.perm, n, s.x, s.y, s.z, d->m, a->sb); d->launches++; }
    { k_adj_moments<<<csgd_grid(s.nn, wb), AT, 0, st>>>(s.link, s.nn, a->sb, a->xm); d->launches++; }
    { k_adj_jt<<<csgd_grid(n, wb), AT, 0, st>>>(s.offs, s.ids, a->xm, s.x, s.y, s.z, d->m, mux, muy, muz, n, a->G, a->eps * a->eps, a->g, jx, jy, jz); d->launches++; }
    { k_adj_push<<<csgd_grid(s.n_alive, AT), AT, 0, st>>>(s.perm, s.leaf_of, s.link, a->xm, a->g, d->m, s.n_alive, s.nn, jx, jy, jz, d->sc); d->launches++; }
    return csgd_check(d, cudaGetLastError());
}

int save_state(csg_adjoint *a, double *dst)
{
    csgd_t *d = a->d;
    const size_t n = (size_t)a->n;
    double *src[6] = {d->x, d->y, d->z, d->vx, d->vy, d->vz};
    for (int k = 0; k < 6; k++)
        cudaMemcpyAsync(dst + k * n, src[k], sizeof(double) * n, cudaMemcpyDeviceToDevice, d->stream);
    return csgd_check(d, cudaGetLastError());
}

int load_state(csg_adjoint *a, const double *src)
{
    csgd_t *d = a->d;
    const size_t n = (size_t)a->n;
    double *dst[6] = {d->x, d->y, d->z, d->vx, d->vy, d->vz};
    for (int k = 0; k < 6; k++)
        cudaMemcpyAsync(dst[k], src + k * n, sizeof(double) * n, cudaMemcpyDeviceToDevice, d->stream);
    return csgd_check(d, cudaGetLastError());
}

// Mean squared distance of the alive bodies' positions to the target.
int finish_loss(csg_adjoint *a, double *loss)
{
    csgd_t *d = a->d;
    const size_t n = (size_t)a->n;
    a->final_x.resize(3 * n);
    cudaMemcpyAsync(a->final_x.data(), d->x, sizeof(double) * n, cudaMemcpyDeviceToHost, d->stream);
    cudaMemcpyAsync(a->final_x.data() + n, d->y, sizeof(double) * n, cudaMemcpyDeviceToHost, d->stream);
    cudaMemcpyAsync(a->final_x.data() + 2 * n, d->z, sizeof(double) * n, cudaMemcpyDeviceToHost,
                    d->stream);
    int rc = csgd_sync(d);
    if (rc)
        return rc;
    double s = 0.0;
    for (size_t i = 0; i < n; i++) {
        if (!(a->host_m[i] > 0.0))
            continue;
        for (int k = 0; k < 3; k++) {
            const double e = a->final_x[k * n + i] - a->target[3 * i + k];
            s += e * e;
        }
    }
    a->loss = a->n_alive > 0 ? s / a->n_alive : 0.0;
    if (loss)
        *loss = a->loss;
    return CSG_OK;
}

int start_run(csg_adjoint *a, const Body *bodies, const double *target)
{
    csgd_t *d = a->d;
    int rc = csgd_upload_bodies(d, bodies, a->n);
    if (rc)
        return rc;
    a->host_m.resize(a->n);
    a->target.assign(target, target + 3 * (size_t)a->n);
    a->n_alive = 0;
    for (int i = 0; i < a->n; i++) {
        a->host_m[i] = bodies[i].mass;
        if (bodies[i].mass > 0.0)
            a->n_alive++;
    }
    return CSG_OK;
}

} // namespace

extern "C" {

CSG_EXPORT csg_adjoint *csg_adjoint_create(int n, const CsgSimParams *params, int checkpoint_every,
                                           int mode)
{
    if (n < 1 || !params || params->substeps < 1 || checkpoint_every < 1 || params->sph ||
        (mode != CSG_ADJ_TREE && mode != CSG_ADJ_DIRECT) || !(params->dt > 0.0)) {
        csg_thread_set_error(CSG_ERR_BAD_ARG);
        return nullptr;
    }
    csg_adjoint *a = new csg_adjoint();
    a->d = csgd_create();
    if (!a->d) {
        delete a;
        csg_thread_set_error(CSG_ERR_NO_DEVICE);
        return nullptr;
    }
    a->n = n;
    a->T = params->substeps;
    a->K = checkpoint_every;
    a->mode = mode;
    a->G = params->G;
    a->eps = params->softening;
    a->theta = params->theta;
    a->dt = params->dt;
    const size_t ncap = 8 * (size_t)n + 64;
    int rc = csgd_reserve(a->d, n);
    cudaError_t e = cudaSuccess;
    if (!rc) {
        e = alloc(&a->lam, 6 * (size_t)n);
        if (e == cudaSuccess) e = alloc(&a->mu, 3 * (size_t)n);
        if (e == cudaSuccess) e = alloc(&a->jt, 3 * (size_t)n);
        if (e == cudaSuccess) e = alloc(&a->g, 3 * ncap);
        if (e == cudaSuccess) e = alloc(&a->xm, ncap);
        if (e == cudaSuccess) e = alloc(&a->sb, (size_t)n);
        if (e == cudaSuccess) e = alloc(&a->counts, (size_t)n);
        if (e == cudaSuccess) e = csgd_malloc_host((void **)&a->h_total, sizeof(int));
        rc = cuda_rc(a, e);
    }
    if (!rc) {
        const int nck = (a->T + a->K - 1) / a->K;
        for (int k = 0; k < nck && !rc; k++) {
            double *c = nullptr;
            rc = cuda_rc(a, alloc(&c, 6 * (size_t)n));
            if (!rc)
                a->ckpt.push_back(c);
        }
        a->bytes = sizeof(double) * (6 * (size_t)n * (nck + 1) + 6 * (size_t)n + 3 * ncap) +
                   sizeof(double4_32a) * ncap + sizeof(int) * (size_t)n;
    }
    if (rc) {
        csg_adjoint_destroy(a);
        csg_thread_set_error(rc);
        return nullptr;
    }
    csg_thread_set_error(CSG_OK);
    return a;
}

CSG_EXPORT void csg_adjoint_destroy(csg_adjoint *a)
{
    if (!a)
        return;
    if (a->d)
        cudaStreamSynchronize(a->d->stream);
    if (a->h_total)
        cudaFreeHost(a->h_total);
    for (Slot &s : a->slots)
        free_slot(s);
    for (double *c : a->ckpt)
        cudaFree(c);
    void *p[] = {a->lam, a->mu, a->jt, a->g, a->xm, a->sb, a->counts};
    for (void *q : p)
        if (q)
            cudaFree(q);
    if (a->d)
        csgd_destroy(a->d);
    delete a;
}

CSG_EXPORT int csg_adjoint_forward(csg_adjoint *a, const Body *bodies, const double *target,
                                   int record, double *loss, Body *final_out)
{
    if (!a || !bodies || !target)
        return CSG_ERR_BAD_ARG;
    csgd_t *d = a->d;
    a->have_forward = 0;
    a->recorded = 0;
    a->interactions = 0;
    int rc = start_run(a, bodies, target);
    if (!rc)
        rc = ensure_slots(a, record ? a->T + 1 : 1);
    if (!rc)
        rc = save_state(a, a->ckpt[0]);
    if (!rc)
        rc = eval(a, a->slots[0]);
    for (int n = 0; n < a->T && !rc; n++) {
        rc = csgd_kick_drift(d, a->dt);
        if (!rc)
            rc = eval(a, a->slots[record ? n + 1 : 0]);
        if (!rc)
            rc = csgd_kick(d, a->dt);
        if (!rc && (n + 1) % a->K == 0 && n + 1 < a->T)
            rc = save_state(a, a->ckpt[(n + 1) / a->K]);
    }
    if (!rc)
        rc = finish_loss(a, loss);
    if (!rc && final_out) {
        rc = csgd_download_bodies(d, final_out, a->n);
        if (!rc)
            rc = csgd_sync(d);
    }
    if (!rc) {
        a->have_forward = 1;
        a->recorded = record ? 1 : 0;
    }
    return rc;
}

CSG_EXPORT int csg_adjoint_forward_frozen(csg_adjoint *a, const Body *bodies, const double *target,
                                          double *loss)
{
    if (!a || !bodies || !target)
        return CSG_ERR_BAD_ARG;
    if (!a->recorded)
        return CSG_ERR_BAD_ARG; // needs a forward run with record = 1
    csgd_t *d = a->d;
    for (int i = 0; i < a->n; i++) // the lists belong to the recorded run's masses
        if (bodies[i].mass != a->host_m[i])
            return CSG_ERR_BAD_ARG;
    // the recorded run stays the one backward differentiates
    std::vector<double> keep_target = a->target;
    const int keep_alive = a->n_alive;
    int rc = start_run(a, bodies, target);
    if (!rc)
        rc = eval_frozen(a, a->slots[0]);
    for (int n = 0; n < a->T && !rc; n++) {
        rc = csgd_kick_drift(d, a->dt);
        if (!rc)
            rc = eval_frozen(a, a->slots[n + 1]);
        if (!rc)
            rc = csgd_kick(d, a->dt);
    }
    // the recorded run's final positions stay those of the recorded run
    std::vector<double> keep;
    keep.swap(a->final_x);
    const double keep_loss = a->loss;
    if (!rc)
        rc = finish_loss(a, loss);
    a->final_x.swap(keep);
    a->loss = keep_loss;
    a->target.swap(keep_target);
    a->n_alive = keep_alive;
    return rc;
}

CSG_EXPORT int csg_adjoint_backward(csg_adjoint *a, double *grad_x, double *grad_v)
{
    if (!a || !grad_x || !grad_v)
        return CSG_ERR_BAD_ARG;
    if (!a->have_forward)
        return CSG_ERR_BAD_ARG;
    csgd_t *d = a->d;
    cudaStream_t st = d->stream;
    const size_t n = (size_t)a->n;
    // lambda_x(T) = 2 (x_T - target) / n_alive, lambda_v(T) = 0
    std::vector<double> h(6 * n, 0.0);
    for (size_t i = 0; i < n; i++) {
        if (!(a->host_m[i] > 0.0) || a->n_alive == 0)
            continue;
        for (int k = 0; k < 3; k++)
            h[k * n + i] = 2.0 * (a->final_x[k * n + i] - a->target[3 * i + k]) / a->n_alive;
    }
    cudaMemcpyAsync(a->lam, h.data(), sizeof(double) * 6 * n, cudaMemcpyHostToDevice, st);
    int rc = csgd_sync(d);
    const long long keep_inter = a->interactions; // recomputed segments do not count
    double *lx = a->lam, *ly = lx + n, *lz = ly + n, *lvx = lz + n, *lvy = lvx + n, *lvz = lvy + n;
    auto reverse_step = [&](int step, const Slot &s) {
        const double scale = (step >= 1) ? a->dt : 0.5 * a->dt;
        { k_adj_drift<<<csgd_grid(a->n, AT), AT, 0, st>>>(a->n, d->m, a->dt, scale, lx, ly, lz, lvx, lvy, lvz, a->mu, a->mu + n, a->mu + 2 * n); d->launches++; }
        int r = jt_product(a, s);
        if (!r)
            { k_adj_add<<<csgd_grid(a->n, AT), AT, 0, st>>>(a->n, d->m, a->jt, a->jt + n, a->jt + 2 * n, lx, ly, lz); d->launches++; }
        return r ? r : csgd_check(d, cudaGetLastError());
    };
    if (!rc && a->recorded) {
        for (int step = a->T - 1; step >= 0 && !rc; step--)
            rc = reverse_step(step, a->slots[step]);
    } else if (!rc) {
        // the masses are the run's (uploaded at forward); rebuild each segment
        rc = ensure_slots(a, a->K);
        const int nseg = (a->T + a->K - 1) / a->K;
        for (int seg = nseg - 1; seg >= 0 && !rc; seg--) {
            const int n0 = seg * a->K, n1 = (n0 + a->K < a->T) ? n0 + a->K : a->T;
            rc = load_state(a, a->ckpt[seg]);
            if (!rc)
                rc = eval(a, a->slots[0]);
            for (int step = n0; step < n1 - 1 && !rc; step++) {
                rc = csgd_kick_drift(d, a->dt);
                if (!rc)
                    rc = eval(a, a->slots[step - n0 + 1]);
                if (!rc)
                    rc = csgd_kick(d, a->dt);
            }
            for (int step = n1 - 1; step >= n0 && !rc; step--)
                rc = reverse_step(step, a->slots[step - n0]);
        }
    }
    a->interactions = keep_inter;
    if (!rc) {
        cudaMemcpyAsync(h.data(), a->lam, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, st);
        rc = csgd_sync(d);
    }
    if (rc)
        return rc;
    for (size_t i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) {
            grad_x[3 * i + k] = h[k * n + i];
            grad_v[3 * i + k] = h[(3 + k) * n + i];
        }
    return CSG_OK;
}

CSG_EXPORT int csg_adjoint_stats(csg_adjoint *a, int64_t *device_bytes, int64_t *interactions,
                                 int64_t *launches)
{
    if (!a)
        return CSG_ERR_BAD_ARG;
    if (launches)
        *launches = (int64_t)a->d->launches;
    if (device_bytes)
        *device_bytes = (int64_t)a->bytes;
    if (interactions)
        *interactions = (int64_t)a->interactions;
    return CSG_OK;
}

} // extern "C"
