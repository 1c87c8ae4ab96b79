// dev_state.cu — device state lifetime, Body I/O, leapfrog and cooling kernels.
//
// Compiled with -fmad=false: the leapfrog and cooling kernels then round every
// operation exactly as the reference's C does (src/integrator.c:22-51,
// src/sph.c:200-231), so given equal accelerations they agree bit for bit.
#include "dev_internal.cuh"

#include <atomic>

#include <nvtx3/nvToolsExt.h>

#include <stddef.h>
#include <stdlib.h>
#include <string.h>

namespace {

constexpr double SPH_GAMMA = 5.0 / 3.0;

__global__ void k_unpack(const Body *__restrict__ b, int n, double *x, double *y, double *z,
                         double *vx, double *vy, double *vz, double *ax, double *ay, double *az,
                         double *m, int *type, double *rho, double *P, double *u, double *h)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const Body &q = b[i];
    x[i] = q.x;
    y[i] = q.y;
    z[i] = q.z;
    vx[i] = q.vx;
    vy[i] = q.vy;
    vz[i] = q.vz;
    ax[i] = q.ax;
    ay[i] = q.ay;
    az[i] = q.az;
    m[i] = q.mass;
    type[i] = (int)q.type;
    rho[i] = q.density;
    P[i] = q.pressure;
    u[i] = q.internal_energy;
    h[i] = q.smoothing_h;
}

// Writes back the fields kept in SoA; the quasar fields (spin, accretion
// rate, luminosity, lifetime) keep the values the staging copy holds.
__global__ void k_pack(Body *__restrict__ b, int n, const double *x, const double *y,
                       const double *z, const double *vx, const double *vy, const double *vz,
                       const double *ax, const double *ay, const double *az, const double *rho,
                       const double *P, const double *u, const double *h, const double *m,
                       const int *type)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    Body &q = b[i];
    q.x = x[i];
    q.y = y[i];
    q.z = z[i];
    q.vx = vx[i];
    q.vy = vy[i];
    q.vz = vz[i];
    q.ax = ax[i];
    q.ay = ay[i];
    q.az = az[i];
    q.density = rho[i];
    q.pressure = P[i];
    q.internal_energy = u[i];
    q.smoothing_h = h[i];
    q.mass = m[i];
    // type and the 4 padding bytes after it as one 8-byte word: the padding
    // leaves the device as zeros instead of whatever a wider store would put
    // there (offset 80 of a 168-byte record: 8-byte aligned)
    static_assert(offsetof(Body, type) == 80 && sizeof(Body) % 8 == 0, "Body layout");
    *reinterpret_cast<int2 *>(&q.type) = make_int2(type[i], 0);
}

// Half kick and drift, src/integrator.c:22-31.
__global__ void k_kick_drift(int n, double dt, const double *__restrict__ m, double *x, double *y,
                             double *z, double *vx, double *vy, double *vz,
                             const double *__restrict__ ax, const double *__restrict__ ay,
                             const double *__restrict__ az)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || m[i] <= 0.0)
        return;
    double v0 = vx[i] + 0.5 * ax[i] * dt;
    double v1 = vy[i] + 0.5 * ay[i] * dt;
    double v2 = vz[i] + 0.5 * az[i] * dt;
    vx[i] = v0;
    vy[i] = v1;
    vz[i] = v2;
    x[i] = x[i] + v0 * dt;
    y[i] = y[i] + v1 * dt;
    z[i] = z[i] + v2 * dt;
}

// Half kick, src/integrator.c:45-51.
__global__ void k_kick(int n, double dt, const double *__restrict__ m, double *vx, double *vy,
                       double *vz, const double *__restrict__ ax, const double *__restrict__ ay,
                       const double *__restrict__ az)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || m[i] <= 0.0)
        return;
    vx[i] = vx[i] + 0.5 * ax[i] * dt;
    vy[i] = vy[i] + 0.5 * ay[i] * dt;
    vz[i] = vz[i] + 0.5 * az[i] * dt;
}

// Implicit radiative cooling, src/sph.c:200-231.
__global__ void k_cooling(int n, double dt, const double *__restrict__ m,
                          const int *__restrict__ type, const double *__restrict__ rho, double *u,
                          double *P)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || type[i] != BODY_GAS || m[i] <= 0.0)
        return;
    const double lambda0 = 0.05;
    double ui = u[i];
    double r = rho[i];
    if (ui < 1e-15 || r < 1e-15)
        return;
    double un = ui / (1.0 + dt * lambda0 * r * 0.5 / sqrt(ui));
    if (un < 0.01)
        un = 0.01;
    u[i] = un;
    P[i] = (SPH_GAMMA - 1.0) * r * un;
}

__global__ void k_alive_count(int n, const double *__restrict__ m, DevScalars *sc)
{
    int c = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        c += (m[i] <= 0.0) ? 0 : 1;
    c = __reduce_add_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0 && c)
        atomicAdd(&sc->alive_count, c);
}

template <typename T>
cudaError_t dalloc(T **p, size_t count)
{
    *p = nullptr;
    if (count == 0)
        count = 1;
    return csgd_malloc((void **)p, sizeof(T) * count);
}

} // namespace

// Allocations still allowed before injected failures begin; < 0: no injection.
static std::atomic<long long> g_alloc_allowance{-1};

static bool alloc_injected_failure()
{
    long long a = g_alloc_allowance.load();
    while (a >= 0) {
        if (a == 0)
            return true;
        if (g_alloc_allowance.compare_exchange_weak(a, a - 1))
            return false;
    }
    return false;
}

cudaError_t csgd_malloc(void **p, size_t bytes)
{
    *p = nullptr;
    if (alloc_injected_failure())
        return cudaErrorMemoryAllocation;
    return cudaMalloc(p, bytes);
}

cudaError_t csgd_malloc_host(void **p, size_t bytes)
{
    *p = nullptr;
    if (alloc_injected_failure())
        return cudaErrorMemoryAllocation;
    return cudaMallocHost(p, bytes);
}

extern "C" int csgd_has_device(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n > 0;
}

extern "C" void csgd_set_wait_limit(csgd_t *d, int polls)
{
    cudaStreamSynchronize(d->stream);
    csgd_drop_graph(d); // captured walks carry the limit in their arguments
    d->wait_polls = polls > 0 ? polls : 0;
}

// Fault injection for tests: the next `allow` device or pinned allocations
// of the library succeed, every later one fails (as an out-of-memory GPU
// would) until csg_inject_alloc_failure(-1) clears it.
extern "C" CSG_EXPORT void csg_inject_alloc_failure(long long allow)
{
    g_alloc_allowance.store(allow < 0 ? -1 : allow);
}

namespace {

void free_bodies(csgd_t *d)
{
    void *ptrs[] = {d->x, d->y, d->z, d->vx, d->vy, d->vz, d->ax, d->ay, d->az, d->m,
                    d->rho, d->P, d->u, d->h, d->type, d->aos, d->key, d->key_alt, d->perm,
                    d->perm_alt, d->ext, d->sort_hist, d->lcp, d->cnt, d->base, d->scan_tmp,
                    d->gas, d->w64, d->w32, d->link, d->geo, d->s32, d->child, d->nchild, d->ticket,
                    d->minidx, d->ord_key, d->ord_key_alt, d->ord_id, d->ord_id_alt, d->rank,
                    d->pool, d->gid, d->sgid, d->tasks};
    for (void *p : ptrs)
        if (p)
            cudaFree(p);
    d->x = d->y = d->z = d->vx = d->vy = d->vz = d->ax = d->ay = d->az = d->m = nullptr;
    d->rho = d->P = d->u = d->h = nullptr;
    d->type = nullptr;
    d->aos = nullptr;
    d->key = d->key_alt = nullptr;
    d->perm = d->perm_alt = nullptr;
    d->ext = nullptr;
    d->sort_hist = nullptr;
    d->lcp = nullptr;
    d->cnt = d->base = d->scan_tmp = d->gas = nullptr;
    d->w64 = nullptr;
    d->w32 = nullptr;
    d->link = nullptr;
    d->geo = nullptr;
    d->s32 = nullptr;
    d->child = d->nchild = d->ticket = nullptr;
    d->minidx = nullptr;
    d->ord_key = d->ord_key_alt = nullptr;
    d->ord_id = d->ord_id_alt = d->rank = nullptr;
    d->pool = nullptr;
    d->gid = d->sgid = nullptr;
    d->tasks = nullptr;
    d->task_cap = 0;
    d->cap = 0;
    d->node_cap = 0;
}

} // namespace

// ---- shared helpers ----------------------------------------------------------

int csgd_grid(long long n, int block)
{
    long long g = (n + block - 1) / block;
    return (int)(g > 0 ? g : 1);
}

// Records the first error of a launch sequence; the next csgd_sync reports
// and clears it. Argument errors are returned to the caller at once instead,
// so that a refused call leaves nothing for a later call to report.
void csgd_set_err(csgd_t *d, int code)
{
    if (d->host_err == 0)
        d->host_err = code;
}

int csgd_check(csgd_t *d, cudaError_t e)
{
    if (e == cudaSuccess)
        return CSG_OK;
    csgd_set_err(d, CSG_ERR_CUDA);
    return CSG_ERR_CUDA;
}

extern "C" const char *csgd_error_string(int code)
{
    switch (code) {
    case CSG_OK:
        return "ok";
    case CSG_ERR_CUDA:
        return "CUDA runtime error";
    case CSG_ERR_NOMEM:
        return "out of memory";
    case CSG_ERR_NODE_CAPACITY:
        return "tree needs more than 8*n+64 nodes";
    case CSG_ERR_BAD_ARG:
        return "invalid argument";
    case CSG_ERR_BAD_POOL:
        return "octree pool is not a tree";
    case CSG_ERR_WALK_LIMIT:
        return "tree walk stopped on a malformed tree";
    case CSG_ERR_DEVICE_WAIT:
        return "a device-side wait gave up (bounded wait expired)";
    case CSG_ERR_NO_DEVICE:
        return "no CUDA device";
    case CSG_ERR_UNSUPPORTED:
        return "needs a component that is not linked";
    default:
        return "unknown error";
    }
}

// ---- lifetime ------------------------------------------------------------

extern "C" csgd_t *csgd_create(void)
{
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0)
        return nullptr;
    csgd_t *d = (csgd_t *)calloc(1, sizeof(csgd_t));
    if (!d)
        return nullptr;
    if (cudaStreamCreateWithFlags(&d->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        free(d);
        return nullptr;
    }
    d->stream = d->own_stream;
    if (cudaStreamCreateWithFlags(&d->aux, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&d->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&d->ev_join, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError(); // no overlap then: SPH runs on the main stream
        if (d->aux)
            cudaStreamDestroy(d->aux);
        if (d->ev_fork)
            cudaEventDestroy(d->ev_fork);
        d->aux = nullptr;
        d->ev_fork = d->ev_join = nullptr;
    }
    if (cudaStreamCreateWithFlags(&d->aux2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&d->ev_fork2, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&d->ev_join2, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError(); // no overlap then: pool exports follow the substep
        if (d->aux2)
            cudaStreamDestroy(d->aux2);
        if (d->ev_fork2)
            cudaEventDestroy(d->ev_fork2);
        d->aux2 = nullptr;
        d->ev_fork2 = d->ev_join2 = nullptr;
    }
    d->use_graphs = 1;
    d->n_gal = 1;
    d->walk_warps = 4; // fastest one-warp-per-task shape at 20k..1M bodies
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && sms > 0)
        d->num_sms = sms;
    else
        d->num_sms = 152;
    d->gal_cap = 1;
    if (csgd_malloc((void **)&d->roots, sizeof(DevRoot)) != cudaSuccess ||
        csgd_malloc((void **)&d->sc, sizeof(DevScalars)) != cudaSuccess ||
        csgd_malloc_host((void **)&d->sc_host, sizeof(DevScalars)) != cudaSuccess ||
        csgd_malloc_host((void **)&d->h_int, 4 * sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        csgd_destroy(d); // frees what was made, streams and events included
        return nullptr;
    }
    memset(d->sc_host, 0, sizeof(DevScalars));
    cudaMemsetAsync(d->sc, 0, sizeof(DevScalars), d->stream);
    return d;
}

extern "C" void csgd_destroy(csgd_t *d)
{
    if (!d)
        return;
    cudaStreamSynchronize(d->stream);
    if (d->graph)
        cudaGraphExecDestroy(d->graph);
    free_bodies(d);
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
    if (d->sc)
        cudaFree(d->sc);
    if (d->roots)
        cudaFree(d->roots);
    if (d->sys_n)
        cudaFree(d->sys_n);
    if (d->sc_host)
        cudaFreeHost(d->sc_host);
    if (d->h_int)
        cudaFreeHost(d->h_int);
    if (d->qs)
        cudaFree(d->qs);
    if (d->wpart)
        cudaFree(d->wpart);
    csgd_quasar_free(d);
    if (d->aux) {
        cudaStreamSynchronize(d->aux);
        cudaStreamDestroy(d->aux);
        cudaEventDestroy(d->ev_fork);
        cudaEventDestroy(d->ev_join);
    }
    if (d->aux2) {
        cudaStreamSynchronize(d->aux2);
        cudaStreamDestroy(d->aux2);
        cudaEventDestroy(d->ev_fork2);
        cudaEventDestroy(d->ev_join2);
    }
    for (int k = 0; k < 7; k++)
        if (d->tev[k])
            cudaEventDestroy(d->tev[k]);
    for (int k = 0; k < 3; k++)
        if (d->taux[k])
            cudaEventDestroy(d->taux[k]);
    for (int k = 0; k < 6; k++)
        if (d->bev[k])
            cudaEventDestroy(d->bev[k]);
    if (d->own_stream)
        cudaStreamDestroy(d->own_stream);
    free(d);
}

extern "C" void csgd_set_export_order(csgd_t *d, int on) { d->export_order = on ? 1 : 0; }

extern "C" void csgd_set_stream(csgd_t *d, void *stream)
{
    d->stream = stream ? (cudaStream_t)stream : d->own_stream;
}

extern "C" void *csgd_stream(csgd_t *d) { return (void *)d->stream; }

extern "C" Body *csgd_aos(csgd_t *d) { return d->aos; }

extern "C" int csgd_count(const csgd_t *d) { return d->n; }

extern "C" void csgd_enable_stats(csgd_t *d, int on)
{
    if (d->stats != on && d->graph) { // the captured walk variant changes
        cudaStreamSynchronize(d->stream);
        cudaGraphExecDestroy(d->graph);
        d->graph = nullptr;
    }
    d->stats = on;
}

void csgd_drop_graph(csgd_t *d)
{
    if (d->graph) {
        cudaStreamSynchronize(d->stream);
        cudaGraphExecDestroy(d->graph);
        d->graph = nullptr;
    }
}

extern "C" int csgd_reserve(csgd_t *d, int n)
{
    if (n < 0) {
        return CSG_ERR_BAD_ARG;
    }
    if (n != d->n && d->n_gal > 1) { // the system layout no longer fits: one system
        csgd_drop_graph(d);
        d->n_gal = 1;
        if (d->gid)
            cudaMemsetAsync(d->gid, 0, sizeof(int) * (size_t)d->cap, d->stream);
    }
    d->n = n;
    if (n <= d->cap && d->cap > 0)
        return CSG_OK;
    cudaStreamSynchronize(d->stream);
    csgd_drop_graph(d); // captured pointers are about to change
    free_bodies(d);
    d->cap = d->node_cap = d->task_cap = 0; // nothing is held until every buffer is
    const size_t cap = (size_t)(n > 0 ? n : 1);
    const size_t ncap = 8 * cap + 64; // the reference's pool contract
    bool ok = true;
    ok &= dalloc(&d->x, cap) == cudaSuccess;
    ok &= dalloc(&d->y, cap) == cudaSuccess;
    ok &= dalloc(&d->z, cap) == cudaSuccess;
    ok &= dalloc(&d->vx, cap) == cudaSuccess;
    ok &= dalloc(&d->vy, cap) == cudaSuccess;
    ok &= dalloc(&d->vz, cap) == cudaSuccess;
    ok &= dalloc(&d->ax, cap) == cudaSuccess;
    ok &= dalloc(&d->ay, cap) == cudaSuccess;
    ok &= dalloc(&d->az, cap) == cudaSuccess;
    ok &= dalloc(&d->m, cap) == cudaSuccess;
    ok &= dalloc(&d->rho, cap) == cudaSuccess;
    ok &= dalloc(&d->P, cap) == cudaSuccess;
    ok &= dalloc(&d->u, cap) == cudaSuccess;
    ok &= dalloc(&d->h, cap) == cudaSuccess;
    ok &= dalloc(&d->type, cap) == cudaSuccess;
    ok &= dalloc(&d->aos, cap) == cudaSuccess;
    ok &= dalloc(&d->key, ncap) == cudaSuccess; // the key buffers also sort cells at export
    ok &= dalloc(&d->key_alt, ncap) == cudaSuccess;
    ok &= dalloc(&d->perm, cap) == cudaSuccess;
    ok &= dalloc(&d->perm_alt, cap) == cudaSuccess;
    ok &= dalloc(&d->ext, 3 * cap) == cudaSuccess;
    // radix sort scratch: digit counts and tile counters (8 * 256 + 64 words),
    // then two status buffers of 256 64-bit words per tile; tiles of 512 keys
    // below 64k keys, 1024 below 2M, else 2048 (sized for any key count up to
    // ncap)
    const size_t sort_items = ncap;
    const size_t tiny_items = sort_items < (1u << 16) ? sort_items : (1u << 16) - 1;
    const size_t small_items = sort_items < (2u << 20) ? sort_items : (2u << 20) - 1;
    const size_t tiles_tiny = (tiny_items + 511) / 512;
    const size_t tiles_small = (small_items + 1023) / 1024, tiles_large = (sort_items + 2047) / 2048;
    size_t tiles = tiles_small > tiles_large ? tiles_small : tiles_large;
    tiles = tiles_tiny > tiles ? tiles_tiny : tiles;
    const size_t hist = 256 * tiles;
    d->sort_hist_cap = (int)(4 * hist + 8 * 256 + 64);
    ok &= dalloc(&d->sort_hist, (size_t)d->sort_hist_cap) == cudaSuccess;
    ok &= dalloc(&d->lcp, cap) == cudaSuccess;
    ok &= dalloc(&d->cnt, cap + 1) == cudaSuccess;
    ok &= dalloc(&d->base, cap + 1) == cudaSuccess;
    const size_t scan_len = (cap > hist ? cap : hist);
    d->scan_tmp_cap = (int)(scan_len / 1024 + 4096);
    ok &= dalloc(&d->scan_tmp, (size_t)d->scan_tmp_cap) == cudaSuccess;
    ok &= dalloc(&d->gas, cap) == cudaSuccess;
    ok &= dalloc(&d->w64, ncap) == cudaSuccess;
    ok &= dalloc(&d->w32, ncap) == cudaSuccess;
    ok &= dalloc(&d->link, ncap) == cudaSuccess;
    ok &= dalloc(&d->child, 8 * ncap) == cudaSuccess;
    ok &= dalloc(&d->nchild, ncap) == cudaSuccess;
    ok &= dalloc(&d->ticket, ncap) == cudaSuccess;
    ok &= dalloc(&d->minidx, ncap) == cudaSuccess;
    ok &= dalloc(&d->ord_key, ncap) == cudaSuccess;
    ok &= dalloc(&d->ord_key_alt, ncap) == cudaSuccess;
    ok &= dalloc(&d->ord_id, ncap) == cudaSuccess;
    ok &= dalloc(&d->ord_id_alt, ncap) == cudaSuccess;
    ok &= dalloc(&d->rank, ncap) == cudaSuccess;
    ok &= dalloc(&d->gid, cap) == cudaSuccess;
    ok &= dalloc(&d->sgid, cap) == cudaSuccess;
    const size_t tcap = cap / CSG_WARP + (size_t)d->gal_cap + 2; // >= tasks of any layout
    ok &= dalloc(&d->tasks, tcap) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        free_bodies(d);
        d->n = 0;
        csgd_set_err(d, CSG_ERR_NOMEM);
        return CSG_ERR_NOMEM;
    }
    d->cap = (int)cap;
    d->node_cap = (int)ncap;
    d->task_cap = (int)tcap;
    d->n = n;
    d->n_gal = 1;
    cudaMemsetAsync(d->gid, 0, sizeof(int) * cap, d->stream);
    // the tree stays empty-but-valid until the first build
    cudaMemsetAsync(d->sc, 0, sizeof(DevScalars), d->stream);
    return csgd_check(d, cudaGetLastError());
}

// Cell geometry (SPH, pool export/import) and the reference-layout pool
// staging are allocated on first use: a gravity-only state never holds them
// (184 of the ~370 bytes a node would otherwise take). Not inside a stream
// capture: csgd_prepare_sph allocates them before a substep is captured.
extern "C" int csgd_ensure_tree_extras(csgd_t *d, int geometry, int pool)
{
    const size_t ncap = (size_t)(d->node_cap > 0 ? d->node_cap : 64);
    bool ok = true;
    if (geometry && !d->geo)
        ok &= dalloc(&d->geo, ncap) == cudaSuccess;
    if (geometry && !d->s32)
        ok &= dalloc(&d->s32, ncap) == cudaSuccess;
    if (pool && !d->pool)
        ok &= dalloc(&d->pool, ncap) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        csgd_set_err(d, CSG_ERR_NOMEM);
        return CSG_ERR_NOMEM;
    }
    return CSG_OK;
}

// ---- forests ---------------------------------------------------------------

extern "C" int csgd_set_systems(csgd_t *d, int n_sys, const int *host_counts)
{
    if (n_sys < 1 || n_sys > CSG_MAX_SYSTEMS || (n_sys > 1 && !host_counts)) {
        return CSG_ERR_BAD_ARG;
    }
    long long total = 0;
    for (int g = 0; n_sys > 1 && g < n_sys; g++) {
        if (host_counts[g] < 0) {
            return CSG_ERR_BAD_ARG;
        }
        total += host_counts[g];
    }
    if (n_sys > 1 && total != d->n) {
        return CSG_ERR_BAD_ARG;
    }
    csgd_drop_graph(d); // grid shapes and the system pass change
    if (n_sys > d->gal_cap || (size_t)(d->cap / CSG_WARP) + n_sys + 2 > (size_t)d->task_cap) {
        cudaStreamSynchronize(d->stream);
        DevRoot *r = nullptr;
        WalkTask *t = nullptr;
        int *sn = nullptr;
        const size_t tcap = (size_t)(d->cap > 0 ? d->cap : 1) / CSG_WARP + (size_t)n_sys + 2;
        if (dalloc(&r, (size_t)n_sys) != cudaSuccess || dalloc(&t, tcap) != cudaSuccess ||
            dalloc(&sn, (size_t)n_sys) != cudaSuccess) {
            cudaGetLastError();
            if (r)
                cudaFree(r);
            if (t)
                cudaFree(t);
            csgd_set_err(d, CSG_ERR_NOMEM);
            return CSG_ERR_NOMEM;
        }
        cudaFree(d->roots);
        if (d->tasks)
            cudaFree(d->tasks);
        if (d->sys_n)
            cudaFree(d->sys_n);
        d->roots = r;
        d->tasks = t;
        d->sys_n = sn;
        d->gal_cap = n_sys;
        d->task_cap = (int)tcap;
    }
    d->n_gal = n_sys;
    d->geometry_valid = 0;
    d->gas_valid = 0;
    if (n_sys > 1) {
        d->sys_min_n = INT_MAX;
        d->sys_max_n = 0;
        for (int g = 0; g < n_sys; g++) {
            d->sys_min_n = host_counts[g] < d->sys_min_n ? host_counts[g] : d->sys_min_n;
            d->sys_max_n = host_counts[g] > d->sys_max_n ? host_counts[g] : d->sys_max_n;
        }
        cudaError_t e = cudaMemcpyAsync(d->sys_n, host_counts, sizeof(int) * (size_t)n_sys,
                                        cudaMemcpyHostToDevice, d->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(d->stream); // host_counts is the caller's
        if (e != cudaSuccess)
            return csgd_check(d, e);
    }
    if (d->n == 0 || !d->gid)
        return csgd_check(d, cudaGetLastError());
    if (n_sys == 1) {
        cudaMemsetAsync(d->gid, 0, sizeof(int) * (size_t)d->n, d->stream);
        return csgd_check(d, cudaGetLastError());
    }
    int *h = (int *)malloc(sizeof(int) * (size_t)d->n);
    if (!h) {
        csgd_set_err(d, CSG_ERR_NOMEM);
        return CSG_ERR_NOMEM;
    }
    for (int g = 0, i = 0; g < n_sys; g++)
        for (int k = 0; k < host_counts[g]; k++)
            h[i++] = g;
    cudaError_t e = cudaMemcpyAsync(d->gid, h, sizeof(int) * (size_t)d->n, cudaMemcpyHostToDevice,
                                    d->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(d->stream); // h is pageable and freed next
    free(h);
    return csgd_check(d, e);
}

extern "C" int csgd_system_count(const csgd_t *d) { return d->n_gal; }

// ---- host I/O --------------------------------------------------------------

extern "C" int csgd_unpack_aos(csgd_t *d)
{
    const int n = d->n;
    if (n <= 0)
        return CSG_OK;
    { k_unpack<<<csgd_grid(n, 256), 256, 0, d->stream>>>(d->aos, n, d->x, d->y, d->z, d->vx, d->vy,
                                                        d->vz, d->ax, d->ay, d->az, d->m, d->type,
                                                        d->rho, d->P, d->u, d->h); d->launches++; }
    d->geometry_valid = 0;
    d->gas_valid = 0;
    return csgd_check(d, cudaGetLastError());
}

extern "C" int csgd_upload_bodies(csgd_t *d, const Body *host, int n)
{
    int rc = csgd_reserve(d, n);
    if (rc)
        return rc;
    if (n == 0)
        return CSG_OK;
    cudaMemcpyAsync(d->aos, host, sizeof(Body) * (size_t)n, cudaMemcpyHostToDevice, d->stream);
    return csgd_unpack_aos(d);
}

extern "C" int csgd_pack_aos(csgd_t *d)
{
    const int n = d->n;
    if (n <= 0)
        return CSG_OK;
    { k_pack<<<csgd_grid(n, 256), 256, 0, d->stream>>>(d->aos, n, d->x, d->y, d->z, d->vx, d->vy,
                                                      d->vz, d->ax, d->ay, d->az, d->rho, d->P,
                                                      d->u, d->h, d->m, d->type); d->launches++; }
    return csgd_check(d, cudaGetLastError());
}

// Download into a mapped (pinned) host Body array: only the fields a step or
// an SPH pass can change (x..az at word 0, and with SPH density..smoothing_h
// at word 17 of the 21-word record) are written, straight from the SoA
// arrays; mass, type and the quasar fields of the caller's records stay as
// they are.
__global__ void k_download_direct(double *__restrict__ hb, int n, const double *__restrict__ x,
                                  const double *__restrict__ y, const double *__restrict__ z,
                                  const double *__restrict__ vx, const double *__restrict__ vy,
                                  const double *__restrict__ vz, const double *__restrict__ ax,
                                  const double *__restrict__ ay, const double *__restrict__ az,
                                  const double *__restrict__ rho, const double *__restrict__ P,
                                  const double *__restrict__ u, const double *__restrict__ h,
                                  int words)
{
    const long long total = (long long)words * n;
    for (long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x; f < total;
         f += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(f / words), j = (int)(f - (long long)words * i);
        const double *src[13] = {x, y, z, vx, vy, vz, ax, ay, az, rho, P, u, h};
        hb[21LL * i + (j < 9 ? j : j + 8)] = src[j][i];
    }
}

extern "C" int csgd_download_bodies(csgd_t *d, Body *host, int n)
{
    if (n > d->n || n < 0) {
        return CSG_ERR_BAD_ARG;
    }
    if (n == 0)
        return CSG_OK;

    int rc = csgd_pack_aos(d);
    if (rc)
        return rc;
    cudaMemcpyAsync(host, d->aos, sizeof(Body) * (size_t)n, cudaMemcpyDeviceToHost, d->stream);
    return csgd_check(d, cudaGetLastError());
}

extern "C" int csgd_download_step_fields(csgd_t *d, Body *host, int n, int sph)
{
    static_assert(sizeof(Body) == 168, "21 words per Body");
    double *hv = (double *)csgd_host_view(host);
    if (!hv || n <= 0 || n > d->n)
        return csgd_download_bodies(d, host, n);
    // without SPH a step leaves density..smoothing_h as they were
    const int words = sph ? 13 : 9;
    { k_download_direct<<<4 * d->num_sms, 256, 0, d->stream>>>(hv, n, d->x, d->y, d->z, d->vx, d->vy, d->vz, d->ax, d->ay, d->az, d->rho, d->P, d->u, d->h, words); d->launches++; }
    return csgd_check(d, cudaGetLastError());
}

// ---- leapfrog --------------------------------------------------------------

extern "C" int csgd_kick_drift(csgd_t *d, double dt)
{
    if (d->n <= 0)
        return CSG_OK;
    { k_kick_drift<<<csgd_grid(d->n, 256), 256, 0, d->stream>>>(d->n, dt, d->m, d->x, d->y, d->z,
                                                               d->vx, d->vy, d->vz, d->ax, d->ay,
                                                               d->az); d->launches++; }
    return csgd_check(d, cudaGetLastError());
}

extern "C" int csgd_kick(csgd_t *d, double dt)
{
    if (d->n <= 0)
        return CSG_OK;
    { k_kick<<<csgd_grid(d->n, 256), 256, 0, d->stream>>>(d->n, dt, d->m, d->vx, d->vy, d->vz,
                                                         d->ax, d->ay, d->az); d->launches++; }
    return csgd_check(d, cudaGetLastError());
}

extern "C" int csgd_sph_cooling(csgd_t *d, double dt)
{
    if (d->n <= 0)
        return CSG_OK;
    { k_cooling<<<csgd_grid(d->n, 256), 256, 0, d->stream>>>(d->n, dt, d->m, d->type, d->rho, d->u,
                                                            d->P); d->launches++; }
    return csgd_check(d, cudaGetLastError());
}

// With SPH, the gravity walk and the SPH passes up to the force terms are
// independent (the walk writes the accelerations; SPH writes density,
// pressure, smoothing lengths and its pair terms), so they run on two streams
// and the force sums, which add to the accelerations, wait for both. In a
// captured substep the fork and join become graph edges.
// Phase k of a substep starts: an NVTX range named for the phase (k = 6 only
// closes the last one) and, when timing, event tev[k] on the main stream.
static void phase_mark(csgd_t *d, int k)
{
    static const char *const names[6] = {"csg.kick_drift", "csg.build", "csg.gravity",
                                         "csg.sph", "csg.kick", "csg.cooling"};
    if (k > 0)
        nvtxRangePop();
    if (k < 6)
        nvtxRangePushA(names[k]);
    if (d->timing)
        cudaEventRecord(d->tev[k], d->stream);
}

extern "C" int csgd_substep(csgd_t *d, double dt, const csgd_force_params *p, int sph)
{
    // what a substep allocates on first use, before its first kernel: an
    // allocation failure then leaves the bodies as they were (no-ops inside a
    // capture, which allocates them beforehand)
    int rc = sph ? csgd_prepare_sph(d) : CSG_OK;
    if (!rc && d->export_dst)
        rc = csgd_ensure_tree_extras(d, 1, 1);
    if (!rc)
        rc = csgd_prepare_walk(d, p->precision);
    if (rc)
        return rc;
    phase_mark(d, 0);
    rc = csgd_kick_drift(d, dt);
    phase_mark(d, 1);
    if (!rc)
        rc = csgd_build_tree(d, sph);
    phase_mark(d, 2);
    // the pool export reads the finished tree only: it runs beside the walk
    bool exported = false;
    if (!rc && d->export_dst && d->aux2) {
        const cudaStream_t main = d->stream;
        cudaEventRecord(d->ev_fork2, main);
        cudaStreamWaitEvent(d->aux2, d->ev_fork2, 0);
        d->stream = d->aux2;
        rc = csgd_export_to(d, d->export_dst, d->export_cap);
        d->stream = main;
        cudaEventRecord(d->ev_join2, d->aux2);
        exported = true;
    }
    if (!rc && sph && d->aux && d->n_gal == 1) {
        const cudaStream_t main = d->stream;
        cudaEventRecord(d->ev_fork, main);
        cudaStreamWaitEvent(d->aux, d->ev_fork, 0);
        d->stream = d->aux;
        if (d->timing)
            cudaEventRecord(d->taux[0], d->aux);
        rc = csgd_sph_density(d);
        if (!rc)
            rc = csgd_sph_force_terms(d, 1);
        if (d->timing)
            cudaEventRecord(d->taux[1], d->aux);
        d->stream = main;
        cudaEventRecord(d->ev_join, d->aux);
        const int rg = csgd_gravity(d, p);
        phase_mark(d, 3); // the SPH sums on this stream count as SPH
        cudaStreamWaitEvent(main, d->ev_join, 0); // always rejoin (a capture needs it)
        if (d->timing)
            cudaEventRecord(d->taux[2], main);
        if (!rc)
            rc = rg;
        if (!rc)
            rc = csgd_sph_force_sums(d);
    } else {
        if (!rc)
            rc = csgd_gravity(d, p);
        phase_mark(d, 3);
        if (!rc && sph) {
            rc = csgd_sph_density(d);
            if (!rc)
                rc = csgd_sph_forces(d, 1);
        }
    }
    phase_mark(d, 4);
    if (!rc)
        rc = csgd_kick(d, dt);
    phase_mark(d, 5);
    if (!rc && sph)
        rc = csgd_sph_cooling(d, dt);
    if (exported)
        cudaStreamWaitEvent(d->stream, d->ev_join2, 0); // always rejoin (a capture needs it)
    phase_mark(d, 6);
    return rc;
}

int csgd_prepare_walk(csgd_t *d, int precision)
{
    const bool split = precision == CSG_PREC_FP32_MIXED ? csgd_walk_split(d)
                       : precision == CSG_PREC_FP64     ? csgd_sys_min_n(d) <= csgd_split_max_bodies(d)
                                                        : false;
    if (!split || (d->wpart && d->wpart_cap >= d->cap))
        return CSG_OK;
    csgd_drop_graph(d); // a captured walk holds the old pointer
    if (d->wpart) {
        cudaStreamSynchronize(d->stream);
        cudaFree(d->wpart);
    }
    d->wpart = nullptr;
    d->wpart_cap = 0;
    const size_t cap = (size_t)(d->cap > 0 ? d->cap : 1);
    if (csgd_malloc((void **)&d->wpart, sizeof(double) * 3 * 8 * cap) != cudaSuccess) {
        cudaGetLastError();
        d->wpart = nullptr;
        return CSG_ERR_NOMEM;
    }
    d->wpart_cap = (int)cap;
    return CSG_OK;
}

void csgd_build_mark(csgd_t *d, int k)
{
    if (d->timing && d->bev[k])
        cudaEventRecord(d->bev[k], d->stream);
}

// Adds the phase times of the substep just queued (waits for it). SPH that
// overlapped the walk on its own stream counts its own span plus the sums
// after the rejoin (the main stream's wait for it is in neither phase, only
// in the substep's total); the gravity phase is then the walk alone.
static int add_phase_times(csgd_t *d, int sph_overlapped)
{
    if (cudaEventSynchronize(d->tev[6]) != cudaSuccess)
        return csgd_check(d, cudaGetLastError());
    float t[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, whole = 0.f, aux = 0.f;
    for (int k = 0; k < 6; k++)
        if (cudaEventElapsedTime(&t[k], d->tev[k], d->tev[k + 1]) != cudaSuccess)
            return csgd_check(d, cudaGetLastError());
    if (cudaEventElapsedTime(&whole, d->tev[0], d->tev[6]) != cudaSuccess)
        return csgd_check(d, cudaGetLastError());
    if (sph_overlapped && (cudaEventElapsedTime(&aux, d->taux[0], d->taux[1]) != cudaSuccess ||
                           cudaEventElapsedTime(&t[3], d->taux[2], d->tev[4]) != cudaSuccess))
        return csgd_check(d, cudaGetLastError());
    for (int k = 0; k < 5; k++) {
        float b = 0.f;
        if (cudaEventElapsedTime(&b, d->bev[k], d->bev[k + 1]) != cudaSuccess)
            return csgd_check(d, cudaGetLastError());
        d->build_ms[k] += b;
    }
    for (int k = 0; k < 6; k++)
        d->phase_ms[k] += t[k];
    d->phase_ms[3] += aux;
    d->phase_ms[6] += whole;
    d->timed_substeps++;
    return CSG_OK;
}

extern "C" int csgd_set_phase_timing(csgd_t *d, int on)
{
    if (on && !d->tev[0]) {
        for (int k = 0; k < 7; k++)
            if (cudaEventCreate(&d->tev[k]) != cudaSuccess)
                return csgd_check(d, cudaGetLastError());
        for (int k = 0; k < 3; k++)
            if (cudaEventCreate(&d->taux[k]) != cudaSuccess)
                return csgd_check(d, cudaGetLastError());
        for (int k = 0; k < 6; k++)
            if (cudaEventCreate(&d->bev[k]) != cudaSuccess)
                return csgd_check(d, cudaGetLastError());
    }
    d->timing = on ? 1 : 0;
    if (on) { // a new measurement; turning it off keeps the sums for reading
        for (int k = 0; k < 5; k++)
            d->build_ms[k] = 0.0;
        for (int k = 0; k < 7; k++)
            d->phase_ms[k] = 0.0;
        d->timed_substeps = 0;
    }
    return CSG_OK;
}

extern "C" int csgd_phase_times(const csgd_t *d, double ms[12], long long *substeps)
{
    for (int k = 0; k < 7; k++)
        ms[k] = d->phase_ms[k];
    for (int k = 0; k < 5; k++)
        ms[7 + k] = d->build_ms[k];
    *substeps = d->timed_substeps;
    return CSG_OK;
}

// ---- synchronisation and queries ---------------------------------------

extern "C" int csgd_sync(csgd_t *d)
{
    cudaError_t e = cudaMemcpyAsync(d->sc_host, d->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost,
                                    d->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(d->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        d->host_err = 0;
        return CSG_ERR_CUDA;
    }
    int rc = d->host_err;
    d->host_err = 0;
    const int dev_err = d->sc_host->err;
    if (dev_err) {
        cudaMemsetAsync(&d->sc->err, 0, sizeof(int), d->stream);
        cudaStreamSynchronize(d->stream);
        if (!rc)
            rc = dev_err;
    }
    return rc;
}

extern "C" int csgd_set_substep_export(csgd_t *d, OctreeNode *dst, int capacity)
{
    // the export stages its records in the pool buffer (allocated here, never
    // inside a capture)
    const bool ok = dst && d->aux2 && d->export_order && d->n_gal == 1 &&
                    csgd_ensure_tree_extras(d, 1, 1) == CSG_OK;
    d->export_dst = ok ? dst : nullptr;
    d->export_cap = d->export_dst ? capacity : 0;
    return d->export_dst != nullptr;
}

extern "C" void *csgd_host_view(const void *p)
{
    cudaPointerAttributes a;
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost && a.devicePointer)
        return a.devicePointer;
    return nullptr;
}

extern "C" int csgd_node_count(csgd_t *d, int *n_nodes)
{
    int rc = csgd_sync(d);
    *n_nodes = d->sc_host->n_nodes;
    return rc;
}

extern "C" int csgd_interactions(csgd_t *d, int64_t *total)
{
    int rc = csgd_sync(d);
    *total = (int64_t)d->sc_host->interactions;
    return rc;
}

extern "C" int csgd_reset_stats(csgd_t *d)
{
    // interactions, walk_steps, walk_active are adjacent
    cudaMemsetAsync(&d->sc->interactions, 0, 3 * sizeof(unsigned long long), d->stream);
    return csgd_check(d, cudaGetLastError());
}

extern "C" int csgd_walk_stats(csgd_t *d, int64_t *interactions, int64_t *warp_steps,
                               int64_t *active_lane_steps)
{
    int rc = csgd_sync(d);
    *interactions = (int64_t)d->sc_host->interactions;
    *warp_steps = (int64_t)d->sc_host->walk_steps;
    *active_lane_steps = (int64_t)d->sc_host->walk_active;
    return rc;
}

extern "C" int csgd_alive_count(csgd_t *d, int *count)
{
    cudaMemsetAsync(&d->sc->alive_count, 0, sizeof(int), d->stream);
    if (d->n > 0) {
        int g = csgd_grid(d->n, 256);
        if (g > 152 * 8)
            g = 152 * 8;
        { k_alive_count<<<g, 256, 0, d->stream>>>(d->n, d->m, d->sc); d->launches++; }
    }
    int rc = csgd_sync(d);
    *count = d->sc_host->alive_count;
    return rc;
}

extern "C" unsigned long long csgd_launch_count(const csgd_t *d) { return d->launches; }

extern "C" void csgd_enable_graphs(csgd_t *d, int on) { d->use_graphs = on; }

static bool graph_matches(const csgd_t *d, double dt, const csgd_force_params *p, int sph)
{
    return d->graph && d->graph_key[0] == dt && d->graph_key[1] == p->G &&
           d->graph_key[2] == p->softening && d->graph_key[3] == p->theta &&
           d->graph_prec == p->precision && d->graph_sph == sph && d->graph_n == d->n &&
           d->graph_stream == d->stream && d->graph_export == d->export_dst &&
           d->graph_export_cap == d->export_cap;
}

// Captures one substep on the state's stream. Returns CSG_OK or an error (the
// caller then runs the substeps without a graph).
static int capture_substep(csgd_t *d, double dt, const csgd_force_params *p, int sph)
{
    if (d->graph) {
        cudaGraphExecDestroy(d->graph);
        d->graph = nullptr;
    }
    if (sph && csgd_prepare_sph(d))
        return CSG_ERR_NOMEM;
    if (d->export_dst && csgd_ensure_tree_extras(d, 1, 1))
        return CSG_ERR_NOMEM;
    if (csgd_prepare_walk(d, p->precision))
        return CSG_ERR_NOMEM;
    // host-side flags a substep resets anyway; start from the same state
    d->gas_valid = 0;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(d->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return CSG_ERR_CUDA;
    }
    const unsigned long long l0 = d->launches;
    int rc = csgd_substep(d, dt, p, sph);
    cudaError_t e = cudaStreamEndCapture(d->stream, &g);
    const unsigned long long per = d->launches - l0;
    d->launches = l0; // counted again on every replay
    if (rc || e != cudaSuccess || !g) {
        if (g)
            cudaGraphDestroy(g);
        cudaGetLastError();
        d->host_err = 0;
        return rc ? rc : CSG_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&d->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        cudaGetLastError();
        d->graph = nullptr;
        return CSG_ERR_CUDA;
    }
    d->graph_launches = per;
    d->graph_key[0] = dt;
    d->graph_key[1] = p->G;
    d->graph_key[2] = p->softening;
    d->graph_key[3] = p->theta;
    d->graph_prec = p->precision;
    d->graph_sph = sph;
    d->graph_n = d->n;
    d->graph_stream = d->stream;
    d->graph_export = d->export_dst;
    d->graph_export_cap = d->export_cap;
    return CSG_OK;
}

extern "C" int csgd_substeps(csgd_t *d, int k, double dt, const csgd_force_params *p, int sph)
{
    if (k <= 0)
        return CSG_OK;
    if (d->timing) { // direct launches, each substep's phase events read back
        const int overlapped = sph && d->aux && d->n_gal == 1;
        int rc = CSG_OK;
        for (int i = 0; i < k && !rc; i++) {
            rc = csgd_substep(d, dt, p, sph);
            if (!rc)
                rc = add_phase_times(d, overlapped);
        }
        return rc;
    }
    if (d->use_graphs && d->n > 0 && d->stream != nullptr && !graph_matches(d, dt, p, sph)) {
        const int crc = capture_substep(d, dt, p, sph);
        if (crc == CSG_ERR_NOMEM) // nothing ran; a later call captures again
            return crc;
        if (crc != CSG_OK)
            d->use_graphs = 0; // run without graphs from now on
    }
    if (d->use_graphs && d->graph) {
        for (int i = 0; i < k; i++) {
            if (cudaGraphLaunch(d->graph, d->stream) != cudaSuccess)
                return csgd_check(d, cudaGetLastError());
            d->launches += d->graph_launches;
        }
        d->gas_valid = 0;
        d->geometry_valid = sph ? 1 : 0;
        d->imported = 0;
        return CSG_OK;
    }
    int rc = CSG_OK;
    for (int i = 0; i < k && !rc; i++)
        rc = csgd_substep(d, dt, p, sph);
    return rc;
}
