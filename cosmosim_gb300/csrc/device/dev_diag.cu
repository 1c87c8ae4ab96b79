// dev_diag.cu — FP64 diagnostics and pipe-peak probes.
//
// Direct-sum accelerations of a body sample over all bodies of its system (the formula of
// the reference's test helper, tests/test_physics.c:54-71) and the total
// energy KE + softened PE (tests/test_physics.c:34-52), both in FP64. The
// j range is split over blocks; each block writes its partial sums and a
// second kernel adds them in a fixed order, so results are deterministic.
//
// The probes time long independent FMA chains (8 per thread) and report the
// FP32 and FP64 CUDA-core throughput of this GPU: the denominators for the
// walk kernels, which are bound by those pipes, not by tensor cores or HBM.
#include "dev_fpint.cuh"
#include "dev_internal.cuh"

namespace {

constexpr int DT = 256;       // threads per block
constexpr int JCHUNKS = 64;   // j-range splits for the direct sum

__global__ void __launch_bounds__(DT) k_direct(const double *__restrict__ x,
                                               const double *__restrict__ y,
                                               const double *__restrict__ z,
                                               const double *__restrict__ m,
                                               const int *__restrict__ gid, int n,
                                               const int *__restrict__ idx, int ns, double G,
                                               double eps2, double *__restrict__ part)
{
    __shared__ double sx[DT], sy[DT], sz[DT], sm[DT];
    __shared__ int sg[DT];
    const int k = blockIdx.x * DT + threadIdx.x;
    const int chunk = blockIdx.y;
    const int per = (n + JCHUNKS - 1) / JCHUNKS;
    const int j0 = chunk * per, j1 = min(n, j0 + per);
    const int i = (k < ns) ? idx[k] : -1;
    const double xi = (i >= 0) ? x[i] : 0.0, yi = (i >= 0) ? y[i] : 0.0, zi = (i >= 0) ? z[i] : 0.0;
    const int gi = (i >= 0) ? gid[i] : -1; // only bodies of the same system attract
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int t = j0; t < j1; t += DT) {
        const int j = t + threadIdx.x;
        __syncthreads();
        if (j < j1) {
            sx[threadIdx.x] = x[j];
            sy[threadIdx.x] = y[j];
            sz[threadIdx.x] = z[j];
            sm[threadIdx.x] = (m[j] <= 0.0) ? 0.0 : m[j];
            sg[threadIdx.x] = gid[j];
        }
        __syncthreads();
        const int cnt = min(DT, j1 - t);
        if (i >= 0) {
            for (int q = 0; q < cnt; q++) {
                if (t + q == i || sg[q] != gi)
                    continue;
                double dx = sx[q] - xi, dy = sy[q] - yi, dz = sz[q] - zi;
                double r2 = dx * dx + dy * dy + dz * dz + eps2;
                double inv = 1.0 / (r2 * sqrt(r2));
                double f = G * sm[q] * inv;
                ax += f * dx;
                ay += f * dy;
                az += f * dz;
            }
        }
    }
    if (k < ns) {
        double *p = part + ((size_t)chunk * ns + k) * 3;
        p[0] = ax;
        p[1] = ay;
        p[2] = az;
    }
}

__global__ void k_direct_sum(const double *__restrict__ part, int ns, double *__restrict__ out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ns)
        return;
    double a[3] = {0.0, 0.0, 0.0};
    for (int c = 0; c < JCHUNKS; c++)
        for (int d = 0; d < 3; d++)
            a[d] += part[((size_t)c * ns + k) * 3 + d];
    for (int d = 0; d < 3; d++)
        out[3 * (size_t)k + d] = a[d];
}

// 1/r in FP64 with few FP64 operations: FP32 rsqrt seed y0 (rel. error
// < 2^-21), e = 1 - r2*y0^2 by one fused multiply-add (y0^2 exact), then
// y0 (1 + e/2 + 3e^2/8) (the series of (1-e)^-1/2; the next term is < 2^-60).
__device__ __forceinline__ double inv_r(double r2)
{
    const float r2f = (float)r2;
    if (r2f >= 1e-30f && r2f <= 1e30f) {
        const double y0 = (double)rsqrtf(r2f);
        const double e = fma(-r2, y0 * y0, 1.0);
        return fma(y0 * e, fma(0.375, e, 0.5), y0);
    }
    return 1.0 / sqrt(r2);
}

// Potential energy: row i against columns j > i, rows split over blocks;
// each thread writes its row sum, reduced afterwards.
__global__ void __launch_bounds__(DT) k_potential_rows(const double *__restrict__ x,
                                                       const double *__restrict__ y,
                                                       const double *__restrict__ z,
                                                       const double *__restrict__ m,
                                                       const int *__restrict__ gid, int n,
                                                       double G, double eps2,
                                                       double *__restrict__ row)
{
    __shared__ double sx[DT], sy[DT], sz[DT], sm[DT];
    __shared__ int sg[DT];
    const int i = blockIdx.x * DT + threadIdx.x;
    const double xi = (i < n) ? x[i] : 0.0, yi = (i < n) ? y[i] : 0.0, zi = (i < n) ? z[i] : 0.0;
    const int gi = (i < n) ? gid[i] : -1;
    const double mi = (i < n && m[i] > 0.0) ? m[i] : 0.0;
    double pe = 0.0;
    const int jstart = blockIdx.x * DT; // columns from the block's first row
    for (int t = jstart; t < n; t += DT) {
        const int j = t + threadIdx.x;
        __syncthreads();
        if (j < n) {
            sx[threadIdx.x] = x[j];
            sy[threadIdx.x] = y[j];
            sz[threadIdx.x] = z[j];
            sm[threadIdx.x] = (m[j] > 0.0) ? m[j] : 0.0;
            sg[threadIdx.x] = gid[j];
        }
        __syncthreads();
        const int cnt = min(DT, n - t);
        if (i < n) {
            for (int q = 0; q < cnt; q++) {
                if (t + q <= i || sg[q] != gi)
                    continue;
                const double dx = sx[q] - xi, dy = sy[q] - yi, dz = sz[q] - zi;
                const double r2 = fma(dx, dx, fma(dy, dy, fma(dz, dz, eps2)));
                pe = fma(-sm[q], inv_r(r2), pe);
            }
        }
    }
    if (i < n)
        row[i] = G * mi * pe;
}

__global__ void k_energy_reduce(const double *__restrict__ row, const double *__restrict__ m,
                                const double *__restrict__ vx, const double *__restrict__ vy,
                                const double *__restrict__ vz, int n, double *__restrict__ out)
{
    // one block; fixed-order tree reduction in shared memory
    __shared__ double ske[1024], spe[1024];
    double ke = 0.0, pe = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double mm = (m[i] > 0.0) ? m[i] : 0.0;
        ke += 0.5 * mm * (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]);
        pe += row[i];
    }
    ske[threadIdx.x] = ke;
    spe[threadIdx.x] = pe;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            ske[threadIdx.x] += ske[threadIdx.x + s];
            spe[threadIdx.x] += spe[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = ske[0];
        out[1] = spe[0];
    }
}

template <typename T>
__global__ void k_fma_probe(T *out, int iters, T a, T b)
{
    T x0 = (T)threadIdx.x * (T)1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    T x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
        x0 = x0 * a + b;
        x1 = x1 * a + b;
        x2 = x2 * a + b;
        x3 = x3 * a + b;
        x4 = x4 * a + b;
        x5 = x5 * a + b;
        x6 = x6 * a + b;
        x7 = x7 * a + b;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

} // namespace

extern "C" int csgd_direct_forces(csgd_t *d, const int *host_idx, int ns, double G,
                                  double softening, double *host_out)
{
    if (ns <= 0)
        return CSG_OK;
    if (ns > d->n || !host_idx)
        return CSG_ERR_BAD_ARG;
    for (int k = 0; k < ns; k++)
        if (host_idx[k] < 0 || host_idx[k] >= d->n)
            return CSG_ERR_BAD_ARG;
    int *didx = nullptr;
    double *part = nullptr, *out = nullptr;
    cudaError_t e = csgd_malloc((void **)&didx, sizeof(int) * (size_t)ns);
    if (e == cudaSuccess)
        e = csgd_malloc((void **)&part, sizeof(double) * 3 * (size_t)ns * JCHUNKS);
    if (e == cudaSuccess)
        e = csgd_malloc((void **)&out, sizeof(double) * 3 * (size_t)ns);
    int rc = CSG_OK;
    if (e == cudaSuccess) {
        cudaMemcpyAsync(didx, host_idx, sizeof(int) * (size_t)ns, cudaMemcpyHostToDevice, d->stream);
        dim3 grid((ns + DT - 1) / DT, JCHUNKS);
        { k_direct<<<grid, DT, 0, d->stream>>>(d->x, d->y, d->z, d->m, d->gid, d->n, didx, ns, G, softening * softening, part); d->launches++; }
        { k_direct_sum<<<csgd_grid(ns, 256), 256, 0, d->stream>>>(part, ns, out); d->launches++; }
        cudaMemcpyAsync(host_out, out, sizeof(double) * 3 * (size_t)ns, cudaMemcpyDeviceToHost, d->stream);
        rc = csgd_sync(d);
    } else {
        cudaGetLastError();
        rc = CSG_ERR_NOMEM;
    }
    cudaFree(didx);
    cudaFree(part);
    cudaFree(out);
    return rc;
}

extern "C" int csgd_energy(csgd_t *d, double G, double softening, double *ke, double *pe)
{
    const int n = d->n;
    double *row = nullptr, *out = nullptr;
    cudaError_t e = csgd_malloc((void **)&row, sizeof(double) * (size_t)(n > 0 ? n : 1));
    if (e == cudaSuccess)
        e = csgd_malloc((void **)&out, 2 * sizeof(double));
    int rc = CSG_OK;
    if (e == cudaSuccess && n > 0) {
        { k_potential_rows<<<csgd_grid(n, DT), DT, 0, d->stream>>>(d->x, d->y, d->z, d->m, d->gid, n, G, softening * softening, row); d->launches++; }
        { k_energy_reduce<<<1, 1024, 0, d->stream>>>(row, d->m, d->vx, d->vy, d->vz, n, out); d->launches++; }
        double h[2] = {0.0, 0.0};
        cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, d->stream);
        rc = csgd_sync(d);
        *ke = h[0];
        *pe = h[1];
    } else if (e != cudaSuccess) {
        cudaGetLastError();
        rc = CSG_ERR_NOMEM;
    } else {
        *ke = *pe = 0.0;
    }
    cudaFree(row);
    cudaFree(out);
    return rc;
}

// FP32 and FP64 FMA throughput (TFLOP/s, 2 flop per FMA) of the current device.
extern "C" CSG_EXPORT int csg_measure_fp_peaks(double *fp32_tflops, double *fp64_tflops)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return CSG_ERR_NO_DEVICE;
    }
    const int blocks = sms * 8, threads = 256;
    const size_t nthr = (size_t)blocks * threads;
    float *o32 = nullptr;
    double *o64 = nullptr;
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
        return CSG_ERR_CUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc = CSG_OK;
    if (csgd_malloc((void **)&o32, nthr * sizeof(float)) != cudaSuccess ||
        csgd_malloc((void **)&o64, nthr * sizeof(double)) != cudaSuccess) {
        rc = CSG_ERR_NOMEM;
    } else {
        const int it32 = 8192, it64 = 512;
        float best32 = 1e30f, best64 = 1e30f, ms = 0.f;
        for (int rep = 0; rep < 3; rep++) {
            cudaEventRecord(e0, s);
            k_fma_probe<float><<<blocks, threads, 0, s>>>(o32, it32, 0.999999f, 1e-7f);
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            cudaEventElapsedTime(&ms, e0, e1);
            best32 = ms < best32 ? ms : best32;
            cudaEventRecord(e0, s);
            k_fma_probe<double><<<blocks, threads, 0, s>>>(o64, it64, 0.999999, 1e-7);
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            cudaEventElapsedTime(&ms, e0, e1);
            best64 = ms < best64 ? ms : best64;
        }
        *fp32_tflops = 2.0 * 8.0 * it32 * (double)nthr / (best32 * 1e-3) / 1e12;
        *fp64_tflops = 2.0 * 8.0 * it64 * (double)nthr / (best64 * 1e-3) / 1e12;
        if (cudaGetLastError() != cudaSuccess)
            rc = CSG_ERR_CUDA;
    }
    cudaFree(o32);
    cudaFree(o64);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    return rc;
}

// ---- direct sum without allocation -----------------------------------------
//
// Callers that cannot allocate device memory — code inside an engine or
// renderer that owns a fixed GPU budget and its own allocator, a real-time
// thread that must not block on cudaMalloc/cudaFree (both can synchronise the
// device) — can still run the FP64 direct-sum check on buffers they already
// hold. Its scratch (per-chunk partial sums) lives in the file-scope array
// below instead of cudaMalloc'd memory: 16 chunks x 4096 bodies x 3 doubles =
// 1.5 MiB, held by every GPU that loads the library until the process exits.
// All calls share that array, so calls that overlap on the GPU race; every
// call overwrites each partial it later reads, so nothing needs clearing.

constexpr int NOALLOC_CHUNKS = 16;
constexpr int NOALLOC_MAX_SAMPLE = 4096;
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) double g_noalloc_partials[NOALLOC_CHUNKS * NOALLOC_MAX_SAMPLE * 3];

#include <mutex>

namespace {

std::mutex g_noalloc_mutex;
double *g_noalloc_ptr[NOALLOC_MAX_DEVICES];

__global__ void __launch_bounds__(DT) k_direct_noalloc(const double *__restrict__ x,
                                                       const double *__restrict__ y,
                                                       const double *__restrict__ z,
                                                       const double *__restrict__ m,
                                                       const int *__restrict__ sys, int n,
                                                       const int *__restrict__ idx, int ns,
                                                       double G, double eps2,
                                                       double *__restrict__ part)
{
    __shared__ double sx[DT], sy[DT], sz[DT], sm[DT];
    __shared__ int sg[DT];
    const int k = blockIdx.x * DT + threadIdx.x;
    const int chunk = blockIdx.y;
    const int per = (n + NOALLOC_CHUNKS - 1) / NOALLOC_CHUNKS;
    const int j0 = chunk * per, j1 = min(n, j0 + per);
    // A sample index outside [0, n) reads nothing: its row becomes NaN.
    const int i = (k < ns) ? idx[k] : -1;
    const bool valid = (unsigned)i < (unsigned)n;
    const double xi = valid ? x[i] : 0.0, yi = valid ? y[i] : 0.0, zi = valid ? z[i] : 0.0;
    const int gi = (valid && sys) ? sys[i] : 0; // only bodies of the same system attract
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int t = j0; t < j1; t += DT) {
        const int j = t + threadIdx.x;
        __syncthreads();
        if (j < j1) {
            sx[threadIdx.x] = x[j];
            sy[threadIdx.x] = y[j];
            sz[threadIdx.x] = z[j];
            sm[threadIdx.x] = (m[j] <= 0.0) ? 0.0 : m[j];
            sg[threadIdx.x] = sys ? sys[j] : 0;
        }
        __syncthreads();
        const int cnt = min(DT, j1 - t);
        if (valid) {
            for (int q = 0; q < cnt; q++) {
                if (t + q == i || sg[q] != gi)
                    continue;
                double dx = sx[q] - xi, dy = sy[q] - yi, dz = sz[q] - zi;
                double r2 = dx * dx + dy * dy + dz * dz + eps2;
                double inv = 1.0 / (r2 * sqrt(r2));
                double f = G * sm[q] * inv;
                ax += f * dx;
                ay += f * dy;
                az += f * dz;
            }
        }
    }
    if (k < ns) {
        if (!valid)
            ax = ay = az = __longlong_as_double(0x7ff8000000000000ll);
        double *p = part + ((size_t)chunk * ns + k) * 3;
        p[0] = ax;
        p[1] = ay;
        p[2] = az;
    }
}

__global__ void k_direct_noalloc_sum(const double *__restrict__ part, int ns,
                                     double *__restrict__ out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ns)
        return;
    double a[3] = {0.0, 0.0, 0.0};
    for (int c = 0; c < NOALLOC_CHUNKS; c++)
        for (int d = 0; d < 3; d++)
            a[d] += part[((size_t)c * ns + k) * 3 + d];
    for (int d = 0; d < 3; d++)
        out[3 * (size_t)k + d] = a[d];
}

} // namespace

// The device address of the scratch array on the current device, looked up
// once per device (the first call on a device does it, so that call should
// come before any stream capture on that device). The address belongs to the
// device's primary context: after a cudaDeviceReset the cached address is
// stale, so a process that resets a device must not call the entry point on
// it again.
static int noalloc_scratch(double **ptr)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        cudaGetLastError();
        return CSG_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_partials) != cudaSuccess || !p) {
            cudaGetLastError();
            return CSG_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = (double *)p;
    }
    *ptr = g_noalloc_ptr[dev];
    return CSG_OK;
}

extern "C" CSG_EXPORT int csg_direct_forces_noalloc(const double *x, const double *y,
                                                    const double *z, const double *mass,
                                                    const int *sys, int n, const int *idx, int m,
                                                    double G, double softening, double *out,
                                                    void *stream)
{
    if (n < 0 || m < 0 || m > NOALLOC_MAX_SAMPLE)
        return CSG_ERR_BAD_ARG;
    if (m == 0)
        return CSG_OK;
    if (!x || !y || !z || !mass || !idx || !out || n == 0)
        return CSG_ERR_BAD_ARG;
    double *part = nullptr;
    int rc = noalloc_scratch(&part);
    if (rc)
        return rc;
    cudaStream_t s = (cudaStream_t)stream;
    dim3 grid((m + DT - 1) / DT, NOALLOC_CHUNKS);
    k_direct_noalloc<<<grid, DT, 0, s>>>(x, y, z, mass, sys, n, idx, m, G, softening * softening, part);
    k_direct_noalloc_sum<<<(m + 255) / 256, 256, 0, s>>>(part, m, out);
    if (cudaGetLastError() != cudaSuccess)
        return CSG_ERR_CUDA;
    return CSG_OK;
}

// ---- integer-pipe division and square root: self-check ----------------------
//
// div_rn and sqrt_rn (dev_fpint.cuh) against the compiler's correctly rounded
// operators, bit for bit, on n seeded operand pairs of several kinds: operands
// of moderate exponents, arbitrary bit patterns (zeros, subnormals,
// infinities, NaNs, exponents near the fast path's bounds), integer operands
// over small odd divisors (exact quotients and ties), power-of-two divisors,
// signed zeros and SPH-like distances and smoothing lengths.

namespace {

__device__ __forceinline__ unsigned long long xs_next(unsigned long long &s)
{
    s ^= s << 13;
    s ^= s >> 7;
    s ^= s << 17;
    return s;
}

__device__ __forceinline__ double rand_moderate(unsigned long long &s, int span)
{
    const unsigned long long r = xs_next(s);
    const long long e = 1023 + (long long)(r % (unsigned long long)(2 * span + 1)) - span;
    return __longlong_as_double((long long)((r & (1ull << 63)) | ((unsigned long long)e << 52) |
                                            (xs_next(s) & fpint::MANT)));
}

__global__ void k_check_div_sqrt(unsigned long long seed, long long n, unsigned long long *out)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    unsigned long long bad_div = 0, bad_sqrt = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        unsigned long long s = (seed ^ ((unsigned long long)i * 0x9E3779B97F4A7C15ull)) | 1ull;
        xs_next(s);
        xs_next(s);
        double a, b;
        switch ((unsigned)(xs_next(s) % 8)) {
        case 0:
        case 1:
            a = rand_moderate(s, 60);
            b = rand_moderate(s, 60);
            break;
        case 2:
            a = __longlong_as_double((long long)xs_next(s));
            b = __longlong_as_double((long long)xs_next(s));
            break;
        case 3: {
            const unsigned sh = 11 + (unsigned)(xs_next(s) % 40);
            a = (double)(long long)(xs_next(s) >> sh);
            const double odd[6] = {3.0, 5.0, 7.0, 9.0, 11.0, 1.0 + (double)(xs_next(s) & 255) * 2.0};
            b = odd[xs_next(s) % 6] * ((xs_next(s) & 1) ? 1.0 : -1.0);
            break;
        }
        case 4:
            a = rand_moderate(s, 500);
            b = __longlong_as_double((long long)((unsigned long long)(1023 + (long long)(xs_next(s) % 1001) - 500)
                                                 << 52));
            break;
        case 5:
            a = (xs_next(s) & 1) ? 0.0 : -0.0;
            b = rand_moderate(s, 1000);
            break;
        case 6: // exponents near the fast path's limits
            a = rand_moderate(s, 1022);
            b = rand_moderate(s, 1022);
            break;
        default: { // distances, smoothing lengths, densities of the SPH passes
            const double r = (double)(xs_next(s) >> 11) * 0x1p-53 * 4.0;
            const double h = 0.01 + (double)(xs_next(s) >> 11) * 0x1p-53;
            a = (xs_next(s) & 1) ? r * r : r;
            b = (xs_next(s) & 1) ? h : h * h * h * 3.141592653589793;
            break;
        }
        }
        if (__double_as_longlong(div_rn(a, b)) != __double_as_longlong(__ddiv_rn(a, b)))
            bad_div++;
        const double x = (xs_next(s) & 3) ? fabs(a) : a;
        if (__double_as_longlong(sqrt_rn(x)) != __double_as_longlong(__dsqrt_rn(x)))
            bad_sqrt++;
    }
    if (bad_div)
        atomicAdd(&out[0], bad_div);
    if (bad_sqrt)
        atomicAdd(&out[1], bad_sqrt);
}

} // namespace

extern "C" CSG_EXPORT int csg_check_div_sqrt(int64_t n, uint64_t seed, int64_t *div_mismatches,
                                             int64_t *sqrt_mismatches)
{
    if (n < 0 || !div_mismatches || !sqrt_mismatches)
        return CSG_ERR_BAD_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return CSG_ERR_NO_DEVICE;
    }
    unsigned long long *out = nullptr;
    if (csgd_malloc((void **)&out, 2 * sizeof(unsigned long long)) != cudaSuccess) {
        cudaGetLastError();
        return CSG_ERR_NOMEM;
    }
    unsigned long long h[2] = {0, 0};
    int rc = CSG_OK;
    if (cudaMemset(out, 0, sizeof(h)) != cudaSuccess)
        rc = CSG_ERR_CUDA;
    if (!rc && n > 0) {
        k_check_div_sqrt<<<sms * 8, 256>>>((unsigned long long)seed, (long long)n, out);
        if (cudaGetLastError() != cudaSuccess)
            rc = CSG_ERR_CUDA;
    }
    if (!rc && cudaMemcpy(h, out, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = CSG_ERR_CUDA;
    cudaFree(out);
    *div_mismatches = (int64_t)h[0];
    *sqrt_mismatches = (int64_t)h[1];
    return rc;
}
