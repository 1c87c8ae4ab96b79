// dev_ics.cu — exponential-disk initial conditions on the device.
//
// The host generator (csrc/host/ics.c, the recipe of the reference's
// src/initial_conditions.c:40-112 with the benchmark parameters) draws 10
// uniforms per disk body from one seeded xorshift64 stream (Marsaglia,
// shifts 13/7/17). That generator is linear over GF(2): one step is a 64x64
// bit matrix M, so the state before any draw k is M^k s0. Each thread jumps
// to its run of 16 bodies with the precomputed powers M^(2^b) and then draws
// sequentially, so every body gets exactly the host's random numbers; the
// arithmetic repeats the host's operation order (compiled without fused
// multiply-add). log, exp, sin, cos and sqrt are CUDA's: positions and
// velocities agree with the host's to a few ulp.
#include "dev_internal.cuh"

#include <mutex>

namespace {

constexpr int RUN = 16;         // bodies per thread
constexpr double IPI = 3.14159265358979323846;

unsigned long long xs_step(unsigned long long x)
{
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    return x;
}

struct Gen {
    unsigned long long s;
    __device__ double uniform()
    {
        unsigned long long x = s;
        x ^= x << 13;
        x ^= x >> 7;
        x ^= x << 17;
        s = x;
        return (double)(x >> 11) * (1.0 / 9007199254740992.0);
    }
    __device__ double normal()
    {
        double u1 = uniform();
        double u2 = uniform();
        if (u1 < 1e-15)
            u1 = 1e-15;
        return sqrt(-2.0 * log(u1)) * cos(2.0 * IPI * u2);
    }
};

__device__ double plummer_menc(double m, double a, double r)
{
    if (m <= 0.0)
        return 0.0;
    return m * r * r * r / pow(r * r + a * a, 1.5);
}

// chunk c -> (system, first body of the run)
__global__ void k_disks(const csgd_disk_plan *__restrict__ plans, const int *__restrict__ counts,
                        const int *__restrict__ body_off, const int *__restrict__ chunk_off,
                        int n_sys, const XsJumpTable *__restrict__ jt, Body *__restrict__ out)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= chunk_off[n_sys])
        return;
    int g = 0;
    while (g + 1 < n_sys && chunk_off[g + 1] <= c) // few systems: linear is fine
        g++;
    const csgd_disk_plan p = plans[g];
    const int n = counts[g];
    const int first = (p.smbh > 0.0 && n > 0) ? 1 : 0;
    const int i0 = (c - chunk_off[g]) * RUN; // body index within the system
    Body *o = out + body_off[g];
    const int nd = n - first;
    const double mi = nd > 0 ? p.mass / nd : 0.0;
    const double rmax = 4.0 * p.rd;
    const double spacing = rmax / sqrt((double)(n > 0 ? n : 1));
    // state before the run's first draw: M^(10 (i - first)) s0
    int i = i0;
    if (i < first) {
        Body &b = o[0];
        b = Body{};
        b.mass = p.smbh;
        b.type = BODY_SMBH;
        i = first;
    }
    Gen r{p.seed ? p.seed : 1ull};
    r.s = xs_jump(jt, r.s, 10ull * (unsigned long long)(i - first));
    for (; i < i0 + RUN && i < n; i++) {
        Body &b = o[i];
        b = Body{};
        double u = r.uniform();
        if (u < 1e-15)
            u = 1e-15;
        double rad = -p.rd * log(1.0 - u * (1.0 - exp(-rmax / p.rd)));
        double th0 = 2.0 * IPI * r.uniform();
        double arm = log(rad / p.rd + 0.1) / 0.27;
        double th = th0 + 0.35 * exp(-rad / (rmax * 0.8)) * sin(2.0 * (th0 - arm));
        b.x = rad * cos(th);
        b.y = rad * sin(th);
        b.z = r.normal() * p.zh;
        b.mass = mi;
        double x = rad / p.rd;
        double menc = p.mass * (1.0 - exp(-x) * (1.0 + x)) + p.smbh +
                      plummer_menc(p.bulge_mass, p.bulge_a, rad);
        if (rad < 1e-10)
            rad = 1e-10;
        double vc = sqrt(menc / rad);
        double disp = 0.05 * vc;
        double vt = vc + r.normal() * disp;
        double vr = r.normal() * disp;
        b.vx = -vt * sin(th) + vr * cos(th);
        b.vy = vt * cos(th) + vr * sin(th);
        b.vz = r.normal() * disp * 0.1;
        if (u < p.gas_frac) {
            b.type = BODY_GAS;
            double mg = p.mass * (1.0 - exp(-x));
            double vloc = sqrt(mg / rad);
            b.internal_energy = 0.5 * vloc * vloc / (CSG_SPH_GAMMA - 1.0);
            b.smoothing_h = spacing * 2.0;
        }
    }
}

} // namespace

// Runs start below 10 * 2^36 draws; the quasar step's offsets are far smaller.
const XsJumpTable &xs_jump_table_host()
{
    static XsJumpTable t;
    static std::once_flag once;
    std::call_once(once, [] {
        for (int j = 0; j < 64; j++)
            t.col[0][j] = xs_step(1ull << j);
        for (int b = 1; b < XS_JUMP_LEVELS; b++)
            for (int j = 0; j < 64; j++) // M^(2^b) = M^(2^(b-1)) o M^(2^(b-1))
                t.col[b][j] = xs_apply(t.col[b - 1], t.col[b - 1][j]);
    });
    return t;
}

extern "C" int csgd_generate_disks(void *stream, const csgd_disk_plan *plans, const int *counts,
                                   int n_sys, Body *out)
{
    if (n_sys < 1 || !plans || !counts || !out)
        return CSG_ERR_BAD_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    // offsets of bodies and of runs
    const size_t words = 2 * ((size_t)n_sys + 1);
    int *h = (int *)malloc(sizeof(int) * words);
    if (!h)
        return CSG_ERR_NOMEM;
    int *boff = h, *coff = h + n_sys + 1;
    boff[0] = coff[0] = 0;
    for (int g = 0; g < n_sys; g++) {
        if (counts[g] < 0) {
            free(h);
            return CSG_ERR_BAD_ARG;
        }
        boff[g + 1] = boff[g] + counts[g];
        coff[g + 1] = coff[g] + (counts[g] + RUN - 1) / RUN;
    }
    const int chunks = coff[n_sys];
    void *dmem = nullptr;
    const size_t bytes = sizeof(XsJumpTable) + sizeof(csgd_disk_plan) * n_sys +
                         sizeof(int) * (words + n_sys);
    if (csgd_malloc(&dmem, bytes) != cudaSuccess) {
        cudaGetLastError();
        free(h);
        return CSG_ERR_NOMEM;
    }
    char *p = (char *)dmem;
    XsJumpTable *djt = (XsJumpTable *)p;
    csgd_disk_plan *dplans = (csgd_disk_plan *)(p + sizeof(XsJumpTable));
    int *dints = (int *)(p + sizeof(XsJumpTable) + sizeof(csgd_disk_plan) * n_sys);
    cudaMemcpyAsync(djt, &xs_jump_table_host(), sizeof(XsJumpTable), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dplans, plans, sizeof(csgd_disk_plan) * n_sys, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dints, counts, sizeof(int) * n_sys, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dints + n_sys, h, sizeof(int) * words, cudaMemcpyHostToDevice, s);
    if (chunks > 0)
        k_disks<<<(chunks + 127) / 128, 128, 0, s>>>(dplans, dints, dints + n_sys,
                                                     dints + n_sys + (n_sys + 1), n_sys, djt, out);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s); // h and the scratch are freed next
    cudaFree(dmem);
    free(h);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return CSG_ERR_CUDA;
    }
    return CSG_OK;
}

extern "C" int csgd_upload_device_bodies(csgd_t *d, const Body *device_bodies, int n)
{
    int rc = csgd_reserve(d, n);
    if (rc || n == 0)
        return rc;
    cudaMemcpyAsync(d->aos, device_bodies, sizeof(Body) * (size_t)n, cudaMemcpyDeviceToDevice,
                    d->stream);
    return csgd_unpack_aos(d);
}
