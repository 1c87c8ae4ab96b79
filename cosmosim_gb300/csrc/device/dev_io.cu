// dev_io.cu — snapshot export of the alive bodies as packed float records,
// and stable compaction of dead bodies, both on the device.
//
// Snapshots follow the two consumers the reference feeds from the Body array:
// the Unreal plugin's 64-byte FCosmosimBodyGPU
// (ue/CosmosimPlugin/Source/CosmosimPlugin/Public/CosmosimSubsystem.h:15-27,
// filled by CosmosimSubsystem.cpp:12-43) and the renderer's 10-float vertex
// record (src/renderer.c:348-365): bodies whose mass is not <= 0, in index order,
// at most max_bodies of them, each field converted to float. Building the
// records on the device moves 40 or 64 bytes per alive body to the host
// instead of the 168-byte Body.
//
// Compaction keeps the alive bodies in their order (src/quasar.c:511-523).
#include "dev_internal.cuh"

namespace {

constexpr int IT = 256;

// Snapshots skip a body when mass <= 0.0 (a NaN mass is kept); compaction
// keeps a body when mass > 0.0 (a NaN mass is dropped), as the reference's
// two loops do.
template <bool COMPACT>
__global__ void k_keep_flags(int n, const double *__restrict__ m, int *__restrict__ flag)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        flag[i] = COMPACT ? (m[i] > 0.0 ? 1 : 0) : (m[i] <= 0.0 ? 0 : 1);
}

__global__ void k_snapshot(int format, int n, int max_out, const int *__restrict__ pos,
                           const double *__restrict__ m, const double *__restrict__ x,
                           const double *__restrict__ y, const double *__restrict__ z,
                           const double *__restrict__ vx, const double *__restrict__ vy,
                           const double *__restrict__ vz, const int *__restrict__ type,
                           const double *__restrict__ u, const double *__restrict__ rho,
                           const Body *__restrict__ aos, float *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || m[i] <= 0.0)
        return;
    const int k = pos[i];
    if (k >= max_out)
        return;
    if (format == CSG_SNAPSHOT_RENDER) {
        float *o = out + 10 * (size_t)k;
        o[0] = (float)x[i];
        o[1] = (float)y[i];
        o[2] = (float)z[i];
        o[3] = (float)m[i];
        o[4] = (float)vx[i];
        o[5] = (float)vy[i];
        o[6] = (float)vz[i];
        o[7] = (float)type[i];
        o[8] = (float)u[i];
        o[9] = (float)rho[i];
        return;
    }
    const Body &b = aos[i];
    float4 *o = (float4 *)(out + 16 * (size_t)k);
    o[0] = make_float4((float)x[i], (float)y[i], (float)z[i], (float)m[i]);
    o[1] = make_float4((float)vx[i], (float)vy[i], (float)vz[i], (float)type[i]);
    o[2] = make_float4((float)u[i], (float)rho[i], (float)b.lifetime, (float)b.luminosity);
    o[3] = make_float4((float)b.spin_x, (float)b.spin_y, (float)b.spin_z, 0.0f);
}

template <typename T>
__global__ void k_compact(int n, const int *__restrict__ keep, const int *__restrict__ pos,
                          const T *__restrict__ src, T *__restrict__ dst)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && keep[i])
        dst[pos[i]] = src[i];
}

} // namespace

extern "C" int csgd_snapshot_f32(csgd_t *d, int format, float *out, int out_is_device,
                                 int max_bodies, int *count_out)
{
    *count_out = 0;
    if ((format != CSG_SNAPSHOT_UE && format != CSG_SNAPSHOT_RENDER) || max_bodies < 0 ||
        (max_bodies > 0 && !out)) {
        return CSG_ERR_BAD_ARG;
    }
    const int n = d->n;
    if (n <= 0 || max_bodies == 0)
        return CSG_OK;
    cudaStream_t s = d->stream;
    const int stride = (format == CSG_SNAPSHOT_RENDER) ? 10 : 16;
    int *flag = d->cnt, *pos = d->base; // tree scratch: free between builds
    { k_keep_flags<false><<<csgd_grid(n, IT), IT, 0, s>>>(n, d->m, flag); d->launches++; }
    int rc = csg_scan_exclusive(d, flag, pos, n, nullptr);
    if (rc)
        return rc;
    cudaMemcpyAsync(d->h_int, pos + n, sizeof(int), cudaMemcpyDeviceToHost, s);
    rc = csgd_sync(d);
    const int total = *d->h_int;
    if (rc)
        return rc;
    const int k = total < max_bodies ? total : max_bodies;
    float *dst = out;
    float *tmp = nullptr;
    if (!out_is_device) {
        if (csgd_malloc((void **)&tmp, sizeof(float) * stride * (size_t)(k > 0 ? k : 1)) !=
            cudaSuccess) {
            cudaGetLastError();
            csgd_set_err(d, CSG_ERR_NOMEM);
            return CSG_ERR_NOMEM;
        }
        dst = tmp;
    }
    { k_snapshot<<<csgd_grid(n, IT), IT, 0, s>>>(format, n, k, pos, d->m, d->x, d->y, d->z, d->vx, d->vy, d->vz, d->type, d->u, d->rho, d->aos, dst); d->launches++; }
    if (!out_is_device && k > 0)
        cudaMemcpyAsync(out, tmp, sizeof(float) * stride * (size_t)k, cudaMemcpyDeviceToHost, s);
    rc = csgd_sync(d);
    if (tmp)
        cudaFree(tmp);
    if (!rc)
        *count_out = k;
    return rc;
}

extern "C" int csgd_compact(csgd_t *d, int *new_n)
{
    const int n = d->n;
    *new_n = n;
    if (d->n_gal > 1) { // the system layout would no longer match
        return CSG_ERR_UNSUPPORTED;
    }
    if (n <= 0)
        return CSG_OK;
    cudaStream_t s = d->stream;
    int *keep = d->cnt, *pos = d->base;
    { k_keep_flags<true><<<csgd_grid(n, IT), IT, 0, s>>>(n, d->m, keep); d->launches++; }
    int rc = csg_scan_exclusive(d, keep, pos, n, nullptr);
    if (rc)
        return rc;
    // the Body staging carries the fields the hot path does not keep in SoA
    rc = csgd_pack_aos(d);
    if (rc)
        return rc;
    void *tmp = nullptr;
    if (csgd_malloc(&tmp, sizeof(Body) * (size_t)n) != cudaSuccess) {
        cudaGetLastError();
        csgd_set_err(d, CSG_ERR_NOMEM);
        return CSG_ERR_NOMEM;
    }
    const int g = csgd_grid(n, IT);
    { k_compact<Body><<<g, IT, 0, s>>>(n, keep, pos, d->aos, (Body *)tmp); d->launches++; }
    cudaMemcpyAsync(d->aos, tmp, sizeof(Body) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    double *cols[] = {d->x, d->y, d->z, d->vx, d->vy, d->vz, d->ax, d->ay, d->az, d->m,
                      d->rho, d->P, d->u, d->h};
    for (double *c : cols) {
        { k_compact<double><<<g, IT, 0, s>>>(n, keep, pos, c, (double *)tmp); d->launches++; }
        cudaMemcpyAsync(c, tmp, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    }
    { k_compact<int><<<g, IT, 0, s>>>(n, keep, pos, d->type, (int *)tmp); d->launches++; }
    cudaMemcpyAsync(d->type, tmp, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(d->h_int, pos + n, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    const int kept = *d->h_int;
    cudaFree(tmp);
    if (e != cudaSuccess)
        return csgd_check(d, e);
    rc = csgd_sync(d);
    if (rc)
        return rc;
    d->n = kept;
    d->geometry_valid = 0;
    d->gas_valid = 0;
    *new_n = kept;
    return CSG_OK;
}
