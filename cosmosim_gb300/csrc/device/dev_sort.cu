// dev_sort.cu — exclusive scan and stable LSD radix sort used by the tree build.
//
// Radix sort: 8-bit digits, three kernels per digit (tile histogram, scan of
// the digit-major histogram, stable scatter); tiles of 1024 keys below 2M keys,
// 4096 above. Stability inside a tile comes
// from giving each warp a contiguous slice of the tile and ranking equal
// digits with __match_any_sync in input order; across tiles from the
// digit-major exclusive scan. Stability matters: keys that tie keep caller
// index order, which the tree build relies on (reference inserts bodies in
// index order, src/octree.c:163-168).
#include "dev_internal.cuh"

namespace {

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

constexpr int SORT_THREADS = 256;
constexpr int SORT_WARPS = SORT_THREADS / CSG_WARP;
// Items per lane: 16 (tiles of 4096 keys) for large sorts, 4 (tiles of 1024)
// below 2M keys, so that a 100k-key sort still spreads over ~100 blocks.
constexpr int sort_tile(int ipl) { return SORT_WARPS * CSG_WARP * ipl; }
constexpr int RADIX = 256;

__device__ __forceinline__ int warp_incl_scan(int v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o)
            v += t;
    }
    return v;
}

// Exclusive scan of one 4096-item tile; writes the tile total to sums[block].
__global__ void k_scan_tile(const int *__restrict__ in, int *__restrict__ out, int n,
                            const int *__restrict__ limit, int *__restrict__ sums)
{
    __shared__ int warp_tot[SCAN_THREADS / 32];
    const int lim = limit ? min(n, *limit) : n;
    const long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int local = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        long long i = base + k;
        v[k] = (i < lim) ? in[i] : 0;
        local += v[k];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = warp_incl_scan(local);
    if (lane == 31)
        warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int t = warp_tot[lane];
        int ti = warp_incl_scan(t);
        warp_tot[lane] = ti - t;
    }
    __syncthreads();
    int run = warp_tot[warp] + incl - local;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        long long i = base + k;
        if (i < n)
            out[i] = run;
        run += v[k];
    }
    if (threadIdx.x == SCAN_THREADS - 1)
        sums[blockIdx.x] = run;
}

// Exclusive scan of up to SCAN_SMALL items by one block, which walks the input
// in 4096-item tiles (each warp reads 128 consecutive items) and carries the
// running total from tile to tile. One launch instead of the
// tile/recursion/add/total sequence for the small scans a substep does;
// writes out[n] = total.
constexpr int SCAN_SMALL = 16 * SCAN_TILE;

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_small(const int *__restrict__ in,
                                                             int *__restrict__ out, int n,
                                                             const int *__restrict__ limit)
{
    __shared__ int warp_tot[SCAN_THREADS / 32];
    __shared__ int tile_tot;
    const int lim = limit ? min(n, *limit) : n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int carry = 0;
    for (int t0 = 0; t0 < n; t0 += SCAN_TILE) {
        const int base = t0 + threadIdx.x * SCAN_ITEMS;
        int v[SCAN_ITEMS];
        int local = 0;
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; k++) {
            const int i = base + k;
            v[k] = (i < lim) ? in[i] : 0;
            local += v[k];
        }
        const int incl = warp_incl_scan(local);
        if (lane == 31)
            warp_tot[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            const int t = warp_tot[lane];
            const int ti = warp_incl_scan(t);
            warp_tot[lane] = ti - t;
            if (lane == 31)
                tile_tot = ti;
        }
        __syncthreads();
        int run = carry + warp_tot[warp] + incl - local;
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; k++) {
            const int i = base + k;
            if (i < n)
                out[i] = run;
            run += v[k];
        }
        carry += tile_tot;
        __syncthreads(); // warp_tot and tile_tot are rewritten by the next tile
    }
    if (threadIdx.x == 0)
        out[n] = carry;
}

__global__ void k_scan_add(int *__restrict__ out, int n, const int *__restrict__ offs)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        out[i] += offs[i / SCAN_TILE];
}

__global__ void k_scan_total(int *__restrict__ out, int n, const int *__restrict__ total)
{
    out[n] = *total;
}

// ---- radix sort kernels ----

template <int IPL>
__global__ void k_radix_hist(const unsigned long long *__restrict__ key, int n, int shift,
                             unsigned int *__restrict__ hist, int nblocks)
{
    __shared__ unsigned int h[RADIX];
    for (int i = threadIdx.x; i < RADIX; i += blockDim.x)
        h[i] = 0;
    __syncthreads();
    const long long t0 = (long long)blockIdx.x * sort_tile(IPL);
    for (int k = threadIdx.x; k < sort_tile(IPL); k += blockDim.x) {
        long long i = t0 + k;
        if (i < n)
            atomicAdd(&h[(unsigned)(key[i] >> shift) & (RADIX - 1)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < RADIX; i += blockDim.x)
        hist[(size_t)i * nblocks + blockIdx.x] = h[i];
}

template <int IPL>
__global__ void k_radix_scatter(const unsigned long long *__restrict__ key_in,
                                const int *__restrict__ val_in,
                                unsigned long long *__restrict__ key_out,
                                int *__restrict__ val_out, int n, int shift,
                                const int *__restrict__ offs, int nblocks)
{
    __shared__ int wcount[SORT_WARPS][RADIX];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < SORT_WARPS * RADIX; i += blockDim.x)
        (&wcount[0][0])[i] = 0;
    __syncthreads();
    const long long w0 =
        (long long)blockIdx.x * sort_tile(IPL) + (long long)warp * (CSG_WARP * IPL);
    const unsigned lt = (1u << lane) - 1u;
    // pass 1: per-warp digit counts
    for (int c = 0; c < IPL; c++) {
        long long i = w0 + c * CSG_WARP + lane;
        int dg = (i < n) ? (int)((key_in[i] >> shift) & (RADIX - 1)) : RADIX;
        unsigned peers = __match_any_sync(0xffffffffu, dg);
        if (dg < RADIX && (peers & lt) == 0)
            wcount[warp][dg] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // per digit: tile offset + counts of earlier warps
    for (int dg = threadIdx.x; dg < RADIX; dg += blockDim.x) {
        int run = offs[(size_t)dg * nblocks + blockIdx.x];
        for (int w = 0; w < SORT_WARPS; w++) {
            int c = wcount[w][dg];
            wcount[w][dg] = run;
            run += c;
        }
    }
    __syncthreads();
    // pass 2: stable placement in input order
    for (int c = 0; c < IPL; c++) {
        long long i = w0 + c * CSG_WARP + lane;
        unsigned long long k = 0;
        int v = 0;
        int dg = RADIX;
        if (i < n) {
            k = key_in[i];
            v = val_in[i];
            dg = (int)((k >> shift) & (RADIX - 1));
        }
        unsigned peers = __match_any_sync(0xffffffffu, dg);
        int pos = 0;
        if (dg < RADIX) {
            pos = wcount[warp][dg] + __popc(peers & lt);
            key_out[pos] = k;
            val_out[pos] = v;
        }
        __syncwarp();
        if (dg < RADIX && (peers & lt) == 0)
            wcount[warp][dg] += __popc(peers);
        __syncwarp();
    }
}

} // namespace

int csg_scan_exclusive(csgd_t *d, const int *in, int *out, int n, const int *count_limit)
{
    if (n <= 0) {
        cudaMemsetAsync(out, 0, sizeof(int), d->stream);
        return csgd_check(d, cudaGetLastError());
    }
    if (n <= SCAN_SMALL) {
        { k_scan_small<<<1, SCAN_THREADS, 0, d->stream>>>(in, out, n, count_limit); d->launches++; }
        return csgd_check(d, cudaGetLastError());
    }
    // level sizes: n -> ceil(n/T) -> ... -> 1
    int nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    int *sums = d->scan_tmp;
    int needed = 0;
    for (int m = nb; m > 1; m = (m + SCAN_TILE - 1) / SCAN_TILE)
        needed += 2 * m + 2;
    needed += 2;
    if (needed > d->scan_tmp_cap) {
        csgd_set_err(d, CSG_ERR_NOMEM);
        return CSG_ERR_NOMEM;
    }
    { k_scan_tile<<<nb, SCAN_THREADS, 0, d->stream>>>(in, out, n, count_limit, sums); d->launches++; }
    if (nb > 1) {
        // scan the block sums (exclusive, total at sums_out[nb]) and add back
        int *sums_out = sums + nb + 1;
        // temporarily shift the scratch window for the recursive level
        int *saved = d->scan_tmp;
        int saved_cap = d->scan_tmp_cap;
        d->scan_tmp = sums_out + nb + 1;
        d->scan_tmp_cap = saved_cap - 2 * (nb + 1);
        int rc = csg_scan_exclusive(d, sums, sums_out, nb, nullptr);
        d->scan_tmp = saved;
        d->scan_tmp_cap = saved_cap;
        if (rc)
            return rc;
        { k_scan_add<<<csgd_grid(n, 256), 256, 0, d->stream>>>(out, n, sums_out); d->launches++; }
        { k_scan_total<<<1, 1, 0, d->stream>>>(out, n, sums_out + nb); d->launches++; }
    } else {
        { k_scan_total<<<1, 1, 0, d->stream>>>(out, n, sums); d->launches++; }
    }
    return csgd_check(d, cudaGetLastError());
}

int csg_radix_sort(csgd_t *d, unsigned long long *key, int *val, unsigned long long *key_alt,
                   int *val_alt, int n, int bits)
{
    if (n <= 1)
        return CSG_OK;
    const bool small = n < (2 << 20);
    const int tile = small ? sort_tile(4) : sort_tile(16);
    const int nblocks = (n + tile - 1) / tile;
    const int hn = RADIX * nblocks;
    if (2 * hn + 1 > d->sort_hist_cap) {
        csgd_set_err(d, CSG_ERR_NOMEM);
        return CSG_ERR_NOMEM;
    }
    unsigned int *hist = d->sort_hist;
    int *offs = (int *)(d->sort_hist + hn);
    unsigned long long *ki = key, *ko = key_alt;
    int *vi = val, *vo = val_alt;
    const int passes = (bits + 7) / 8;
    for (int p = 0; p < passes; p++) {
        const int shift = 8 * p;
        if (small)
            { k_radix_hist<4><<<nblocks, SORT_THREADS, 0, d->stream>>>(ki, n, shift, hist, nblocks); d->launches++; }
        else
            { k_radix_hist<16><<<nblocks, SORT_THREADS, 0, d->stream>>>(ki, n, shift, hist, nblocks); d->launches++; }
        int rc = csg_scan_exclusive(d, (const int *)hist, offs, hn, nullptr);
        if (rc)
            return rc;
        if (small)
            { k_radix_scatter<4><<<nblocks, SORT_THREADS, 0, d->stream>>>(ki, vi, ko, vo, n, shift, offs, nblocks); d->launches++; }
        else
            { k_radix_scatter<16><<<nblocks, SORT_THREADS, 0, d->stream>>>(ki, vi, ko, vo, n, shift, offs, nblocks); d->launches++; }
        unsigned long long *tk = ki;
        ki = ko;
        ko = tk;
        int *tv = vi;
        vi = vo;
        vo = tv;
    }
    if (ki != key) {
        cudaMemcpyAsync(key, ki, sizeof(unsigned long long) * (size_t)n, cudaMemcpyDeviceToDevice,
                        d->stream);
        cudaMemcpyAsync(val, vi, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, d->stream);
    }
    return csgd_check(d, cudaGetLastError());
}
