// dev_sort.cu — exclusive scan and stable LSD radix sort used by the tree build.
//
// Radix sort: 8-bit digits; one kernel counts the digits of every pass, then
// one single-pass kernel per digit (tiles of 512 keys below 64k keys, 1024
// below 2M, 2048 above) finds each tile's offsets by decoupled look-back and writes the tile
// out reordered by digit in shared memory (coalesced runs). Stability inside a
// tile comes from giving each warp a contiguous slice of the tile and ranking
// equal digits in input order (a lane's peers, the lanes holding the same
// digit, from nine ballots on the digit's bits); across tiles from the
// look-back's tile order. Stability matters: keys that tie keep caller index
// order, which the tree build relies on (reference inserts bodies in index
// order, src/octree.c:163-168).
#include "dev_internal.cuh"

namespace {

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

constexpr int SORT_THREADS = 256;
constexpr int SORT_WARPS = SORT_THREADS / CSG_WARP;
// Items per lane: 8 (tiles of 2048 keys) for large sorts, 4 (tiles of 1024)
// below 2M keys, so that a 100k-key sort still spreads over ~100 blocks, and 2
// (tiles of 512) below 64k keys.
constexpr int sort_tile(int ipl) { return SORT_WARPS * CSG_WARP * ipl; }
constexpr int RADIX = 256;

// Lanes of the warp whose value equals this lane's (values 0..511): the
// intersection over the nine bits of the ballots that agree with this lane's
// bit. All lanes take part.
__device__ __forceinline__ unsigned same_digit_lanes(unsigned v)
{
    unsigned m = 0xffffffffu;
#pragma unroll
    for (int b = 0; b < 9; b++) {
        const unsigned bal = __ballot_sync(0xffffffffu, (v >> b) & 1u);
        m &= ((v >> b) & 1u) ? bal : ~bal;
    }
    return m;
}

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
    pdl_enter();
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
    pdl_enter();
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
    pdl_enter();
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        out[i] += offs[i / SCAN_TILE];
}

__global__ void k_scan_total(int *__restrict__ out, int n, const int *__restrict__ total)
{
    pdl_enter();
    out[n] = *total;
}

// ---- radix sort kernels ----
//
// LSD radix sort, 8 bits per pass, in the single-pass form with decoupled
// look-back (Merrill & Garland, "Single-pass Parallel Prefix Scan with
// Decoupled Look-back", 2016; applied to radix sorting as "Onesweep", Adinets
// & Merrill 2022): one kernel counts the digits of every pass in one read of
// the keys; then each pass is one kernel. A block takes the next tile index
// from a counter (so every earlier tile belongs to a block that is already
// running), counts its tile's digits, publishes them, and sums the published
// counts of the tiles before it, walking back until a tile that has
// published its inclusive prefix. With the global digit offsets that gives
// every key its place; within a tile keys keep their input order (stable).

constexpr unsigned long long LB_AGG = 1ull << 62; // tile count published
constexpr unsigned long long LB_PRE = 1ull << 63; // inclusive prefix published
constexpr unsigned long long LB_VAL = LB_AGG - 1;
constexpr int LB_WINDOW = 8; // tiles whose status words a look-back step reads at once

// layout of the sort scratch (32-bit words): digit counts [8][256], tile
// counters [8], padding to an 8-byte boundary, then two status buffers of
// 64-bit words, [tile][256] each (pass p uses buffer p % 2)
constexpr int SORT_COUNTS = 0;
constexpr int SORT_TILE_CTR = 8 * RADIX;
constexpr int SORT_STATUS = 8 * RADIX + 64;

__device__ __forceinline__ void lb_store(unsigned long long *p, unsigned long long v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ unsigned long long lb_load(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Waits (at most `limit` polls) until the status word q carries a published
// count or prefix; returns it, or 0 after giving up (CSG_ERR_DEVICE_WAIT
// recorded). The look-back's only wait.
__device__ unsigned long long lb_wait(const unsigned long long *q, int limit, DevScalars *sc)
{
    unsigned long long v = lb_load(q);
    int spins = 0;
    while (!(v & (LB_AGG | LB_PRE)) && ++spins < limit)
        v = lb_load(q);
    if (!(v & (LB_AGG | LB_PRE))) {
        dev_fail(sc, CSG_ERR_DEVICE_WAIT);
        return 0ull;
    }
    return v;
}

// Digit counts of passes 0..passes-1 (counts[pass][digit], zeroed before).
__global__ void __launch_bounds__(SORT_THREADS) k_radix_counts(const unsigned long long *__restrict__ key,
                                                               int n, const int *__restrict__ n_dev,
                                                               int passes,
                                                               unsigned int *__restrict__ counts)
{
    pdl_enter();
    if (n_dev)
        n = max(0, min(n, *n_dev));
    __shared__ unsigned int h[8][RADIX];
    for (int i = threadIdx.x; i < 8 * RADIX; i += blockDim.x)
        (&h[0][0])[i] = 0;
    __syncthreads();
    // plain shared-memory atomics: measured faster than aggregating equal
    // digits of a warp first (the ballots cost more than the collisions)
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const unsigned long long k = key[i];
        for (int p = 0; p < passes; p++)
            atomicAdd(&h[p][(int)((k >> (8 * p)) & (RADIX - 1))], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * RADIX; i += blockDim.x) {
        const unsigned c = (&h[0][0])[i];
        if (c)
            atomicAdd(&counts[i], c);
    }
}

// One pass: keys/values of a tile to their places. counts: this pass's 256
// digit counts; status / status_next: this pass's and the next pass's status
// buffers (this pass clears its tile's entries of the next one).
//
// The tile's keys stay in registers after one coalesced read. Each key's rank
// among the equal digits of its warp slice comes from the ballots; per-digit
// counts give every key its place in the tile sorted by digit (stable: warp
// slices in order, within a slice input order). The tile is reordered so in
// shared memory, then written out in tile order, so consecutive threads write
// consecutive slots of one digit's run: coalesced stores instead of up to 32
// scattered ones per warp instruction.
template <int IPL>
__global__ void __launch_bounds__(SORT_THREADS) k_radix_onesweep(
    const unsigned long long *__restrict__ key_in, const int *__restrict__ val_in,
    unsigned long long *__restrict__ key_out, int *__restrict__ val_out, int n, int shift,
    const unsigned int *__restrict__ counts, int *__restrict__ tile_ctr,
    unsigned long long *status, unsigned long long *__restrict__ status_next, int nblocks,
    const int *__restrict__ n_dev, DevScalars *sc, int wait_polls)
{
    pdl_enter();
    constexpr int TILE = sort_tile(IPL);
    if (n_dev) { // key count known on the device only: the grid covers the bound
        n = max(0, min(n, *n_dev));
        nblocks = (n + TILE - 1) / TILE;
    }
    static_assert(SORT_THREADS == RADIX, "one digit per thread");
    __shared__ unsigned long long s_key[TILE];
    __shared__ int s_val[TILE];
    __shared__ int wcount[SORT_WARPS][RADIX]; // a warp's digit counts, then its offsets
    __shared__ int s_tds[RADIX];              // where each digit's run starts in the tile
    __shared__ long long s_glob[RADIX];       // ... and in the output
    __shared__ int warp_tot[SORT_WARPS];
    __shared__ int sh_tile;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0)
        sh_tile = atomicAdd(tile_ctr, 1);
    for (int i = threadIdx.x; i < SORT_WARPS * RADIX; i += blockDim.x)
        (&wcount[0][0])[i] = 0;
    __syncthreads();
    const int tile = sh_tile;
    if (tile >= nblocks) // only when the live count is below the bound
        return;
    status_next[(size_t)tile * RADIX + threadIdx.x] = 0ull;
    const long long t0 = (long long)tile * TILE;
    const long long w0 = t0 + (long long)warp * (CSG_WARP * IPL);
    const unsigned lt = (1u << lane) - 1u;
    unsigned long long k[IPL];
    int v[IPL], rank[IPL];
#pragma unroll
    for (int c = 0; c < IPL; c++) {
        const long long i = w0 + c * CSG_WARP + lane;
        const bool ok = i < n;
        k[c] = ok ? key_in[i] : 0ull;
        v[c] = ok ? val_in[i] : 0;
        const int dg = ok ? (int)((k[c] >> shift) & (RADIX - 1)) : RADIX;
        const unsigned peers = same_digit_lanes((unsigned)dg);
        rank[c] = (dg < RADIX ? wcount[warp][dg] : 0) + __popc(peers & lt);
        __syncwarp();
        if (dg < RADIX && (peers & lt) == 0)
            wcount[warp][dg] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // per digit (one thread each): the warps' offsets inside the digit's run
    const int dg = threadIdx.x;
    int tot = 0;
    for (int w = 0; w < SORT_WARPS; w++) {
        const int cw = wcount[w][dg];
        wcount[w][dg] = tot;
        tot += cw;
    }
    unsigned long long *mine = status + (size_t)tile * RADIX + dg;
    lb_store(mine, (tile == 0 ? LB_PRE : LB_AGG) | (unsigned long long)tot);
    // global exclusive offset of the digit (block scan of the pass's counts)
    // and the digit's start inside the tile (block scan of the tile's counts)
    const int c = (int)counts[dg];
    const int incl = warp_incl_scan(c);
    const int tincl = warp_incl_scan(tot);
    if (lane == 31)
        warp_tot[warp] = incl;
    __syncthreads();
    int gex = incl - c;
    for (int w = 0; w < warp; w++)
        gex += warp_tot[w];
    __syncthreads();
    if (lane == 31)
        warp_tot[warp] = tincl;
    __syncthreads();
    int tds = tincl - tot;
    for (int w = 0; w < warp; w++)
        tds += warp_tot[w];
    // keys of this digit in earlier tiles: the words of LB_WINDOW tiles back
    // are read at once (their loads in flight together), then summed nearest
    // first until a tile with its inclusive prefix; a word not yet published
    // is waited for alone
    long long excl = 0;
    if (tile > 0) {
        bool fin = false;
        for (int j = tile - 1; j >= 0 && !fin; j -= LB_WINDOW) {
            unsigned long long w[LB_WINDOW];
#pragma unroll
            for (int q = 0; q < LB_WINDOW; q++)
                w[q] = j - q >= 0 ? lb_load(status + (size_t)(j - q) * RADIX + dg) : LB_PRE;
#pragma unroll
            for (int q = 0; q < LB_WINDOW; q++) {
                if (fin)
                    break;
                unsigned long long vv = w[q];
                if (!(vv & (LB_AGG | LB_PRE)))
                    vv = lb_wait(status + (size_t)(j - q) * RADIX + dg, wait_polls, sc);
                if (!vv) { // gave up (recorded): leave the wait
                    fin = true;
                    break;
                }
                excl += (long long)(vv & LB_VAL);
                fin = (vv & LB_PRE) != 0; // tile 0 always has it: j - q < 0 is never read
            }
        }
        lb_store(mine, LB_PRE | (unsigned long long)(excl + tot));
    }
    s_tds[dg] = tds;
    s_glob[dg] = (long long)gex + excl;
    __syncthreads();
    // the tile sorted by digit, in shared memory
#pragma unroll
    for (int cc = 0; cc < IPL; cc++) {
        const long long i = w0 + cc * CSG_WARP + lane;
        if (i < n) {
            const int d = (int)((k[cc] >> shift) & (RADIX - 1));
            const int lp = s_tds[d] + wcount[warp][d] + rank[cc];
            s_key[lp] = k[cc];
            s_val[lp] = v[cc];
        }
    }
    __syncthreads();
    // written out in tile order: runs of one digit land on consecutive slots
    const int count = (int)min((long long)TILE, (long long)n - t0);
#pragma unroll
    for (int cc = 0; cc < IPL; cc++) {
        const int j = threadIdx.x + cc * SORT_THREADS;
        if (j < count) {
            const unsigned long long kk = s_key[j];
            const int d = (int)((kk >> shift) & (RADIX - 1));
            const long long pos = s_glob[d] + (j - s_tds[d]);
            if (pos >= 0 && pos < n) {
                key_out[pos] = kk;
                val_out[pos] = s_val[j];
            }
        }
    }
}

// A look-back wait on a status word that nothing publishes: it must give up
// after `limit` polls and record CSG_ERR_DEVICE_WAIT (the failure path of
// the sort's only wait, without a sort around it).
__global__ void k_wait_probe(const unsigned long long *word, int limit, DevScalars *sc)
{
    if (threadIdx.x == 0 && blockIdx.x == 0)
        lb_wait(word, limit, sc);
}

} // namespace

// The real sort keeps the default limit: there a wait only ever waits on a
// tile whose block is already running, and a tile that gave up would leave
// holes in the permutation later kernels index with.
extern "C" int csgd_check_device_wait(csgd_t *d, int polls, int *status)
{
    if (polls < 1 || !status)
        return CSG_ERR_BAD_ARG;
    unsigned long long *word = nullptr;
    if (csgd_malloc((void **)&word, sizeof(unsigned long long)) != cudaSuccess) {
        cudaGetLastError();
        return CSG_ERR_NOMEM;
    }
    cudaMemsetAsync(word, 0, sizeof(unsigned long long), d->stream);
    { k_wait_probe<<<1, 32, 0, d->stream>>>(word, polls, d->sc); d->launches++; }
    int rc = csgd_check(d, cudaGetLastError());
    const int got = rc ? rc : csgd_sync(d); // collects (and clears) the device error
    cudaFree(word);
    *status = got;
    return rc;
}

int csg_scan_exclusive(csgd_t *d, const int *in, int *out, int n, const int *count_limit)
{
    if (n <= 0) {
        cudaMemsetAsync(out, 0, sizeof(int), d->stream);
        return csgd_check(d, cudaGetLastError());
    }
    if (n <= SCAN_SMALL) {
        csgd_launch(d, k_scan_small, 1, SCAN_THREADS, d->stream, in, out, n, count_limit);
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
    csgd_launch(d, k_scan_tile, nb, SCAN_THREADS, d->stream, in, out, n, count_limit, sums);
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
        csgd_launch(d, k_scan_add, csgd_grid(n, 256), 256, d->stream, out, n, sums_out);
        csgd_launch(d, k_scan_total, 1, 1, d->stream, out, n, sums_out + nb);
    } else {
        csgd_launch(d, k_scan_total, 1, 1, d->stream, out, n, sums);
    }
    return csgd_check(d, cudaGetLastError());
}

int csg_radix_sort(csgd_t *d, unsigned long long *key, int *val, unsigned long long *key_alt,
                   int *val_alt, int n, int bits, const int *n_dev)
{
    if (n <= 1)
        return CSG_OK;
    const bool small = n < (2 << 20), tiny = n < (1 << 16);
    const int tile = tiny ? sort_tile(2) : small ? sort_tile(4) : sort_tile(8);
    const int nblocks = (n + tile - 1) / tile;
    const size_t status_words = (size_t)RADIX * nblocks; // 64-bit words per buffer
    const int passes = (bits + 7) / 8;
    if (passes < 1)
        return CSG_OK;
    if (passes > 8 || SORT_STATUS + 4 * status_words > (size_t)d->sort_hist_cap) {
        csgd_set_err(d, CSG_ERR_NOMEM);
        return CSG_ERR_NOMEM;
    }
    unsigned int *counts = d->sort_hist + SORT_COUNTS;
    int *tile_ctr = (int *)(d->sort_hist + SORT_TILE_CTR);
    unsigned long long *status = (unsigned long long *)(d->sort_hist + SORT_STATUS);
    // counts, counters and the first pass's status buffer start at zero
    cudaMemsetAsync(d->sort_hist, 0, sizeof(unsigned int) * SORT_STATUS + 8 * status_words,
                    d->stream);
    int gc = d->num_sms * 4;
    if (gc > nblocks)
        gc = nblocks;
    csgd_launch(d, k_radix_counts, gc, SORT_THREADS, d->stream, key, n, n_dev, passes, counts);
    unsigned long long *ki = key, *ko = key_alt;
    int *vi = val, *vo = val_alt;
    for (int p = 0; p < passes; p++) {
        const int shift = 8 * p;
        unsigned long long *st = status + (size_t)(p & 1) * status_words;
        unsigned long long *st_next = status + (size_t)((p + 1) & 1) * status_words;
        if (tiny)
            csgd_launch(d, k_radix_onesweep<2>, nblocks, SORT_THREADS, d->stream, ki, vi, ko, vo, n, shift, counts + RADIX * p, tile_ctr + p, st, st_next, nblocks, n_dev, d->sc, CSG_WAIT_POLLS_DEFAULT);
        else if (small)
            csgd_launch(d, k_radix_onesweep<4>, nblocks, SORT_THREADS, d->stream, ki, vi, ko, vo, n, shift, counts + RADIX * p, tile_ctr + p, st, st_next, nblocks, n_dev, d->sc, CSG_WAIT_POLLS_DEFAULT);
        else
            csgd_launch(d, k_radix_onesweep<8>, nblocks, SORT_THREADS, d->stream, ki, vi, ko, vo, n, shift, counts + RADIX * p, tile_ctr + p, st, st_next, nblocks, n_dev, d->sc, CSG_WAIT_POLLS_DEFAULT);
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

namespace {
__global__ void k_iota(int *__restrict__ v, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        v[i] = i;
}
} // namespace

extern "C" int csgd_sort_keys(csgd_t *d, const unsigned long long *keys, int n, int bits,
                              unsigned long long *out_keys, int *out_index)
{
    if (n < 0 || bits < 1 || bits > 64 || (n > 0 && (!keys || !out_keys || !out_index))) {
        return CSG_ERR_BAD_ARG;
    }
    if (n == 0)
        return CSG_OK;
    int rc = csgd_reserve(d, n);
    if (rc)
        return rc;
    cudaStream_t s = d->stream;
    cudaMemcpyAsync(d->key, keys, sizeof(unsigned long long) * (size_t)n, cudaMemcpyHostToDevice, s);
    { k_iota<<<csgd_grid(n, 256), 256, 0, s>>>(d->perm, n); d->launches++; }
    rc = csg_radix_sort(d, d->key, d->perm, d->key_alt, d->perm_alt, n, bits);
    if (rc)
        return rc;
    cudaMemcpyAsync(out_keys, d->key, sizeof(unsigned long long) * (size_t)n,
                    cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(out_index, d->perm, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, s);
    return csgd_sync(d);
}
