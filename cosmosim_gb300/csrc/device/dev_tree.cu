// dev_tree.cu — octree build from sorted octant keys, bottom-up moments,
// reference-order pool export and caller-pool import.
//
// The reference inserts bodies one by one into a pointer octree
// (src/octree.c:52-169). The cell structure that produces depends only on the
// body positions: a cell holding two or more alive bodies is split into the
// octants that hold bodies, down to depth 64 (src/octree.c:5, 71-79). This
// file builds the same cells in parallel:
//   1. bbox of the alive bodies -> root cube (src/octree.c:118-159);
//   2. each body's octant digit per level, 3 bits (east | south<<1 |
//      bottom<<2, src/octree.c:30-40), packed most-significant-first into a
//      63-bit key for levels 0..20 — so ascending key order is the reference's
//      depth-first child order;
//   3. stable radix sort of (key, body index);
//   4. bodies that share all 21 levels get the digits of levels 21..63 and
//      are ordered by them (rare: closer than 2^-21 of the root cube);
//   5. cells are maximal runs of sorted bodies with a common digit prefix; a
//      run of >= 2 bodies at level L (< 64) is an internal cell, a body alone
//      at its level is a leaf, a run of >= 2 at level 64 is one leaf whose
//      body_index is its lowest body index (the reference's max-depth leaf);
//   6. each sorted position a starts the internal cells of levels
//      (lcp(a-1,a), lcp(a,a+1)] and possibly its leaf, so an exclusive scan of
//      those counts numbers all cells in depth-first preorder.
// Cell centres are recomputed with the reference's own arithmetic
// (centre +/- 0.5*half_size per level, half_size*0.5), so split decisions and
// geometry are identical to the reference's bit for bit.
#include "dev_fpint.cuh"
#include "dev_internal.cuh"

#include <float.h>

namespace {

constexpr unsigned long long SIGN64 = 0x8000000000000000ull;
constexpr int KEY_MASK21 = (1 << 21) - 1;

__device__ __forceinline__ unsigned long long ord_enc(double v)
{
    unsigned long long u = (unsigned long long)__double_as_longlong(v);
    return (u & SIGN64) ? ~u : (u | SIGN64);
}

__device__ __forceinline__ double ord_dec(unsigned long long e)
{
    unsigned long long u = (e & SIGN64) ? (e & ~SIGN64) : ~e;
    return __longlong_as_double((long long)u);
}

__device__ __forceinline__ bool is_alive(double m) { return !(m <= 0.0); }

// Spreads the low 21 bits of v to every third bit (bit k -> bit 3k).
__device__ __forceinline__ unsigned long long spread3(unsigned long long v)
{
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

// One level of the reference descent: octant code, then the child cube
// (src/octree.c:30-50 and :87-90, :105-108).
__device__ __forceinline__ int descend_one(double px, double py, double pz, double &cx,
                                           double &cy, double &cz, double &hs)
{
    int q = (px >= cx ? 1 : 0) | (py < cy ? 2 : 0) | (pz < cz ? 4 : 0);
    double ox = (q & 1) ? 0.5 : -0.5;
    double oy = (q & 2) ? -0.5 : 0.5;
    double oz = (q & 4) ? -0.5 : 0.5;
    cx = cx + ox * hs;
    cy = cy + oy * hs;
    cz = cz + oz * hs;
    hs = hs * 0.5;
    return q;
}

// Digits of levels [l0, l0+nl) packed most-significant-first, after descending
// l0 levels; also returns the cube reached.
__device__ unsigned long long exact_digits(double px, double py, double pz, const DevRoot *r,
                                           int l0, int nl)
{
    double cx = r->c0[0], cy = r->c0[1], cz = r->c0[2], hs = r->hs0;
    for (int l = 0; l < l0; l++)
        descend_one(px, py, pz, cx, cy, cz, hs);
    unsigned long long k = 0;
    for (int l = 0; l < nl; l++)
        k = (k << 3) | (unsigned long long)descend_one(px, py, pz, cx, cy, cz, hs);
    return k;
}

__device__ __forceinline__ int clz_levels(unsigned long long x) { return (__clzll(x) - 1) / 3; }

// Number of leading levels two sorted positions share (0..64); -1 when they
// belong to different systems of a forest (no common cell).
__device__ __forceinline__ int lcp_pos(const unsigned long long *__restrict__ key,
                                       const unsigned long long *__restrict__ ext,
                                       const int *__restrict__ sgid, int a, int b)
{
    if (sgid[a] != sgid[b])
        return -1;
    unsigned long long ka = key[a], kb = key[b];
    if (ka != kb)
        return clz_levels(ka ^ kb);
    const unsigned long long *ea = ext + 3 * (size_t)a, *eb = ext + 3 * (size_t)b;
    if (ea[0] != eb[0])
        return 21 + clz_levels(ea[0] ^ eb[0]);
    if (ea[1] != eb[1])
        return 42 + clz_levels(ea[1] ^ eb[1]);
    return (ea[2] != eb[2]) ? 63 : 64;
}

// Digit of level l (0..63) of sorted position p.
__device__ __forceinline__ int digit_at(const unsigned long long *__restrict__ key,
                                        const unsigned long long *__restrict__ ext, int p, int l)
{
    if (l < 21)
        return (int)((key[p] >> (3 * (20 - l))) & 7ull);
    if (l < 42)
        return (int)((ext[3 * (size_t)p] >> (3 * (41 - l))) & 7ull);
    if (l < 63)
        return (int)((ext[3 * (size_t)p + 1] >> (3 * (62 - l))) & 7ull);
    return (int)(ext[3 * (size_t)p + 2] & 7ull);
}

// ---- 1. bbox -----------------------------------------------------------

__global__ void k_reset(DevScalars *sc, DevRoot *roots, int n_gal)
{
    pdl_enter();
    for (int g = threadIdx.x; g < n_gal; g += blockDim.x) {
        for (int a = 0; a < 3; a++) {
            roots[g].omin[a] = ~0ull;
            roots[g].omax[a] = 0ull;
        }
        roots[g].n_alive = 0;
    }
    if (threadIdx.x == 0) {
        sc->n_alive = 0;
        sc->deep = 0;
        sc->n_gas = 0;
        sc->key_slow = 0;
        sc->n_tasks = 0;
        sc->task_next = 0;
    }
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v)
{
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long t = __shfl_xor_sync(0xffffffffu, v, o);
        v = t < v ? t : v;
    }
    return v;
}
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v)
{
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long t = __shfl_xor_sync(0xffffffffu, v, o);
        v = t > v ? t : v;
    }
    return v;
}

// Alive-body bbox (src/octree.c:118-139). NaN coordinates never win a
// comparison in the reference, so they are left out here too.
// Grid-stride pass; each warp keeps a running box and count for the system
// its bodies belong to (a system's bodies are contiguous) and flushes it with
// one set of atomics when the system changes or at the end, so a single
// system costs one flush per warp, not one per 32 bodies. Lanes of a warp
// that straddles a system boundary fall back to per-lane atomics.
__device__ __forceinline__ void bbox_flush(DevRoot *roots, int g, unsigned long long lo[3],
                                           unsigned long long hi[3], int &cnt)
{
#pragma unroll
    for (int a = 0; a < 3; a++) {
        lo[a] = warp_min_u64(lo[a]);
        hi[a] = warp_max_u64(hi[a]);
    }
    for (int o = 16; o > 0; o >>= 1)
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0 && g >= 0) {
        for (int a = 0; a < 3; a++) {
            if (lo[a] != ~0ull)
                atomicMin(&roots[g].omin[a], lo[a]);
            if (hi[a] != 0ull)
                atomicMax(&roots[g].omax[a], hi[a]);
        }
        if (cnt)
            atomicAdd(&roots[g].n_alive, cnt);
    }
    for (int a = 0; a < 3; a++) {
        lo[a] = ~0ull;
        hi[a] = 0ull;
    }
    cnt = 0;
}

__global__ void k_bbox(const double *__restrict__ x, const double *__restrict__ y,
                       const double *__restrict__ z, const double *__restrict__ m,
                       const int *__restrict__ gid, int n, DevRoot *roots, DevScalars *gsc)
{
    pdl_enter();
    unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0ull, 0ull, 0ull};
    int cnt = 0;
    int cur_g = -1; // warp-uniform: the system the running box belongs to
    bool bad = false; // a non-finite mass, or a non-finite position of a live body
    for (long long base = (long long)blockIdx.x * blockDim.x; base < n;
         base += (long long)gridDim.x * blockDim.x) {
        const long long i = base + threadIdx.x;
        const int g = (i < n) ? gid[i] : -1;
        if (g >= 0) {
            const double mi = m[i];
            bad |= !isfinite(mi) ||
                   (is_alive(mi) && !(isfinite(x[i]) && isfinite(y[i]) && isfinite(z[i])));
        }
        const int g0 = __shfl_sync(0xffffffffu, g, 0);
        if (!__all_sync(0xffffffffu, g == g0 || g < 0)) { // straddles systems
            if (g >= 0 && is_alive(m[i])) {
                const double p[3] = {x[i], y[i], z[i]};
                for (int a = 0; a < 3; a++) {
                    if (p[a] != p[a])
                        continue;
                    atomicMin(&roots[g].omin[a], ord_enc(p[a]));
                    atomicMax(&roots[g].omax[a], ord_enc(p[a]));
                }
                atomicAdd(&roots[g].n_alive, 1);
            }
            continue;
        }
        if (g0 != cur_g) {
            if (cur_g >= 0)
                bbox_flush(roots, cur_g, lo, hi, cnt);
            cur_g = g0;
        }
        if (g >= 0 && is_alive(m[i])) {
            cnt++;
            const double p[3] = {x[i], y[i], z[i]};
#pragma unroll
            for (int a = 0; a < 3; a++) {
                if (p[a] != p[a])
                    continue;
                const unsigned long long e = ord_enc(p[a]);
                lo[a] = e < lo[a] ? e : lo[a];
                hi[a] = e > hi[a] ? e : hi[a];
            }
        }
    }
    // the warps' last running boxes: combined in the block first, one set of
    // atomics per system the block ends on (one per block for a single system)
    __shared__ unsigned long long s_lo[32][3], s_hi[32][3];
    __shared__ int s_cnt[32], s_g[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        lo[a] = warp_min_u64(lo[a]);
        hi[a] = warp_max_u64(hi[a]);
    }
    for (int o = 16; o > 0; o >>= 1)
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if (lane == 0) {
        s_g[warp] = cur_g;
        s_cnt[warp] = cnt;
        for (int a = 0; a < 3; a++) {
            s_lo[warp][a] = lo[a];
            s_hi[warp][a] = hi[a];
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int g = -1, c = 0;
        unsigned long long l[3] = {~0ull, ~0ull, ~0ull}, h[3] = {0ull, 0ull, 0ull};
        const int nw = (int)(blockDim.x >> 5);
        for (int w = 0; w <= nw; w++) {
            const int gw = w < nw ? s_g[w] : -1;
            if (w == nw || (gw >= 0 && gw != g)) {
                if (g >= 0) { // flush the system collected so far
                    for (int a = 0; a < 3; a++) {
                        if (l[a] != ~0ull)
                            atomicMin(&roots[g].omin[a], l[a]);
                        if (h[a] != 0ull)
                            atomicMax(&roots[g].omax[a], h[a]);
                    }
                    if (c)
                        atomicAdd(&roots[g].n_alive, c);
                }
                if (w == nw)
                    break;
                g = gw;
                c = 0;
                for (int a = 0; a < 3; a++) {
                    l[a] = ~0ull;
                    h[a] = 0ull;
                }
            }
            if (gw < 0)
                continue;
            c += s_cnt[w];
            for (int a = 0; a < 3; a++) {
                l[a] = s_lo[w][a] < l[a] ? s_lo[w][a] : l[a];
                h[a] = s_hi[w][a] > h[a] ? s_hi[w][a] : h[a];
            }
        }
    }
    if (bad)
        dev_fail(gsc, CSG_ERR_BAD_ARG);
}

// Root cube, reference src/octree.c:141-159, plus the fast-key parameters.
__device__ void root_cube(DevRoot *sc)
{
    if (sc->n_alive == 0) {
        sc->c0[0] = sc->c0[1] = sc->c0[2] = 0.0;
        sc->hs0 = 1.0;
        sc->fast_keys = 0;
        sc->key_scale = 0.0;
        sc->key_off[0] = sc->key_off[1] = sc->key_off[2] = 0.0;
        sc->key_tol = 1ll << 32;
        return;
    }
    double lo[3], hi[3];
    for (int a = 0; a < 3; a++) {
        lo[a] = (sc->omin[a] == ~0ull) ? DBL_MAX : ord_dec(sc->omin[a]);
        hi[a] = (sc->omax[a] == 0ull) ? -DBL_MAX : ord_dec(sc->omax[a]);
        sc->c0[a] = (lo[a] + hi[a]) * 0.5;
    }
    double ext = hi[0] - lo[0];
    if (hi[1] - lo[1] > ext)
        ext = hi[1] - lo[1];
    if (hi[2] - lo[2] > ext)
        ext = hi[2] - lo[2];
    double hs = ext * 0.5;
    hs = hs * 1.01;
    if (hs < 1e-10)
        hs = 1.0;
    sc->hs0 = hs;
    // Fast keys: t = p * 2^20/hs + (2^20 - c0 * 2^20/hs), one fused
    // multiply-add per axis, lies within ~2 R 2^-32 grid units of the exact
    // descent, R = 1 + max|c0|/hs (the roundings of 2^20/hs, of c0 * 2^20/hs
    // and of the sums, each <= R 2^-33 or 2^-32). Bodies within the guard
    // (64 R 2^-32) of a split point take the exact descent. All values are
    // kept x 2^32 (exact) so that floor and fraction come from one int64.
    double r = fmax(fabs(sc->c0[0]), fmax(fabs(sc->c0[1]), fabs(sc->c0[2]))) / hs + 1.0;
    double tol = 64.0 * r * 0x1p-32;
    bool finite = isfinite(sc->c0[0]) && isfinite(sc->c0[1]) && isfinite(sc->c0[2]) &&
                  isfinite(hs) && hs > 0.0;
    sc->fast_keys = (finite && tol < 0.25) ? 1 : 0;
    const double scale = finite ? 1048576.0 / hs : 0.0;
    sc->key_scale = scale * 0x1p32;
    for (int a = 0; a < 3; a++)
        sc->key_off[a] = finite ? (1048576.0 - sc->c0[a] * scale) * 0x1p32 : 0.0;
    sc->key_tol = sc->fast_keys ? (long long)(64.0 * r) + 1 : (1ll << 32);
}

// Root cube of every system, then where each system's alive bodies start in
// the sorted order (systems sort in id order) and the total alive count.
__global__ void k_root(DevScalars *sc, DevRoot *roots, int n_gal)
{
    pdl_enter();
    // After an error (non-finite input found by k_bbox, or an earlier failure
    // not yet collected) the tree is built empty: no key is formed from the
    // bodies and nothing downstream walks them.
    const bool failed = sc->err != 0;
    for (int g = threadIdx.x; g < n_gal; g += blockDim.x) {
        if (failed)
            roots[g].n_alive = 0;
        root_cube(&roots[g]);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int off = 0;
        for (int g = 0; g < n_gal; g++) {
            roots[g].first = off;
            roots[g].root = roots[g].end = 0;
            off += roots[g].n_alive;
        }
        sc->n_alive = off;
    }
}

// ---- 2. keys -----------------------------------------------------------

// Key grid index of one coordinate when it is clear of every split point by
// the guard; t32 = grid position x 2^32 (one FP64 fused multiply-add), its
// integer part >> 32 is the index, its low 32 bits the fraction.
__device__ __forceinline__ bool fast_coord(double p, double scale, double off, long long tol,
                                           int &i)
{
    const double t32 = fma(p, scale, off);
    if (!(t32 >= 0.0 && t32 < 0x1p53)) // also NaN
        return false;
    const long long v = __double2ll_rz(t32);
    const long long frac = v & 0xFFFFFFFFll;
    if (v < tol || v > (1ll << 53) - tol || frac < tol || frac > (1ll << 32) - tol)
        return false;
    i = (int)(v >> 32);
    return true;
}

__global__ void k_keys(const double *__restrict__ x, const double *__restrict__ y,
                       const double *__restrict__ z, const double *__restrict__ m,
                       const int *__restrict__ gid, int n, DevScalars *gsc,
                       const DevRoot *__restrict__ roots, unsigned long long *__restrict__ key,
                       int *__restrict__ perm)
{
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    perm[i] = i;
    if (!is_alive(m[i]) || gsc->err != 0) { // see k_root: after an error no body is keyed
        key[i] = CSG_DEAD_KEY;
        return;
    }
    const DevRoot *sc = &roots[gid[i]];
    const double px = x[i], py = y[i], pz = z[i];
    int ix, iy, iz;
    if (sc->fast_keys && fast_coord(px, sc->key_scale, sc->key_off[0], sc->key_tol, ix) &&
        fast_coord(py, sc->key_scale, sc->key_off[1], sc->key_tol, iy) &&
        fast_coord(pz, sc->key_scale, sc->key_off[2], sc->key_tol, iz)) {
        // east = upper x half; south = lower y half; bottom = lower z half
        unsigned long long sx = (unsigned long long)ix;
        unsigned long long sy = (unsigned long long)(~iy & KEY_MASK21);
        unsigned long long sz = (unsigned long long)(~iz & KEY_MASK21);
        key[i] = spread3(sx) | (spread3(sy) << 1) | (spread3(sz) << 2);
    } else {
        key[i] = exact_digits(px, py, pz, sc, 0, 21);
        atomicAdd(&gsc->key_slow, 1ull);
    }
}

// ---- 4. positions that share a 63-bit key ------------------------------

// System of every sorted position (-1 past the alive bodies).
__global__ void k_sgid(const DevScalars *sc, const int *__restrict__ perm,
                       const int *__restrict__ gid, int *__restrict__ sgid, int n)
{
    pdl_enter();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n)
        sgid[p] = (p < sc->n_alive) ? gid[perm[p]] : -1;
}

__device__ __forceinline__ bool same_key(const unsigned long long *key, const int *sgid, int a,
                                         int b)
{
    return key[a] == key[b] && sgid[a] == sgid[b];
}

__global__ void k_deep_mark(const double *__restrict__ x, const double *__restrict__ y,
                            const double *__restrict__ z, DevScalars *sc,
                            const DevRoot *__restrict__ roots,
                            const unsigned long long *__restrict__ key,
                            const int *__restrict__ sgid, const int *__restrict__ perm,
                            unsigned long long *__restrict__ ext)
{
    pdl_enter();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int na = sc->n_alive;
    if (p >= na)
        return;
    bool deep = (p > 0 && same_key(key, sgid, p - 1, p)) ||
                (p + 1 < na && same_key(key, sgid, p, p + 1));
    if (!deep)
        return;
    const int b = perm[p];
    const DevRoot *r = &roots[sgid[p]];
    ext[3 * (size_t)p + 0] = exact_digits(x[b], y[b], z[b], r, 21, 21);
    ext[3 * (size_t)p + 1] = exact_digits(x[b], y[b], z[b], r, 42, 21);
    ext[3 * (size_t)p + 2] = exact_digits(x[b], y[b], z[b], r, 63, 1);
    atomicAdd(&sc->deep, 1);
}

__device__ __forceinline__ bool ext_less(const unsigned long long *e, int a, int b)
{
    for (int w = 0; w < 3; w++) {
        unsigned long long ea = e[3 * (size_t)a + w], eb = e[3 * (size_t)b + w];
        if (ea != eb)
            return ea < eb;
    }
    return false;
}

// Orders each run of equal 63-bit keys by its deeper digits; insertion sort is
// stable, so equal full keys keep body index order.
__global__ void k_deep_sort(DevScalars *sc, const unsigned long long *__restrict__ key,
                            const int *__restrict__ sgid, int *__restrict__ perm,
                            unsigned long long *__restrict__ ext)
{
    pdl_enter();
    if (sc->deep == 0)
        return;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int na = sc->n_alive;
    if (p >= na)
        return;
    if (!(p + 1 < na && same_key(key, sgid, p, p + 1)) || (p > 0 && same_key(key, sgid, p - 1, p)))
        return; // not the start of a run
    int e = p + 1;
    while (e < na && same_key(key, sgid, p, e))
        e++;
    for (int i = p + 1; i < e; i++) {
        unsigned long long t0 = ext[3 * (size_t)i], t1 = ext[3 * (size_t)i + 1],
                           t2 = ext[3 * (size_t)i + 2];
        int tp = perm[i];
        int j = i - 1;
        while (j >= p) {
            unsigned long long u0 = ext[3 * (size_t)j], u1 = ext[3 * (size_t)j + 1],
                               u2 = ext[3 * (size_t)j + 2];
            bool greater = (u0 != t0) ? (u0 > t0) : (u1 != t1) ? (u1 > t1) : (u2 > t2);
            if (!greater)
                break;
            ext[3 * (size_t)(j + 1)] = u0;
            ext[3 * (size_t)(j + 1) + 1] = u1;
            ext[3 * (size_t)(j + 1) + 2] = u2;
            perm[j + 1] = perm[j];
            j--;
        }
        ext[3 * (size_t)(j + 1)] = t0;
        ext[3 * (size_t)(j + 1) + 1] = t1;
        ext[3 * (size_t)(j + 1) + 2] = t2;
        perm[j + 1] = tp;
    }
}

// ---- 5/6. cells ----------------------------------------------------------

__global__ void k_count(DevScalars *sc, const unsigned long long *__restrict__ key,
                        const unsigned long long *__restrict__ ext, const int *__restrict__ sgid,
                        signed char *__restrict__ lcp, int *__restrict__ cnt)
{
    pdl_enter();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int na = sc->n_alive;
    if (p >= na)
        return;
    int P = (p > 0) ? lcp_pos(key, ext, sgid, p - 1, p) : -1;
    int Q = (p + 1 < na) ? lcp_pos(key, ext, sgid, p, p + 1) : -1;
    lcp[p] = (signed char)Q;
    int internal = min(Q, CSG_MAX_LEVEL - 1) - P;
    cnt[p] = (internal > 0 ? internal : 0) + (P < CSG_MAX_LEVEL ? 1 : 0);
}

__device__ int search_hi(const unsigned long long *key, const unsigned long long *ext,
                         const int *sgid, int na, int p, int L)
{
    int q = p, step = 1;
    while (true) {
        int t = q + step;
        if (t >= na || lcp_pos(key, ext, sgid, p, t) < L)
            break;
        q = t;
        step <<= 1;
    }
    while (step > 1) {
        step >>= 1;
        int t = q + step;
        if (t < na && lcp_pos(key, ext, sgid, p, t) >= L)
            q = t;
    }
    return q;
}

__device__ int search_lo(const unsigned long long *key, const unsigned long long *ext,
                         const int *sgid, int p, int L)
{
    int q = p, step = 1;
    while (true) {
        int t = q - step;
        if (t < 0 || lcp_pos(key, ext, sgid, t, p) < L)
            break;
        q = t;
        step <<= 1;
    }
    while (step > 1) {
        step >>= 1;
        int t = q - step;
        if (t >= 0 && lcp_pos(key, ext, sgid, t, p) >= L)
            q = t;
    }
    return q;
}

__device__ __forceinline__ int parent_id(const unsigned long long *key,
                                         const unsigned long long *ext, const int *sgid,
                                         const signed char *lcp, const int *base, int p, int P,
                                         int L, int id)
{
    if (L == 0)
        return -1;
    if (L - 1 > P)
        return id - 1; // the cell one level up starts at p as well
    int a = search_lo(key, ext, sgid, p, L - 1);
    int Pa = (a > 0) ? (int)lcp[a - 1] : -1;
    return base[a] + (L - 1) - (Pa + 1);
}

__device__ __forceinline__ void write_cell(csgd_t dd, DevScalars *sc, double hs0, int id,
                                           int parent, int L, int first, int count, int next,
                                           int body)
{
    if (id >= dd.node_cap) {
        dev_fail(sc, CSG_ERR_NODE_CAPACITY);
        return;
    }
    double hs = ldexp(hs0, -L);
    double s = 2.0 * hs;
    double s2 = s * s;
    // the structural fields only: k_moments writes every cell's centre of
    // mass and mass
    NodeW64 &w = dd.w64[id];
    w.s2 = s2;
    *(int2 *)&w.next = make_int2(next, body);
    NodeW32 &v = dd.w32[id];
    v.s2 = (float)s2;
    *(int4 *)&v.next = make_int4(next, body, __float_as_int((float)s), 0);
    dd.link[id] = NodeLink{parent, L, first, count};
    int4 *c = (int4 *)(dd.child + 8 * (size_t)id);
    c[0] = make_int4(-1, -1, -1, -1);
    c[1] = make_int4(-1, -1, -1, -1);
    dd.nchild[id] = 0;
    dd.ticket[id] = 0;
}

// leaf_of[p]: the leaf cell that starts at sorted position p, or -1 (a
// position inside a depth-64 multi-body leaf).
__global__ void k_nodes(csgd_t dd, DevScalars *sc, const DevRoot *__restrict__ roots,
                        const unsigned long long *__restrict__ key,
                        const unsigned long long *__restrict__ ext, const int *__restrict__ sgid,
                        const signed char *__restrict__ lcp, const int *__restrict__ base,
                        const int *__restrict__ perm, int *__restrict__ leaf_of)
{
    pdl_enter();
    // one thread per cell (and, for positions without a leaf, per position;
    // grid-stride beyond the grid): the cells of a position are written by as
    // many threads, so no thread walks the searches of a whole column of levels
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    const int na = sc->n_alive;
    if (t0 == 0) {
        int total = (na == 0) ? 1 : base[na];
        sc->n_nodes = total;
        if (total > dd.node_cap)
            dev_fail(sc, CSG_ERR_NODE_CAPACITY);
        if (na == 0) { // empty root, reference src/octree.c:141-144
            write_cell(dd, sc, 1.0, 0, -1, 0, 0, 0, 1, -1);
            double2 *w = (double2 *)&dd.w64[0];
            w[0] = w[1] = make_double2(0.0, 0.0);
            float4 *v = (float4 *)&dd.w32[0];
            v[0] = make_float4(0.f, 0.f, 0.f, 0.f);
            v[1] = make_float4(0.f, 0.f, 0.f, dd.w32[0].s2);
            dd.minidx[0] = make_int2(INT_MAX, INT_MAX);
            return;
        }
    }
    if (na == 0)
        return;
    const int total = base[na];
    const int limit = max(total, na);
    for (int c = t0; c < limit; c += gridDim.x * blockDim.x) {
        if (c < na && c > 0 && (int)lcp[c - 1] >= CSG_MAX_LEVEL)
            leaf_of[c] = -1; // bodies equal to depth 64 after the first share its leaf
        if (c >= total)
            continue;
        // the position whose cells include id c: the last p with base[p] <= c
        int lo = 0, hi = na - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (base[mid] <= c)
                lo = mid;
            else
                hi = mid - 1;
        }
        const int p = lo;
        const double hs0 = roots[sgid[p]].hs0;
        const int P = (p > 0) ? (int)lcp[p - 1] : -1;
        const int Q = (int)lcp[p];
        const int j = c - base[p];
        const int internal = min(Q, CSG_MAX_LEVEL - 1) - P; // levels P+1 .. before the leaf
        if (j < internal) {
            const int L = P + 1 + j;
            const int hi_p = search_hi(key, ext, sgid, na, p, L);
            const int parent = parent_id(key, ext, sgid, lcp, base, p, P, L, c);
            write_cell(dd, sc, hs0, c, parent, L, p, hi_p - p + 1, base[hi_p + 1], -1);
        } else { // the leaf (a position without one has no cell to land here)
            const int L = min(max(P, Q) + 1, CSG_MAX_LEVEL); // equal to depth 64: one leaf
            const int hi_p =
                (Q == CSG_MAX_LEVEL) ? search_hi(key, ext, sgid, na, p, CSG_MAX_LEVEL) : p;
            const int parent = parent_id(key, ext, sgid, lcp, base, p, P, L, c);
            write_cell(dd, sc, hs0, c, parent, L, p, hi_p - p + 1, c + 1, perm[p]);
            leaf_of[p] = c;
        }
    }
}

// Root and end cell of every system, and the walk tasks: each system's
// sorted bodies in groups of 32 (one warp each). For a tree imported from a
// caller pool (one system) the root is cell 0 and the end the cell count.
__global__ void k_tasks(DevScalars *sc, DevRoot *roots, int n_gal, const int *__restrict__ base,
                        WalkTask *tasks, int task_cap, int imported)
{
    pdl_enter();
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        int t = 0;
        for (int g = 0; g < n_gal; g++) {
            DevRoot &r = roots[g];
            if (imported) {
                r.first = 0;
                r.root = 0;
                r.end = sc->n_nodes;
            } else if (r.n_alive > 0) {
                r.root = base[r.first];
                r.end = base[r.first + r.n_alive];
            } else {
                r.root = r.end = 0;
            }
            t += (r.n_alive + 31) / 32;
        }
        if (t > task_cap) {
            dev_fail(sc, CSG_ERR_NODE_CAPACITY);
            t = task_cap;
        }
        sc->n_tasks = t;
        sc->task_next = 0;
    }
    // every block fills the tasks of its systems (roots[].first and n_alive
    // were final before this kernel)
    for (int g = blockIdx.x; g < n_gal; g += gridDim.x) {
        int t0 = 0;
        for (int h = 0; h < g; h++) // systems are few; recompute the offset
            t0 += (roots[h].n_alive + 31) / 32;
        const int n = roots[g].n_alive;
        const int first = imported ? 0 : roots[g].first;
        for (int j = threadIdx.x; j * 32 < n; j += blockDim.x) {
            if (t0 + j >= task_cap)
                break;
            WalkTask w;
            w.gal = g;
            w.pos0 = first + 32 * j;
            w.count = min(32, n - 32 * j);
            w.pad = 0;
            tasks[t0 + j] = w;
        }
    }
}

// Kernels over cells loop over ids (grid-stride): the cell count is known on
// the device only, and a grid of about 2n threads covers it in one round for
// the usual trees (cells ~1.3-2 per body) without launching for the capacity.
__global__ void k_link(csgd_t dd, DevScalars *sc, const unsigned long long *__restrict__ key,
                       const unsigned long long *__restrict__ ext)
{
    pdl_enter();
    const int nn = sc->n_nodes;
    if (nn > dd.node_cap)
        return;
    for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < nn; id += gridDim.x * blockDim.x) {
        NodeLink l = dd.link[id];
        if (l.parent < 0 || l.parent >= dd.node_cap)
            continue;
        int dg = digit_at(key, ext, l.first, l.level - 1);
        dd.child[8 * (size_t)l.parent + dg] = id;
        atomicAdd(&dd.nchild[l.parent], 1);
    }
}

// Bottom-up moments: one thread per cell of at most MOM_DIRECT bodies (and
// per leaf); above those, the last child to finish computes its parent, summing the children in
// octant order so the result does not depend on scheduling. The climb
// carries and stores raw sums (sum of m x, sum of m) in the FP64 record, so
// no division sits on its chain of dependent levels; k_moments_norm then
// turns every cell's sums into its centre of mass and writes the FP32 record.
// Only the centre of mass and mass fields are written (write_cell set the
// rest). EXPORT also keeps the two lowest body indices below each cell (the
// pool export order).
__device__ __forceinline__ void put_raw(const csgd_t &dd, int node, double ax, double ay,
                                        double az, double M)
{
    double2 *w = (double2 *)&dd.w64[node];
    w[0] = make_double2(ax, ay);
    w[1] = make_double2(az, M);
}

__device__ __forceinline__ void put_moments(const csgd_t &dd, int node, double sx, double sy,
                                            double sz, double M)
{
    double2 *w = (double2 *)&dd.w64[node];
    w[0] = make_double2(sx, sy);
    w[1] = make_double2(sz, M);
    float4 hi = make_float4((float)sx, (float)sy, (float)sz, (float)M);
    float *v = (float *)&dd.w32[node];
    *(float4 *)v = hi;
    v[4] = (float)(sx - (double)hi.x);
    v[5] = (float)(sy - (double)hi.y);
    v[6] = (float)(sz - (double)hi.z);
}

// Cell moments. A cell with at most MOM_DIRECT bodies, and every leaf, sums
// its sorted bodies directly (one thread per cell, no atomics); a larger cell
// is formed from its children's moments by the last child to finish (a ticket
// per cell), climbing from the directly summed cells whose parent is large.
// A single-body leaf keeps the body's position exactly (the reference's leaf
// centre); bodies that coincide to depth 64 share one leaf, in caller index
// order, so the two smallest caller indices of a cell are its first two.
constexpr int MOM_DIRECT = 16;

// The ticket of a cell: one gpu-scope acquire-release add. Release: this
// thread's sums (stored above) are visible to whichever child takes the last
// ticket; acquire: the last child sees every sibling's sums (the adds on one
// ticket form a release sequence).
__device__ __forceinline__ int ticket_take(int *p)
{
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
    return old;
}

template <bool EXPORT>
__device__ __forceinline__ void moments_climb(const csgd_t &dd, int node, int parent, double ax,
                                              double ay, double az, double M, int2 mi)
{
    while (true) {
        put_raw(dd, node, ax, ay, az, M);
        if (EXPORT)
            dd.minidx[node] = mi;
        if (parent < 0 || parent >= node)
            break; // preorder: a parent always precedes its children
        // the parent's children, their count and its own parent are fixed
        // since k_link: their loads run while the sums above drain
        const int4 *cp = (const int4 *)(dd.child + 8 * (size_t)parent);
        const int4 c03 = __ldg(cp), c47 = __ldg(cp + 1);
        const int nc = __ldg(&dd.nchild[parent]);
        const int up = __ldg(&dd.link[parent].parent);
        if (ticket_take(&dd.ticket[parent]) != nc - 1)
            break;
        M = 0.0;
        ax = ay = az = 0.0;
        int m1 = INT_MAX, m2 = INT_MAX;
        const int ch[8] = {c03.x, c03.y, c03.z, c03.w, c47.x, c47.y, c47.z, c47.w};
        for (int q = 0; q < 8; q++) {
            const int c = ch[q];
            if (c < 0)
                continue;
            const double2 *cw = (const double2 *)&dd.w64[c];
            const double2 xy = __ldcg(cw), zm = __ldcg(cw + 1);
            M += zm.y;
            ax += xy.x;
            ay += xy.y;
            az += zm.x;
            if (EXPORT) {
                int2 cmi = __ldcg(&dd.minidx[c]);
                int cand[2] = {cmi.x, cmi.y};
                for (int j = 0; j < 2; j++) {
                    int v2 = cand[j];
                    if (v2 < m1) {
                        m2 = m1;
                        m1 = v2;
                    } else if (v2 < m2) {
                        m2 = v2;
                    }
                }
            }
        }
        mi = make_int2(m1, m2);
        node = parent;
        parent = up;
    }
}

// Bodies summed directly, four bodies' loads in flight at a time; the additions
// keep the sorted order (M += m, then sum += m x as one fused multiply-add).
constexpr int MOM_LOADS = 4;

template <bool EXPORT>
__device__ __forceinline__ void moments_cell(const csgd_t &dd, int id, const double *__restrict__ x,
                                             const double *__restrict__ y,
                                             const double *__restrict__ z,
                                             const double *__restrict__ m,
                                             const int *__restrict__ perm)
{
    const NodeLink l = dd.link[id];
    const bool leaf = dd.nchild[id] == 0;
    if ((!leaf && l.count > MOM_DIRECT) || l.count < 1)
        return; // formed by the climb (or a cell without bodies)
    // a parent of at most MOM_DIRECT bodies sums its own bodies
    const int pcount = (l.parent >= 0) ? __ldg(&dd.link[l.parent].count) : INT_MAX;
    double M = 0.0, ax = 0.0, ay = 0.0, az = 0.0;
    int2 mi = make_int2(INT_MAX, INT_MAX);
    for (int k0 = 0; k0 < l.count; k0 += MOM_LOADS) {
        int bb[MOM_LOADS];
        double mv[MOM_LOADS], xv[MOM_LOADS], yv[MOM_LOADS], zv[MOM_LOADS];
#pragma unroll
        for (int j = 0; j < MOM_LOADS; j++)
            bb[j] = (k0 + j < l.count) ? perm[l.first + k0 + j] : -1;
#pragma unroll
        for (int j = 0; j < MOM_LOADS; j++) {
            if (bb[j] >= 0) {
                mv[j] = m[bb[j]];
                xv[j] = x[bb[j]];
                yv[j] = y[bb[j]];
                zv[j] = z[bb[j]];
            }
        }
#pragma unroll
        for (int j = 0; j < MOM_LOADS; j++) {
            if (bb[j] < 0)
                break;
            const int b = bb[j];
            const double mb = mv[j];
            M += mb;
            ax += mb * xv[j];
            ay += mb * yv[j];
            az += mb * zv[j];
            if (EXPORT) {
                if (b < mi.x) {
                    mi.y = mi.x;
                    mi.x = b;
                } else if (b < mi.y) {
                    mi.y = b;
                }
            }
        }
    }
    if (pcount <= MOM_DIRECT) {
        put_raw(dd, id, ax, ay, az, M); // the parent sums its own bodies
        if (EXPORT)
            dd.minidx[id] = mi;
        return;
    }
    moments_climb<EXPORT>(dd, id, l.parent, ax, ay, az, M, mi);
}

// Raw sums to centre of mass, every cell: a single-body leaf keeps the body's
// position exactly (the reference's leaf centre), any other cell takes
// (sum m x) / (sum m), the reciprocal correctly rounded off the FP64 pipe.
__global__ void k_moments_norm(csgd_t dd, DevScalars *sc, const double *__restrict__ x,
                               const double *__restrict__ y, const double *__restrict__ z)
{
    pdl_enter();
    const int nn = sc->n_nodes;
    if (nn > dd.node_cap || sc->n_alive == 0)
        return;
    for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < nn; id += gridDim.x * blockDim.x) {
        const NodeLink l = dd.link[id];
        if (l.count < 1)
            continue;
        const double2 *w = (const double2 *)&dd.w64[id];
        const double2 xy = w[0], zm = w[1];
        const int body = dd.w64[id].body;
        if (l.count == 1 && body >= 0) {
            put_moments(dd, id, x[body], y[body], z[body], zm.y);
        } else {
            const double inv = div_rn(1.0, zm.y);
            put_moments(dd, id, xy.x * inv, xy.y * inv, zm.x * inv, zm.y);
        }
    }
}

template <bool EXPORT>
__global__ void __launch_bounds__(256, 4) k_moments(csgd_t dd, DevScalars *sc, const double *__restrict__ x,
                          const double *__restrict__ y, const double *__restrict__ z,
                          const double *__restrict__ m, const int *__restrict__ perm)
{
    pdl_enter();
    const int nn = sc->n_nodes;
    if (nn > dd.node_cap || sc->n_alive == 0)
        return;
    for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < nn; id += gridDim.x * blockDim.x)
        moments_cell<EXPORT>(dd, id, x, y, z, m, perm);
}

// FP32 neighbour-search record of one cell (see NodeS32).
__device__ __forceinline__ void write_s32(const csgd_t &dd, int id, double cx, double cy,
                                          double cz, double hs, int body, int next)
{
    NodeS32 r;
    r.cx = (float)cx;
    r.cy = (float)cy;
    r.cz = (float)cz;
    r.hs = (float)hs;
    r.cmax = fmaxf(fabsf(r.cx), fmaxf(fabsf(r.cy), fabsf(r.cz))) + r.hs;
    r.bx = r.by = r.bz = 0.0f;
    r.body = body;
    if (body >= 0) {
        if (body >= dd.n) {
            r.body = -3; // a caller pool naming a body that does not exist
        } else if (dd.m[body] <= 0.0) {
            r.body = -2;
        } else {
            r.bx = (float)dd.x[body];
            r.by = (float)dd.y[body];
            r.bz = (float)dd.z[body];
        }
    }
    r.next = next;
    r.pad0 = r.pad1 = 0;
    dd.s32[id] = r;
}

// Geometric cube of every cell, with the reference's arithmetic.
__global__ void k_geometry(csgd_t dd, DevScalars *sc, const DevRoot *__restrict__ roots,
                           const unsigned long long *__restrict__ key,
                           const unsigned long long *__restrict__ ext,
                           const int *__restrict__ sgid)
{
    pdl_enter();
    const int nn = sc->n_nodes;
    if (nn > dd.node_cap)
        return;
    for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < nn; id += gridDim.x * blockDim.x) {
        NodeLink l = dd.link[id];
        const DevRoot *r = &roots[sc->n_alive > 0 ? sgid[l.first] : 0];
        double cx = r->c0[0], cy = r->c0[1], cz = r->c0[2], hs = r->hs0;
        for (int lev = 0; lev < l.level; lev++) {
            int q = digit_at(key, ext, l.first, lev);
            double ox = (q & 1) ? 0.5 : -0.5;
            double oy = (q & 2) ? -0.5 : 0.5;
            double oz = (q & 4) ? -0.5 : 0.5;
            cx = cx + ox * hs;
            cy = cy + oy * hs;
            cz = cz + oz * hs;
            hs = hs * 0.5;
        }
        dd.geo[id] = make_double4_32a(cx, cy, cz, hs);
        write_s32(dd, id, cx, cy, cz, hs, dd.w64[id].body, dd.w64[id].next);
    }
}

// ---- export in the reference's allocation order --------------------------
//
// The reference allocates a cell while inserting some body k (index order).
// With S = the cell's bodies and T = its parent's, that k is max(min S,
// second-smallest of T); cells allocated during one insertion come in
// increasing depth, and at the one depth where two appear (the split that
// finally separates the old body j from k) j's cell comes first. Sorting
// cells by (k, depth, [min S == k]) therefore reproduces pool numbering.

// The export kernels stride over the cells (their count is known on the
// device only) with a grid sized for the usual trees, not for the capacity:
// they run beside the walk and should hold few of its warp slots.
__global__ void k_order_keys(csgd_t dd, DevScalars *sc)
{
    const int nn = min(sc->n_nodes, dd.node_cap);
    for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < nn; id += gridDim.x * blockDim.x) {
        NodeLink l = dd.link[id];
        unsigned long long k;
        if (l.parent < 0) {
            k = 0ull;
        } else {
            int s0 = dd.minidx[id].x;
            int t1 = dd.minidx[l.parent].y;
            int kc = max(s0, t1);
            k = ((unsigned long long)(kc + 1) << 8) | ((unsigned long long)l.level << 1) |
                (s0 == kc ? 1ull : 0ull);
        }
        dd.ord_key[id] = k;
        dd.ord_id[id] = id;
    }
}

__global__ void k_rank(csgd_t dd, DevScalars *sc)
{
    const int nn = min(sc->n_nodes, dd.node_cap);
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nn; r += gridDim.x * blockDim.x)
        dd.rank[dd.ord_id[r]] = r;
}

// Pool records in the reference's numbering, written to dst (device memory or
// a caller's mapped host array of `capacity` cells; a larger tree is refused).
__global__ void k_export(csgd_t dd, DevScalars *sc, OctreeNode *__restrict__ dst, int capacity)
{
    const int nn = min(sc->n_nodes, dd.node_cap);
    if (nn > capacity) {
        if (blockIdx.x == 0 && threadIdx.x == 0)
            dev_fail(sc, CSG_ERR_NODE_CAPACITY);
        return;
    }
    for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < nn; id += gridDim.x * blockDim.x) {
        NodeW64 w = dd.w64[id];
        double4_32a g = dd.geo[id];
        OctreeNode o;
        o.cx = w.cx;
        o.cy = w.cy;
        o.cz = w.cz;
        o.total_mass = w.m;
        o.center_x = g.x;
        o.center_y = g.y;
        o.center_z = g.z;
        o.half_size = g.w;
        o.body_index = w.body;
        for (int q = 0; q < 8; q++) {
            int c = dd.child[8 * (size_t)id + q];
            o.children[q] = (c >= 0) ? dd.rank[c] : -1;
        }
        dst[dd.rank[id]] = o;
    }
}

// Streams the exported records (nn cells, nn read on the device) from the
// device staging array to a caller's mapped host array in address order:
// 16-byte words when both ends allow, 8-byte words otherwise.
__global__ void k_pool_out(const OctreeNode *__restrict__ src, OctreeNode *__restrict__ dst,
                           const DevScalars *__restrict__ sc, int capacity, int node_cap)
{
    const int nn = min(sc->n_nodes, node_cap);
    if (nn > capacity)
        return; // refused by k_export
    const size_t bytes = sizeof(OctreeNode) * (size_t)nn;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if ((((size_t)src | (size_t)dst) & 15) == 0) {
        const size_t n16 = bytes / 16;
        const int4 *s4 = (const int4 *)src;
        int4 *d4 = (int4 *)dst;
        for (size_t i = t0; i < n16; i += stride)
            d4[i] = s4[i];
        if (t0 == 0 && (bytes & 15)) // OctreeNode is 8-byte aligned: at most one tail word
            ((unsigned long long *)dst)[bytes / 8 - 1] = ((const unsigned long long *)src)[bytes / 8 - 1];
    } else {
        const size_t n8 = bytes / 8;
        const unsigned long long *s8 = (const unsigned long long *)src;
        unsigned long long *d8 = (unsigned long long *)dst;
        for (size_t i = t0; i < n8; i += stride)
            d8[i] = s8[i];
    }
}

// ---- import of a caller pool ---------------------------------------------
// parent links, subtree sizes (bottom-up), preorder ids (walk up summing the
// sizes of earlier siblings), then the walk/SPH records in preorder.

constexpr int IMPORT_MAX_DEPTH = 4096;

__global__ void k_imp_links(csgd_t dd, DevScalars *sc, int nn, int root, int *__restrict__ par,
                            int *__restrict__ slot)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn)
        return;
    const OctreeNode &o = dd.pool[i];
    int nc = 0;
    for (int q = 0; q < 8; q++) {
        int c = o.children[q];
        if (c < 0)
            continue;
        if (c >= nn || c == root) {
            dev_fail(sc, CSG_ERR_BAD_POOL);
            continue;
        }
        if (atomicCAS(&par[c], -1, i) != -1) {
            dev_fail(sc, CSG_ERR_BAD_POOL);
            continue;
        }
        slot[c] = q;
        nc++;
    }
    dd.nchild[i] = nc;
    dd.ticket[i] = 0;
}

__global__ void k_imp_sizes(csgd_t dd, DevScalars *sc, int nn, const int *__restrict__ par,
                            int *__restrict__ size)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn || dd.nchild[i] != 0)
        return;
    int node = i, s = 1, steps = 0;
    while (true) {
        size[node] = s;
        int p = par[node];
        if (p < 0)
            break;
        if (++steps > IMPORT_MAX_DEPTH) {
            dev_fail(sc, CSG_ERR_BAD_POOL);
            break;
        }
        __threadfence();
        int t = atomicAdd(&dd.ticket[p], 1);
        if (t != dd.nchild[p] - 1)
            break;
        __threadfence();
        s = 1;
        for (int q = 0; q < 8; q++) {
            int c = dd.pool[p].children[q];
            if (c >= 0)
                s += __ldcg(&size[c]);
        }
        node = p;
    }
}

__global__ void k_imp_write(csgd_t dd, DevScalars *sc, int nn, int root,
                            const int *__restrict__ par, const int *__restrict__ slot,
                            const int *__restrict__ size)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn || sc->err != 0)
        return; // links or sizes already found the pool is not a tree
    // preorder id = sum over the path of (1 + sizes of earlier siblings)
    int id = 0, depth = 0, node = i;
    while (node != root) {
        int p = par[node];
        if (p < 0)
            return; // not reachable from root: not part of the tree
        if (++depth > IMPORT_MAX_DEPTH) {
            dev_fail(sc, CSG_ERR_BAD_POOL);
            return;
        }
        int off = 1;
        for (int q = 0; q < slot[node]; q++) {
            int c = dd.pool[p].children[q];
            if (c >= 0)
                off += size[c];
        }
        id += off;
        node = p;
    }
    if (i == root)
        sc->n_nodes = size[root];
    if (id < 0 || id >= dd.node_cap) {
        dev_fail(sc, CSG_ERR_NODE_CAPACITY);
        return;
    }
    const OctreeNode &o = dd.pool[i];
    double s = 2.0 * o.half_size;
    NodeW64 w;
    w.cx = o.cx;
    w.cy = o.cy;
    w.cz = o.cz;
    w.m = o.total_mass;
    w.s2 = s * s;
    w.next = id + size[i];
    w.body = o.body_index >= 0 ? o.body_index : -1;
    dd.w64[id] = w;
    NodeW32 v;
    v.cx = (float)o.cx;
    v.cy = (float)o.cy;
    v.cz = (float)o.cz;
    v.lx = (float)(o.cx - (double)v.cx);
    v.ly = (float)(o.cy - (double)v.cy);
    v.lz = (float)(o.cz - (double)v.cz);
    v.m = (float)o.total_mass;
    v.next = w.next;
    v.body = w.body;
    v.s2 = (float)w.s2;
    v.s = (float)s;
    v.pad = 0.0f;
    dd.w32[id] = v;
    dd.geo[id] = make_double4_32a(o.center_x, o.center_y, o.center_z, o.half_size);
    write_s32(dd, id, o.center_x, o.center_y, o.center_z, o.half_size, w.body, w.next);
    dd.link[id] = NodeLink{-1, depth, -1, 0};
}

} // namespace

// ---- host side -------------------------------------------------------------

// Steps 1-3: root cube, keys, sorted order of the alive bodies (n_alive).
// Sort key of the system pass: the system of each key-sorted body (dead
// bodies, already last, get the largest value).
__global__ void k_gal_keys(const DevScalars *sc, const int *__restrict__ perm,
                           const int *__restrict__ gid, unsigned long long *__restrict__ gk,
                           int *__restrict__ idx, int n, int n_gal)
{
    pdl_enter();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n)
        return;
    gk[p] = (p < sc->n_alive) ? (unsigned long long)gid[perm[p]] : (unsigned long long)n_gal;
    idx[p] = p;
}

__global__ void k_gather_sorted(const int *__restrict__ idx,
                                const unsigned long long *__restrict__ key,
                                const int *__restrict__ perm, unsigned long long *__restrict__ key2,
                                int *__restrict__ perm2, int n)
{
    pdl_enter();
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n)
        return;
    const int p = idx[q];
    key2[q] = key[p];
    perm2[q] = perm[p];
}

// Steps 1-3: root cubes, keys, sorted order of the alive bodies (n_alive),
// by (system, key) for a forest, and each sorted position's system.
static int order_bodies(csgd_t *d)
{
    const int n = d->n;
    cudaStream_t s = d->stream;
    DevScalars *sc = d->sc;
    const int B = 256;
    const int G = d->n_gal;
    csgd_build_mark(d, 0);
    csgd_launch(d, k_reset, 1, 256, s, sc, d->roots, G);
    // few blocks: each warp flushes its running box with atomics on the same
    // words, so fewer warps contend less (4 blocks per SM keep HBM busy)
    int gb = min(csgd_grid(n, B), 4 * d->num_sms);
    csgd_launch(d, k_bbox, gb > 0 ? gb : 1, B, s, d->x, d->y, d->z, d->m, d->gid, n, d->roots, sc);
    csgd_launch(d, k_root, 1, 256, s, sc, d->roots, G);
    if (n > 0)
        csgd_launch(d, k_keys, csgd_grid(n, B), B, s, d->x, d->y, d->z, d->m, d->gid, n, sc, d->roots, d->key, d->perm);
    csgd_build_mark(d, 1);
    int rc = csg_radix_sort(d, d->key, d->perm, d->key_alt, d->perm_alt, n, 64);
    if (rc)
        return rc;
    if (G > 1 && n > 1) {
        // stable pass on the system id: order (system, key)
        const int g = csgd_grid(n, B);
        csgd_launch(d, k_gal_keys, g, B, s, sc, d->perm, d->gid, d->ord_key, d->ord_id, n, G);
        int bits = 1; // system ids 0..G (G marks dead bodies)
        while (bits < 31 && (1 << bits) <= G)
            bits++;
        rc = csg_radix_sort(d, d->ord_key, d->ord_id, d->ord_key_alt, d->ord_id_alt, n, bits);
        if (rc)
            return rc;
        csgd_launch(d, k_gather_sorted, g, B, s, d->ord_id, d->key, d->perm, d->key_alt, d->perm_alt, n);
        // back into (key, perm): the buffers keep their roles, so a captured
        // substep and direct launches always agree on where the order is
        cudaMemcpyAsync(d->key, d->key_alt, sizeof(unsigned long long) * (size_t)n,
                        cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(d->perm, d->perm_alt, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    }
    csgd_launch(d, k_sgid, csgd_grid(n > 0 ? n : 1, B), B, s, sc, d->perm, d->gid, d->sgid, n);
    return csgd_check(d, cudaGetLastError());
}

// Threads for the grid-stride kernels over cells.
static long long cell_threads(const csgd_t *d)
{
    const long long t = 2LL * d->n + 64;
    return t < d->node_cap ? t : d->node_cap;
}

extern "C" int csgd_build_tree(csgd_t *d, int geometry)
{
    const int n = d->n;
    cudaStream_t s = d->stream;
    DevScalars *sc = d->sc;
    const int B = 256;
    int rc = geometry ? csgd_ensure_tree_extras(d, 1, 0) : CSG_OK;
    if (!rc)
        rc = order_bodies(d);
    if (rc)
        return rc;
    const int g = csgd_grid(n > 0 ? n : 1, B);
    csgd_build_mark(d, 2);
    csgd_launch(d, k_deep_mark, g, B, s, d->x, d->y, d->z, sc, d->roots, d->key, d->sgid, d->perm, d->ext);
    csgd_launch(d, k_deep_sort, g, B, s, sc, d->key, d->sgid, d->perm, d->ext);
    csgd_launch(d, k_count, g, B, s, sc, d->key, d->ext, d->sgid, d->lcp, d->cnt);
    rc = csg_scan_exclusive(d, d->cnt, d->base, n, &sc->n_alive);
    if (rc)
        return rc;
    // d->cnt (the counts, consumed by the scan) now holds each position's leaf
    const int gn = csgd_grid(cell_threads(d), B); // >= cells and >= positions
    csgd_launch(d, k_nodes, gn, B, s, *d, sc, d->roots, d->key, d->ext, d->sgid, d->lcp, d->base, d->perm, d->cnt);
    csgd_launch(d, k_link, gn, B, s, *d, sc, d->key, d->ext);
    csgd_build_mark(d, 3);
    if (d->export_order)
        csgd_launch(d, k_moments<true>, gn, B, s, *d, sc, d->x, d->y, d->z, d->m, d->perm);
    else
        csgd_launch(d, k_moments<false>, gn, B, s, *d, sc, d->x, d->y, d->z, d->m, d->perm);
    csgd_launch(d, k_moments_norm, gn, B, s, *d, sc, d->x, d->y, d->z);
    d->minidx_valid = d->export_order;
    csgd_build_mark(d, 4);
    csgd_launch(d, k_tasks, min(d->n_gal, 152), 256, s, sc, d->roots, d->n_gal, d->base, d->tasks, d->task_cap, 0);
    d->geometry_valid = 0;
    d->imported = 0;
    d->gas_valid = 0;
    if (geometry) {
        csgd_launch(d, k_geometry, gn, B, s, *d, sc, d->roots, d->key, d->ext, d->sgid);
        d->geometry_valid = 1;
    }
    csgd_build_mark(d, 5);
    return csgd_check(d, cudaGetLastError());
}

// Export without a host round trip: the cell count is read on the device
// (order keys, sort, ranks and records are sized for `capacity` cells).
// Needs the export order (minidx) of the current tree.
extern "C" int csgd_export_to(csgd_t *d, OctreeNode *dst, int capacity)
{
    if (d->n_gal > 1) // one system only (see csgd_set_systems)
        return CSG_ERR_UNSUPPORTED;
    if (!d->minidx_valid || !dst || capacity < 1)
        return CSG_ERR_BAD_ARG;
    cudaStream_t s = d->stream;
    DevScalars *sc = d->sc;
    const int B = 256;
    if (!d->geometry_valid) {
        const int gn = csgd_grid(cell_threads(d), B);
        { k_geometry<<<gn, B, 0, s>>>(*d, sc, d->roots, d->key, d->ext, d->sgid); d->launches++; }
        d->geometry_valid = 1;
    }
    if (dst != d->pool && !d->pool)
        return CSG_ERR_BAD_ARG; // staging not allocated (csgd_ensure_tree_extras)
    const int bound = capacity < d->node_cap ? capacity : d->node_cap;
    const long long cells = cell_threads(d); // the kernels stride beyond it
    const int g = csgd_grid(cells < bound ? cells : bound, B);
    { k_order_keys<<<g, B, 0, s>>>(*d, sc); d->launches++; }
    int rc = csg_radix_sort(d, d->ord_key, d->ord_id, d->ord_key_alt, d->ord_id_alt, bound, 40,
                            &sc->n_nodes);
    if (rc)
        return rc;
    { k_rank<<<g, B, 0, s>>>(*d, sc); d->launches++; }
    if (dst == d->pool) {
        { k_export<<<g, B, 0, s>>>(*d, sc, dst, capacity); d->launches++; }
    } else { // records land in rank order: stage them, then stream them out in address order
        { k_export<<<g, B, 0, s>>>(*d, sc, d->pool, capacity); d->launches++; }
        // stores to host memory do not wait for completion: a few warps per
        // SM keep the link busy and leave the walk its warp slots
        { k_pool_out<<<d->num_sms, 128, 0, s>>>(d->pool, dst, sc, capacity, d->node_cap); d->launches++; }
    }
    return csgd_check(d, cudaGetLastError());
}

extern "C" int csgd_export_pool(csgd_t *d, OctreeNode *pool, int capacity, int *pool_size_out)
{
    if (d->n_gal > 1) // one system only (see csgd_set_systems)
        return CSG_ERR_UNSUPPORTED;
    int erc = csgd_ensure_tree_extras(d, 1, 1);
    if (erc)
        return erc;
    if (!d->minidx_valid) { // built without the export order: rebuild (same tree) with it
        const int saved = d->export_order;
        d->export_order = 1;
        erc = csgd_build_tree(d, 1);
        d->export_order = saved;
        if (erc)
            return erc;
    }
    // a caller's mapped (pinned) host array takes the records directly
    OctreeNode *mapped = (OctreeNode *)csgd_host_view(pool);
    const int cap = mapped ? capacity : (capacity < d->node_cap ? capacity : d->node_cap);
    int rc = csgd_export_to(d, mapped ? mapped : d->pool, cap);
    if (!rc)
        rc = csgd_node_count(d, pool_size_out); // reports a refused export
    if (rc || mapped)
        return rc;
    const int nn = *pool_size_out;
    cudaMemcpyAsync(pool, d->pool, sizeof(OctreeNode) * (size_t)nn, cudaMemcpyDeviceToHost,
                    d->stream);
    return csgd_sync(d);
}

extern "C" int csgd_import_pool(csgd_t *d, const OctreeNode *pool, int n_nodes, int root)
{
    if (d->n_gal > 1) { // one system only (see csgd_set_systems)
        return CSG_ERR_UNSUPPORTED;
    }
    if (n_nodes <= 0 || n_nodes > d->node_cap || root < 0 || root >= n_nodes) {
        return CSG_ERR_BAD_ARG;
    }
    cudaStream_t s = d->stream;
    DevScalars *sc = d->sc;
    const int B = 256;
    int erc = csgd_ensure_tree_extras(d, 1, 1);
    if (erc)
        return erc;
    // The walks take bodies in key order (neighbours share a warp): order the
    // alive bodies as a build would, then replace the cells by the pool's.
    int rc = order_bodies(d);
    if (rc)
        return rc;
    // scratch: par, slot, size in the (unused here) sort/order buffers
    int *par = d->ord_id, *slot = d->ord_id_alt, *size = d->rank;
    cudaMemcpyAsync(d->pool, pool, sizeof(OctreeNode) * (size_t)n_nodes, cudaMemcpyHostToDevice,
                    s);
    cudaMemsetAsync(par, 0xff, sizeof(int) * (size_t)n_nodes, s);
    const int g = csgd_grid(n_nodes, B);
    { k_imp_links<<<g, B, 0, s>>>(*d, sc, n_nodes, root, par, slot); d->launches++; }
    { k_imp_sizes<<<g, B, 0, s>>>(*d, sc, n_nodes, par, size); d->launches++; }
    { k_imp_write<<<g, B, 0, s>>>(*d, sc, n_nodes, root, par, slot, size); d->launches++; }
    { k_tasks<<<1, 256, 0, s>>>(sc, d->roots, 1, d->base, d->tasks, d->task_cap, 1); d->launches++; }
    d->geometry_valid = 1;
    d->imported = 1;
    d->gas_valid = 0;
    d->minidx_valid = 0;
    return csgd_check(d, cudaGetLastError());
}
