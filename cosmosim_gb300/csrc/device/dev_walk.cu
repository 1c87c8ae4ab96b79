// dev_walk.cu — Barnes-Hut gravity walks (reference src/octree.c:171-234).
//
// Both walks give every body exactly the reference's interaction set: the
// cells it accepts by the monopole test (s*s)/d^2 < theta^2 with d^2 > 0, or
// reaches as leaves other than itself, in depth-first octant order.
//
// Traversal: one warp walks the preorder tree for 32 bodies that are
// neighbours in key order. The warp keeps one cursor; each lane keeps a single
// index `skip` below which it sleeps (it accepted an ancestor or the cell's
// subtree does not concern it). At a cell, active lanes take leaves, accept or
// ask to open; the cursor moves to id+1 (first child) if any active lane
// opens, else to the cell's `next`. Lanes that accepted the cell sleep until
// `next`. No stack, no divergent descent, per-lane depth-first order kept.
// The next 32 cells in preorder are staged per warp in shared memory with one
// coalesced load, and re-staged only when the cursor leaves that window.
//
// FP64 walk: the drop-in precision (k_walk64ws). Openings decided as in the
//   FP32 walk (equal to the reference's FP64 rounding); interactions queued
//   and evaluated densely in FP64 by a second warp per task, with 1/r^3 from
//   an FP32 rsqrt seed by integer arithmetic (one rounding), summed per child
//   subtree of the root as the FP32 walk does; small systems split the same
//   way (k_walk64ws_units), with the same bits. k_walk64_exact instead
//   uses the reference's own operation sequence per step (1/(r2*sqrt(r2)),
//   no fused multiply-add) — bit-identical results on the reference's own
//   tree; used by parity tests.
// FP32-mixed walk: positions and centres as float hi/lo pairs (differences
//   keep ~48 bits), rsqrt/products in FP32, Kahan-compensated FP32 sums per
//   body and per child subtree of the root, added in FP64. Openings within the
//   FP32 error band of the threshold are decided in FP64, so the interaction
//   set equals the FP64 walk's. Systems with few tasks for the GPU are walked
//   by eight warps per task, one per root child (k_walk32_units), with the
//   same bits as one warp per task (k_walk32).
#include "dev_internal.cuh"

namespace {

struct WalkArgs {
    const int *perm;
    const double *x, *y, *z;
    const NodeW64 *w64;
    const NodeW32 *w32;
    const WalkTask *tasks;
    const DevRoot *roots;
    DevScalars *sc;
    double *ax, *ay, *az;
    double G, eps2, theta2, t2lo, t2hi;
    float Gf, eps2f;
    // FP32 opening test: accept when s^2 acc_k < d^2, open when s^2 opn_k > d^2
    // (acc_k, opn_k = (1 +- g) / theta^2); in between, |theta^2 d^2 - s^2| is
    // inside the FP32 error band g s^2 and the FP64 test decides
    float acc_k, opn_k;
    int node_cap;
    int group; // 0: one warp per task; g > 0: take g tasks at a time from a counter
    int wait_polls; // producer/consumer waits give up after this many polls
    double *part;   // split walks: segment partials, part[(3 * k + d) * pstride + body]
    long long pstride;
    // FP64: systems of at most split_max bodies are walked split (sys_n[gal]
    // bodies each in an ensemble, n_bodies for one system); the whole-task
    // walk leaves them out when skip_small is set
    const int *sys_n;
    int n_bodies, split_max, skip_small;
};

// Work distribution shared by the walks. A task is up to 32 consecutive
// sorted bodies of one system. With group == 0 warp w of the grid walks task
// w; otherwise (persistent launch, a few blocks per SM) each warp takes the
// next `group` tasks from sc->task_next until none are left. Every take
// advances the counter, so the loop ends after at most n_tasks/group + 1
// takes per warp.
__device__ __forceinline__ int take_tasks(const WalkArgs &a)
{
    int v = 0;
    if ((threadIdx.x & 31) == 0)
        v = atomicAdd(&a.sc->task_next, a.group);
    return __shfl_sync(0xffffffffu, v, 0);
}

// Resident warps per SM the register allocation is sized for: 32 (64
// registers a thread) for one-warp-per-task launches, 24 (up to 85) for
// persistent ones, whose task loop state would otherwise spill.
constexpr int persist_min_blocks(int warps, bool persist) { return (persist ? 24 : 32) / warps; }

// Walk statistics: interactions, warp steps and lane-steps of lanes that
// had not finished (lane utilisation = active / (32 steps)).
struct WalkStats {
    unsigned long long hits = 0, steps = 0, active = 0;
};

// Validated task: bodies [pos0, pos0+count) and the system's cells [root, end).
struct TaskRange {
    int pos0, count, root, end;
};

template <int WARPS, bool PERSIST, typename Fn>
__device__ __forceinline__ void for_each_task(const WalkArgs &a, Fn fn)
{
    const int nn = a.sc->n_nodes;
    if (nn > a.node_cap || nn < 1)
        return; // no valid tree (capacity error already recorded)
    const int nt = a.sc->n_tasks;
    auto run = [&](int t) {
        const WalkTask w = a.tasks[t];
        const DevRoot &r = a.roots[w.gal];
        const TaskRange tr{w.pos0, w.count, r.root, r.end};
        if (tr.root < 0 || tr.end > nn || tr.root >= tr.end)
            dev_fail(a.sc, CSG_ERR_WALK_LIMIT);
        else
            fn(tr);
    };
    if (!PERSIST) {
        const int t = blockIdx.x * WARPS + (threadIdx.x >> 5);
        if (t < nt)
            run(t);
        return;
    }
    int t = take_tasks(a), tend = t + a.group;
    while (t < nt) {
        run(t);
        if (++t >= tend) {
            t = take_tasks(a);
            tend = t + a.group;
        }
    }
}

// Reference opening decision fl(s2/d2) < theta2 (src/octree.c:202-203),
// without a division unless s2 is within 2^-50 of theta2*d2.
__device__ __forceinline__ bool accept64(double s2, double d2, const WalkArgs &a)
{
    if (!(d2 > 0.0))
        return false;
    if (s2 < a.t2lo * d2)
        return true;
    if (s2 > a.t2hi * d2)
        return false;
    return __ddiv_rn(s2, d2) < a.theta2;
}

// The reference's own FP64 operation sequence per step, one warp per task,
// no fused multiply-add: bit-identical accelerations on the reference's tree.
template <bool STATS>
__device__ __forceinline__ void walk64_exact_task(const WalkArgs &a, NodeW64 *win,
                                                  const TaskRange &tr, WalkStats &st)
{
    const int lane = threadIdx.x & 31;
    const int nn = tr.end;
    const bool valid = lane < tr.count;
    const int me = valid ? a.perm[tr.pos0 + lane] : -1;
    const double px = valid ? a.x[me] : 0.0, py = valid ? a.y[me] : 0.0,
                 pz = valid ? a.z[me] : 0.0;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    int skip = valid ? 0 : INT_MAX;
    int cur = tr.root, wbase = INT_MIN / 2;
    while (cur < nn) {
        if (cur - wbase >= CSG_WARP) {
            wbase = cur;
            __syncwarp();
            if (wbase + lane < nn)
                win[lane] = a.w64[wbase + lane];
            __syncwarp();
        }
        const NodeW64 c = win[cur - wbase];
        bool open = false;
        if (STATS) {
            st.steps++;
            st.active += (cur >= skip);
        }
        if (cur >= skip) {
            if (c.m == 0.0) { // empty cell: reference returns at once (src/octree.c:181-182)
                skip = c.next;
            } else {
                const double dx = __dsub_rn(c.cx, px);
                const double dy = __dsub_rn(c.cy, py);
                const double dz = __dsub_rn(c.cz, pz);
                const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)),
                                            __dmul_rn(dz, dz));
                bool take;
                if (c.body >= 0) {
                    take = (c.body != me);
                } else {
                    take = d2 > 0.0 && __ddiv_rn(c.s2, d2) < a.theta2;
                    if (take)
                        skip = c.next;
                    else
                        open = true;
                }
                if (take) {
                    const double r2 = __dadd_rn(d2, a.eps2);
                    const double inv = __ddiv_rn(1.0, __dmul_rn(r2, __dsqrt_rn(r2)));
                    const double gm = __dmul_rn(a.G, c.m);
                    sx = __dadd_rn(sx, __dmul_rn(__dmul_rn(gm, dx), inv));
                    sy = __dadd_rn(sy, __dmul_rn(__dmul_rn(gm, dy), inv));
                    sz = __dadd_rn(sz, __dmul_rn(__dmul_rn(gm, dz), inv));
                    if (STATS)
                        st.hits++;
                }
            }
        }
        const int nxt = __any_sync(0xffffffffu, open) ? cur + 1 : c.next;
        if (nxt <= cur) { // a malformed tree must not loop
            dev_fail(a.sc, CSG_ERR_WALK_LIMIT);
            break;
        }
        cur = nxt;
    }
    if (valid) {
        a.ax[me] = sx;
        a.ay[me] = sy;
        a.az[me] = sz;
    }
}

__device__ __forceinline__ void add_hits(const WalkArgs &a, const WalkStats &w)
{
    unsigned int h = __reduce_add_sync(0xffffffffu, (unsigned int)w.hits);
    unsigned int ac = __reduce_add_sync(0xffffffffu, (unsigned int)w.active);
    if ((threadIdx.x & 31) == 0) {
        if (h)
            atomicAdd(&a.sc->interactions, (unsigned long long)h);
        atomicAdd(&a.sc->walk_steps, w.steps);
        atomicAdd(&a.sc->walk_active, (unsigned long long)ac);
    }
}

template <bool STATS>
__global__ void __launch_bounds__(8 * CSG_WARP) k_walk64_exact(WalkArgs a)
{
    __shared__ NodeW64 win_all[8][CSG_WARP];
    NodeW64 *win = win_all[threadIdx.x >> 5];
    WalkStats st;
    for_each_task<8, false>(a, [&](const TaskRange &tr) { walk64_exact_task<STATS>(a, win, tr, st); });
    if (STATS)
        add_hits(a, st);
}

// m/r^3 for the queued FP64 walk without FP64 operations (the FP64 pipe is
// the walk's bottleneck on this GPU): from the FP32 rsqrt seed y0 (rel.
// error < 2^-21) by integer arithmetic (m_r3_from_seed: the series of
// (1-e)^-3/2, e = 1 - r2 y0^2, one rounding). The seed's conversion is a bit
// operation. Range checks on the exponents (2^-99 <= r2 < 2^100,
// 2^-863 <= m < 2^865) keep every integer step in range; outside them (and
// for m = 0) the plain expression.
__device__ __forceinline__ double m_inv_r3_q(double m, double r2)
{
    const long long bits = __double_as_longlong(r2);
    const long long mb = __double_as_longlong(m);
    if ((unsigned long long)((bits >> 52) - 924) <= 198ull && // sign clear, exponent 924..1122
        (unsigned long long)((mb >> 52) - 160) < 1728ull)     // sign clear, exponent 160..1887
        return m_r3_from_seed(bits, mb, rsqrtf(f32_from_f64_bits(bits)));
    return m / (r2 * sqrt(r2));
}

// ---- shared FP32 traversal -------------------------------------------------
//
// One step = one cell for the whole warp (the cell record is staged in a
// per-warp shared-memory window, see load_cell). Decisions: FP32 with the difference
// held to ~48 bits (hi/lo pairs); only when theta^2 d^2 lies within the FP32
// error band of s^2 is the reference's FP64 test redone, out of line.

__device__ __noinline__ bool decide64(const WalkArgs &a, int cur, double px, double py, double pz)
{
    const NodeW64 e = a.w64[cur];
    const double ex = e.cx - px, ey = e.cy - py, ez = e.cz - pz;
    return accept64(e.s2, ex * ex + ey * ey + ez * ez, a);
}

struct BodyPos {
    double px, py, pz;
    float hx, hy, hz, lx, ly, lz;
};

__device__ __forceinline__ BodyPos body_pos(const WalkArgs &a, int me, bool valid)
{
    BodyPos b;
    b.px = valid ? a.x[me] : 0.0;
    b.py = valid ? a.y[me] : 0.0;
    b.pz = valid ? a.z[me] : 0.0;
    b.hx = (float)b.px;
    b.hy = (float)b.py;
    b.hz = (float)b.pz;
    b.lx = (float)(b.px - (double)b.hx);
    b.ly = (float)(b.py - (double)b.hy);
    b.lz = (float)(b.pz - (double)b.hz);
    return b;
}

struct Cell {
    float4 A; // hi centre of mass, mass
    float4 B; // lo centre of mass, s^2
    int next, body;
};

// The next 32 cells in preorder are staged per warp in shared memory with one
// coalesced load and re-staged when the cursor leaves that window: the load
// latency is paid once per window instead of on every step's critical path.
__device__ __forceinline__ Cell load_cell(const WalkArgs &a, NodeW32 *win, int &wbase, int cur,
                                          int nn)
{
    if (cur - wbase >= CSG_WARP) { // warp-uniform
        const int lane = threadIdx.x & 31;
        wbase = cur;
        __syncwarp();
        if (wbase + lane < nn)
            win[lane] = a.w32[wbase + lane];
        __syncwarp();
    }
    const float4 *w = (const float4 *)(win + (cur - wbase));
    Cell c;
    c.A = w[0];
    c.B = w[1];
    const int2 nb = *(const int2 *)(w + 2);
    c.next = nb.x;
    c.body = nb.y;
    return c;
}

// Visits cells [cur, nn) of the preorder tree for the warp's 32 bodies, from
// the lane state `skip` (a lane is active at cells >= skip); calls take(cell,
// dx, dy, dz, d2, cur) (under a warp-uniform "some lane takes" branch) for
// every cell the lane interacts with, in the reference's depth-first order;
// after(cur, active) runs once per step for the whole warp. `win` caches 32
// cells from wbase (below wend, the system's end). EMPTY: cells of zero mass
// may occur (caller pools); the reference skips them with everything below.
// Returns with cur >= nn (cur = INT_MAX after a malformed tree).
template <bool EMPTY, typename Take, typename After>
__device__ __forceinline__ void walk_cells_span(const WalkArgs &a, NodeW32 *win, int &cur, int nn,
                                                int wend, int &skip, int &wbase, int me,
                                                bool valid, const BodyPos &b, Take take_fn,
                                                After after_fn)
{
    while (cur < nn) {
        const Cell c = load_cell(a, win, wbase, cur, wend);
        const bool active = cur >= skip;
        bool take = false, open = false;
        if (EMPTY && c.A.w == 0.0f && __any_sync(0xffffffffu, active)) {
            if (a.w64[cur].m == 0.0) { // empty cell (src/octree.c:181-182)
                if (active)
                    skip = c.next;
                after_fn(cur, active);
                if (c.next <= cur) {
                    dev_fail(a.sc, CSG_ERR_WALK_LIMIT);
                    cur = INT_MAX;
                    break;
                }
                cur = c.next;
                continue;
            }
        }
        const float dx = (c.A.x - b.hx) + (c.B.x - b.lx);
        const float dy = (c.A.y - b.hy) + (c.B.y - b.ly);
        const float dz = (c.A.z - b.hz) + (c.B.z - b.lz);
        const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        if (c.body >= 0) { // leaf (warp-uniform): no lane can open it, no vote
            take = active && c.body != me;
            if (__any_sync(0xffffffffu, take))
                take_fn(take, c, dx, dy, dz, d2, cur);
            after_fn(cur, active);
            if (c.next <= cur) {
                dev_fail(a.sc, CSG_ERR_WALK_LIMIT);
                cur = INT_MAX;
                break;
            }
            cur = c.next;
            continue;
        } else {
            bool acc = c.B.w * a.acc_k < d2; // implies d2 > 0
            const bool amb = active && !acc && !(c.B.w * a.opn_k > d2);
            if (amb) // rare
                acc = decide64(a, cur, b.px, b.py, b.pz);
            take = active && acc;
            open = active && !acc;
            if (take)
                skip = c.next;
        }
        if (__any_sync(0xffffffffu, take))
            take_fn(take, c, dx, dy, dz, d2, cur);
        after_fn(cur, active);
        const int nxt = __any_sync(0xffffffffu, open) ? cur + 1 : c.next;
        if (nxt <= cur) { // a malformed tree must not loop
            dev_fail(a.sc, CSG_ERR_WALK_LIMIT);
            cur = INT_MAX;
            break;
        }
        cur = nxt;
    }
}

// The whole preorder range [root, nn) of a system.
template <bool EMPTY, typename Take, typename After>
__device__ __forceinline__ void walk_cells(const WalkArgs &a, NodeW32 *win, int root, int nn,
                                           int me, bool valid, const BodyPos &b, Take take_fn,
                                           After after_fn)
{
    int skip = valid ? 0 : INT_MAX, cur = root, wbase = INT_MIN / 2;
    walk_cells_span<EMPTY>(a, win, cur, nn, nn, skip, wbase, me, valid, b, take_fn, after_fn);
}

// Segments [k0, k0 + g) of a system for the split walks (a tree built here;
// segment k is the subtree of the root's child k, the last, k == 7, running
// to the system's end): the root step (take reports root interactions only
// for k0 == 0: every unit needs the step to know which lanes go on), then the
// segments in order, between(k) before segment k > k0.
template <bool EMPTY, typename Take, typename After, typename Between>
__device__ __forceinline__ void walk_cells_segments(const WalkArgs &a, NodeW32 *win,
                                                    const TaskRange &tr, int k0, int g, int me,
                                                    bool valid, const BodyPos &b, Take take_fn,
                                                    After after_fn, Between between)
{
    int skip = valid ? 0 : INT_MAX, cur = tr.root, wbase = INT_MIN / 2;
    walk_cells_span<EMPTY>(a, win, cur, tr.root + 1, tr.end, skip, wbase, me, valid, b, take_fn,
                           after_fn);
    // cur < end: some lane opened the root
    for (int j = 0; j < k0 && cur < tr.end; j++)
        cur = min(tr.end, max(a.w32[cur].next, cur + 1));
    for (int k = k0; k < k0 + g && cur < tr.end; k++) {
        if (k > k0)
            between(k);
        const int nn = k == 7 ? tr.end : min(tr.end, max(a.w32[cur].next, cur + 1));
        walk_cells_span<EMPTY>(a, win, cur, nn, tr.end, skip, wbase, me, valid, b, take_fn,
                               after_fn);
    }
}

__device__ __forceinline__ void kahan_add(float &s, float &c, float v)
{
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}

// FP32-mixed walk: pair terms in FP32 from ~48-bit position differences,
// summed per lane in blocks (one term per warp step at most, flushed every 8
// steps for the whole warp) that are added with Kahan compensation
// (per-body compensated FP32 summation); G applied once. The step is
// branch-light: every lane computes the pair term and lanes that do not take
// the cell add zero, so the warp never splits on "take".
//
// Sums are closed into double partials: first the root's own term, then one
// per child subtree of the system's root ("segment" k < 8, in child order);
// the body's acceleration is G times the sum of the partials in that order.
// A task can so be walked by one warp (all segments in turn) or by eight
// warps (one segment each; unit 0 also takes the root's term, and 0 + root
// is the root exactly; the partials added by k_walk_sum) with the same bits.
// The launch picks by size.
constexpr int WSEGS = 8;

// A lane's body: its FP64 position and the FP32 high and low parts of it.
struct Lane32 {
    bool valid;
    int me;
    double px, py, pz;
    float hx, hy, hz, lx, ly, lz;
};

__device__ __forceinline__ Lane32 lane32(const WalkArgs &a, const TaskRange &tr)
{
    Lane32 L;
    const int lane = threadIdx.x & 31;
    L.valid = lane < tr.count;
    L.me = L.valid ? a.perm[tr.pos0 + lane] : -1;
    L.px = L.valid ? a.x[L.me] : 0.0;
    L.py = L.valid ? a.y[L.me] : 0.0;
    L.pz = L.valid ? a.z[L.me] : 0.0;
    L.hx = (float)L.px;
    L.hy = (float)L.py;
    L.hz = (float)L.pz;
    L.lx = (float)(L.px - (double)L.hx);
    L.ly = (float)(L.py - (double)L.hy);
    L.lz = (float)(L.pz - (double)L.hz);
    return L;
}

// Cells [cur, nn) in preorder from the lane state `skip` (a lane is active at
// cells >= skip); adds into the compensated sums (sx, cx) ... in blocks of up
// to 8 steps. `win` caches 32 consecutive cells from wbase (kept across
// calls; cells below wend, the system's end). Returns with cur >= nn.
template <bool STATS, bool EMPTY>
__device__ __forceinline__ void walk32_span(const WalkArgs &a, NodeW32 *win, int &cur, int nn,
                                            int wend, int &skip, int &wbase, const Lane32 &L,
                                            float &sx,
                                            float &sy, float &sz, float &cx, float &cy, float &cz,
                                            WalkStats &st)
{
    const int lane = threadIdx.x & 31;
    while (cur < nn) {
        // a block of up to 8 steps: at most one term per lane per step, then
        // one compensated add of the block (warp-uniform)
        float bx = 0.f, by = 0.f, bz = 0.f;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            if (cur >= nn)
                break;
            if (cur - wbase >= CSG_WARP) {
                wbase = cur;
                __syncwarp();
                if (wbase + lane < wend)
                    win[lane] = a.w32[wbase + lane];
                __syncwarp();
            }
            const NodeW32 c = win[cur - wbase];
            const bool active = cur >= skip;
            if (STATS) {
                st.steps++;
                st.active += active;
            }
            const float dx = (c.cx - L.hx) + (c.lx - L.lx);
            const float dy = (c.cy - L.hy) + (c.ly - L.ly);
            const float dz = (c.cz - L.hz) + (c.lz - L.lz);
            const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            bool take;
            int nxt;
            if (c.body >= 0) { // leaf (warp-uniform): nothing to open, no vote
                take = active && c.body != L.me;
                if (EMPTY && take && c.m == 0.0f && a.w64[cur].m == 0.0)
                    take = false;
                nxt = c.next;
            } else {
                bool acc, open;
                if (EMPTY && c.m == 0.0f && a.w64[cur].m == 0.0) { // empty cell of a caller pool
                    acc = false;
                    open = false;
                    if (active)
                        skip = c.next;
                } else {
                    // |theta^2 d^2 - s^2| inside the FP32 error band -> decide in FP64
                    acc = c.s2 * a.acc_k < d2; // implies d2 > 0
                    const bool amb = active && !acc && !(c.s2 * a.opn_k > d2);
                    if (amb) // rare
                        acc = decide64(a, cur, L.px, L.py, L.pz);
                    open = active && !acc;
                }
                take = active && acc;
                skip = take ? c.next : skip;
                nxt = __any_sync(0xffffffffu, open) ? cur + 1 : c.next;
            }
            const float y = rsqrtf(d2 + a.eps2f);
            const float f = take ? c.m * (y * y * y) : 0.0f;
            bx = fmaf(f, dx, bx);
            by = fmaf(f, dy, by);
            bz = fmaf(f, dz, bz);
            if (STATS)
                st.hits += take;
            // every tree built or imported here has next > id; the max keeps
            // the walk finite on any other
            cur = max(nxt, cur + 1);
        }
        kahan_add(sx, cx, bx);
        kahan_add(sy, cy, by);
        kahan_add(sz, cz, bz);
    }
}

// End of the subtree starting at cell c (c < end), kept inside [c + 1, end].
__device__ __forceinline__ int subtree_end(const WalkArgs &a, int c, int end)
{
    return min(end, max(a.w32[c].next, c + 1));
}

// The whole task by one warp: the root, then each child subtree of the root
// as a segment, every one closed into the double sum g. Trees built here give
// the root at most eight children; a caller's pool walked here (never split)
// may give more, each a segment of its own.
template <bool STATS, bool EMPTY>
__device__ __forceinline__ void walk32_task(const WalkArgs &a, NodeW32 *win, const TaskRange &tr,
                                            WalkStats &st)
{
    const int lane = threadIdx.x & 31;
    // the double sums live in shared memory right after the window
    // (g[d * 32 + lane]): registers stay with the traversal
    double *g = reinterpret_cast<double *>(win + CSG_WARP);
    const Lane32 L = lane32(a, tr);
    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    g[lane] = 0.0;
    g[CSG_WARP + lane] = 0.0;
    g[2 * CSG_WARP + lane] = 0.0;
    int skip = L.valid ? 0 : INT_MAX, wbase = INT_MIN / 2, cur = tr.root, nn = tr.root + 1;
    for (;;) {
        walk32_span<STATS, EMPTY>(a, win, cur, nn, tr.end, skip, wbase, L, sx, sy, sz, cx, cy, cz,
                                  st);
        g[lane] += (double)sx - (double)cx;
        g[CSG_WARP + lane] += (double)sy - (double)cy;
        g[2 * CSG_WARP + lane] += (double)sz - (double)cz;
        sx = sy = sz = cx = cy = cz = 0.f;
        // after the root, cur < end says that some lane opened it
        if (cur >= tr.end)
            break;
        nn = subtree_end(a, cur, tr.end);
    }
    if (L.valid) {
        a.ax[L.me] = a.G * g[lane];
        a.ay[L.me] = a.G * g[CSG_WARP + lane];
        a.az[L.me] = a.G * g[2 * CSG_WARP + lane];
    }
}

// Segment k < 8 of a task by one warp (a tree built here); its partial into
// part[k] (3 x pstride), segment 0's with the root's term added first (as the
// whole walk adds them: 0 + root is the root exactly). The root step runs for
// every k: it sets which lanes go on. The root's partial waits in shared
// memory after the window, as in the whole walk.
template <bool STATS, bool EMPTY>
__device__ __forceinline__ void walk32_unit(const WalkArgs &a, NodeW32 *win, const TaskRange &tr,
                                            int k, double *part, long long pstride, WalkStats &st)
{
    const int lane = threadIdx.x & 31;
    double *q = reinterpret_cast<double *>(win + CSG_WARP);
    const Lane32 L = lane32(a, tr);
    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    int skip = L.valid ? 0 : INT_MAX, wbase = INT_MIN / 2, cur = tr.root, nn = tr.root + 1;
    for (bool root = true;; root = false) {
        walk32_span<STATS, EMPTY>(a, win, cur, nn, tr.end, skip, wbase, L, sx, sy, sz, cx, cy, cz,
                                  st);
        if (!root)
            break;
        const bool keep = k == 0;
        q[lane] = keep ? (double)sx - (double)cx : 0.0;
        q[CSG_WARP + lane] = keep ? (double)sy - (double)cy : 0.0;
        q[2 * CSG_WARP + lane] = keep ? (double)sz - (double)cz : 0.0;
        sx = sy = sz = cx = cy = cz = 0.f;
        for (int j = 0; j < k && cur < tr.end; j++)
            cur = subtree_end(a, cur, tr.end);
        if (cur >= tr.end)
            break;
        nn = subtree_end(a, cur, tr.end);
    }
    if (L.valid) {
        part[(3 * k + 0) * pstride + L.me] = q[lane] + ((double)sx - (double)cx);
        part[(3 * k + 1) * pstride + L.me] = q[CSG_WARP + lane] + ((double)sy - (double)cy);
        part[(3 * k + 2) * pstride + L.me] = q[2 * CSG_WARP + lane] + ((double)sz - (double)cz);
    }
}

// a = G (part[0] + ... + part[7]) for every live body, in child order: the
// whole walk's own sum.
// With sys_n (an ensemble's FP64 walk): only bodies of systems of at most
// split_max bodies, the ones the split walk covered.
__global__ void k_walk_sum(const double *__restrict__ part, long long pstride,
                             const double *__restrict__ m, int n, double G, double *ax,
                             double *ay, double *az, const int *__restrict__ gid,
                             const int *__restrict__ sys_n, int split_max)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || m[i] <= 0.0)
        return;
    if (sys_n && sys_n[gid[i]] > split_max)
        return; // walked whole, written by that walk
    double s[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int k = 0; k < WSEGS; k++)
#pragma unroll
        for (int d = 0; d < 3; d++)
            s[d] += part[(3 * k + d) * pstride + i];
    ax[i] = G * s[0];
    ay[i] = G * s[1];
    az[i] = G * s[2];
}

// One warp per (task, segment): unit u walks segment u % 8 of task u / 8.
__global__ void __launch_bounds__(4 * CSG_WARP, 8) k_walk32_units(WalkArgs a, double *part,
                                                                   long long pstride)
{
    constexpr int GCELLS = (3 * CSG_WARP * sizeof(double) + sizeof(NodeW32) - 1) / sizeof(NodeW32);
    __shared__ NodeW32 win_all[4][CSG_WARP + GCELLS];
    NodeW32 *win = win_all[threadIdx.x >> 5];
    WalkStats st;
    const int nn = a.sc->n_nodes;
    if (nn > a.node_cap || nn < 1)
        return;
    const int u = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (u >= a.sc->n_tasks * WSEGS)
        return;
    const WalkTask w = a.tasks[u / WSEGS];
    const DevRoot &r = a.roots[w.gal];
    const TaskRange tr{w.pos0, w.count, r.root, r.end};
    if (tr.root < 0 || tr.end > nn || tr.root >= tr.end)
        dev_fail(a.sc, CSG_ERR_WALK_LIMIT);
    else
        walk32_unit<false, false>(a, win, tr, u % WSEGS, part, pstride, st);
}

template <bool STATS, bool EMPTY, int WARPS, bool PERSIST>
__global__ void __launch_bounds__(WARPS * CSG_WARP, persist_min_blocks(WARPS, PERSIST)) k_walk32(WalkArgs a)
{
    // per warp: the cell window, then the double sums (3 x 32) right after it
    constexpr int GCELLS = (3 * CSG_WARP * sizeof(double) + sizeof(NodeW32) - 1) / sizeof(NodeW32);
    __shared__ NodeW32 win_all[WARPS][CSG_WARP + GCELLS];
    NodeW32 *win = win_all[threadIdx.x >> 5];
    WalkStats st;
    for_each_task<WARPS, PERSIST>(a, [&](const TaskRange &tr) { walk32_task<STATS, EMPTY>(a, win, tr, st); });
    if (STATS)
        add_hits(a, st);
}

// FP64 evaluation: accepted cells are queued per lane in shared memory and
// evaluated in FP64 in batches where every lane has work, in the order they
// were accepted (the reference's depth-first order). The FP64 pipe then does
// useful work on (almost) every lane instead of once per traversal step for
// the few lanes that interact at that step.

// Loads queued entry s of the lane (its cell's centre of mass and mass), or
// zeros when s >= count (no queue read, no cell read). With MARK a negative
// entry is a segment marker (mk; nothing loaded).
template <int Q64, bool MARK>
__device__ __forceinline__ void q64_load(const WalkArgs &a, const int *q, int lane, int head, int s,
                                         int count, double2 &p01, double2 &p23, bool &mk)
{
    p01 = make_double2(0.0, 0.0);
    p23 = p01;
    mk = false;
    if (s < count) {
        const int c = q[((head + s) & (Q64 - 1)) * CSG_WARP + lane];
        if (MARK)
            mk = c < 0;
        if (!MARK || !mk) {
            p01 = __ldg((const double2 *)&a.w64[c]);     // cx, cy
            p23 = __ldg((const double2 *)&a.w64[c] + 1); // cz, m
        }
    }
}

__device__ __forceinline__ void q64_term(const WalkArgs &a, const double2 &p01, const double2 &p23,
                                         double px, double py, double pz, double &sx, double &sy,
                                         double &sz)
{
    const double dx = p01.x - px, dy = p01.y - py, dz = p23.x - pz;
    const double r2 = fma(dx, dx, fma(dy, dy, fma(dz, dz, a.eps2)));
    const double f = m_inv_r3_q(p23.y, r2);
    sx = fma(f, dx, sx);
    sy = fma(f, dy, sy);
    sz = fma(f, dz, sz);
}

// A unit's segment partials: part[(3 * k + d) * pstride + body].
__device__ __forceinline__ void put_partial(const WalkArgs &a, int k, int me, double sx, double sy,
                                            double sz)
{
    a.part[(3 * k + 0) * a.pstride + me] = sx;
    a.part[(3 * k + 1) * a.pstride + me] = sy;
    a.part[(3 * k + 2) * a.pstride + me] = sz;
}

// Evaluates the lane's next `count` queued entries (count >= 0; lanes without
// a body pass 0 and never read their queue), two at a time in queue order.
// The next two cells' loads are in flight while the current two are
// evaluated (few consumer warps per SM at small N, each waiting on its
// loads). MARK: a marker closes segment kc (its partial written, the sum
// restarted).
template <int Q64, bool MARK>
__device__ __forceinline__ void q64_eval(const WalkArgs &a, const int *q, int lane, int &head,
                                         int count, double px, double py, double pz,
                                         double &sx, double &sy, double &sz, int me, int &kc)
{
    count = max(count, 0);
    const int kmax = (int)__reduce_max_sync(0xffffffffu, (unsigned)count);
    double2 a01, a23, b01, b23;
    bool ma, mb;
    q64_load<Q64, MARK>(a, q, lane, head, 0, count, a01, a23, ma);
    q64_load<Q64, MARK>(a, q, lane, head, 1, count, b01, b23, mb);
    for (int s = 0; s < kmax; s += 2) {
        double2 c01, c23, d01, d23;
        bool mc, md;
        q64_load<Q64, MARK>(a, q, lane, head, s + 2, count, c01, c23, mc);
        q64_load<Q64, MARK>(a, q, lane, head, s + 3, count, d01, d23, md);
        if (s < count) {
            if (MARK && ma) { // rare
                put_partial(a, kc++, me, sx, sy, sz);
                sx = sy = sz = 0.0;
            } else {
                q64_term(a, a01, a23, px, py, pz, sx, sy, sz);
            }
        }
        if (s + 1 < count) {
            if (MARK && mb) {
                put_partial(a, kc++, me, sx, sy, sz);
                sx = sy = sz = 0.0;
            } else {
                q64_term(a, b01, b23, px, py, pz, sx, sy, sz);
            }
        }
        a01 = c01;
        a23 = c23;
        b01 = d01;
        b23 = d23;
        ma = mc;
        mb = md;
    }
    head += count;
}

// FP64 walk, producer/consumer form. Each task has two warps: the producer
// walks the tree (walk_cells, the FP32 decisions) and appends each lane's
// accepted cells to that lane's ring in shared memory; the consumer evaluates
// the rings in FP64, in the order the cells were accepted. The traversal
// (FP32/ALU pipes) and the evaluation (FP64 pipe) then overlap on every SM
// instead of alternating in one warp. The warps hand over through per-lane
// head and tail counters in shared memory; every wait polls with a sleep and
// gives up after a.wait_polls polls (recording CSG_ERR_DEVICE_WAIT, then both
// warps leave the task). A pair of the split form (G > 0) walks G segments
// of a task: the root step, then the subtrees of the root's children k0 ..
// k0 + G - 1, with a marker (-1) queued on every lane between two segments.
constexpr int WS_RING = 128;   // ring slots per lane (power of two)
constexpr int WS_BATCH = 8;    // dense batch the consumer waits for
constexpr int WS_PUBLISH = 4;  // the producer publishes its tails every few steps

struct WsShared {
    int ring[WS_RING * CSG_WARP]; // slot-major: ring[slot * 32 + lane]
    int tail[CSG_WARP];           // published by the producer
    int head[CSG_WARP];           // published by the consumer
    int done;                     // producer finished (tails final)
    int broken;                   // a wait gave up: both warps leave
};

__device__ __forceinline__ int ws_load(const volatile int *p) { return *p; }

template <bool STATS, bool EMPTY, int G>
__device__ __forceinline__ void ws_produce(const WalkArgs &a, NodeW32 *win, WsShared &sh,
                                           const TaskRange &tr, int k0, WalkStats &st)
{
    const int lane = threadIdx.x & 31;
    const bool valid = lane < tr.count;
    const int me = valid ? a.perm[tr.pos0 + lane] : -1;
    const BodyPos b = body_pos(a, me, valid);
    int tail = 0, head_seen = 0, steps = 0;
    bool broken = false;
    auto publish = [&]() {
        __threadfence_block(); // ring entries before the tail
        ((volatile int *)sh.tail)[lane] = tail;
    };
    // one entry on every lane that wants to push: waits (warp-uniform) for room
    // (a's fields copied out: a closure holding a reference to a would put
    // the kernel's argument block on the stack)
    const int wait_polls = a.wait_polls;
    DevScalars *const sc = a.sc;
    auto push = [&](bool want, int value) {
        bool full = want && tail - head_seen >= WS_RING;
        if (__any_sync(0xffffffffu, full)) {
            publish();
            for (int i = 0; i < wait_polls; i++) {
                head_seen = ws_load(&sh.head[lane]);
                full = want && tail - head_seen >= WS_RING;
                if (!__any_sync(0xffffffffu, full) || ws_load(&sh.broken))
                    break;
                __nanosleep(64);
            }
            __threadfence_block(); // heads read before slots are overwritten
            if (__any_sync(0xffffffffu, full)) { // gave up (or the consumer did)
                if (lane == 0) {
                    dev_fail(sc, CSG_ERR_DEVICE_WAIT);
                    ((volatile int *)&sh.broken)[0] = 1;
                }
                broken = true;
            }
        }
        if (want && !broken) {
            sh.ring[(tail & (WS_RING - 1)) * CSG_WARP + lane] = value;
            tail++;
        }
    };
    auto take_fn = [&](bool take, const Cell &, float, float, float, float, int cur) {
        if (G > 0 && k0 != 0 && cur == tr.root) // the root's terms are segment 0's
            take = false;
        push(take, cur);
        if (STATS && take && !broken)
            st.hits++;
    };
    auto after_fn = [&](int, bool active) {
        if (STATS) {
            st.steps++;
            st.active += active;
        }
        if (++steps == WS_PUBLISH) {
            steps = 0;
            publish();
        }
    };
    if (G > 0)
        walk_cells_segments<EMPTY>(a, win, tr, k0, G, me, valid, b, take_fn, after_fn,
                                   [&](int) { push(valid, -1); });
    else
        walk_cells<EMPTY>(a, win, tr.root, tr.end, me, valid, b, take_fn, after_fn);
    publish();
    __syncwarp();
    if (lane == 0)
        ((volatile int *)&sh.done)[0] = 1; // after every lane's final tail (fenced above)
}

template <int G>
__device__ __forceinline__ void ws_consume(const WalkArgs &a, WsShared &sh, const TaskRange &tr,
                                           int k0)
{
    const int lane = threadIdx.x & 31;
    const bool valid = lane < tr.count;
    const int me = valid ? a.perm[tr.pos0 + lane] : -1;
    const double px = valid ? a.x[me] : 0.0, py = valid ? a.y[me] : 0.0,
                 pz = valid ? a.z[me] : 0.0;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    int head = 0, polls = 0, kc = k0; // kc: the segment being summed (split form)
    while (true) {
        const bool done = ws_load(&sh.done) != 0; // read before the tails: they are final then
        __threadfence_block();
        const int tail = ws_load(&sh.tail[lane]);
        __threadfence_block(); // the tail before the entries it covers
        const int avail = valid ? tail - head : 0;
        const int amin = (int)__reduce_min_sync(0xffffffffu, (unsigned)(valid ? avail : INT_MAX));
        const int amax = (int)__reduce_max_sync(0xffffffffu, (unsigned)avail);
        int take = 0;
        if (amin >= WS_BATCH)
            take = amin; // dense: every lane has work
        else if (done || amax >= WS_RING - WS_BATCH)
            take = -1; // the rest (done) or relief for a lane whose ring is nearly full
        if (take != 0) {
            const int n = take > 0 ? (valid ? take : 0) : min(avail, done ? avail : WS_BATCH);
            q64_eval<WS_RING, (G > 1)>(a, sh.ring, lane, head, n, px, py, pz, sx, sy, sz, me, kc);
            __threadfence_block(); // entries read before the head is published
            ((volatile int *)sh.head)[lane] = head;
            polls = 0;
            if (done && __all_sync(0xffffffffu, !valid || head == tail))
                break;
            continue;
        }
        if (ws_load(&sh.broken))
            return;
        if (++polls >= a.wait_polls) {
            if (lane == 0) {
                dev_fail(a.sc, CSG_ERR_DEVICE_WAIT);
                ((volatile int *)&sh.broken)[0] = 1;
            }
            return;
        }
        __nanosleep(64);
    }
    if (valid && G > 0) { // the last segment's partial (segment 0's with the root's term),
        put_partial(a, kc, me, sx, sy, sz); // zeros for segments the walk did not reach
        for (int kk = kc + 1; kk < k0 + G; kk++)
            put_partial(a, kk, me, 0.0, 0.0, 0.0);
    } else if (valid) {
        a.ax[me] = a.G * sx;
        a.ay[me] = a.G * sy;
        a.az[me] = a.G * sz;
    }
}

// PAIRS producer/consumer pairs per block (task t of the grid is pair
// t % PAIRS of block t / PAIRS), 12 pairs per SM either way: one pair for
// launches of few tasks (finer blocks balance better over the SMs), two
// otherwise (measured faster from ~100k bodies on).
// One producer/consumer pair per task (G == 0) or per unit of G segments,
// u = (8 / G) * task + k0 / G (partials into a.part).
template <bool STATS, bool EMPTY, int PAIRS, int G>
__device__ __forceinline__ void walk64ws_body(const WalkArgs &a)
{
    __shared__ WsShared sh_all[PAIRS];
    __shared__ NodeW32 win_all[PAIRS][CSG_WARP];
    const int warp = threadIdx.x >> 5, pair = warp >> 1, lane = threadIdx.x & 31;
    WsShared &sh = sh_all[pair];
    const int nn = a.sc->n_nodes;
    if (nn > a.node_cap || nn < 1)
        return;
    const int u = blockIdx.x * PAIRS + pair;
    const int t = G > 0 ? u / (8 / G) : u, k0 = G > 0 ? (u % (8 / G)) * G : 0;
    TaskRange tr{0, 0, 0, 0};
    bool ok = t < a.sc->n_tasks;
    if (ok) {
        const WalkTask w = a.tasks[t];
        const DevRoot &r = a.roots[w.gal];
        tr = TaskRange{w.pos0, w.count, r.root, r.end};
        const bool small = (a.sys_n ? a.sys_n[w.gal] : a.n_bodies) <= a.split_max;
        if (G > 0 ? !small : (small && a.skip_small)) {
            ok = false; // the other form walks this system
        } else if (tr.root < 0 || tr.end > nn || tr.root >= tr.end) {
            if ((warp & 1) == 0 && lane == 0)
                dev_fail(a.sc, CSG_ERR_WALK_LIMIT);
            ok = false;
        }
    }
    if (ok && (warp & 1) == 0) {
        sh.tail[lane] = 0;
        sh.head[lane] = 0;
        if (lane == 0) {
            sh.done = 0;
            sh.broken = 0;
        }
    }
    __syncthreads(); // every thread: counters set before either warp of any pair starts
    if (!ok)
        return; // both warps of the pair
    WalkStats st;
    if ((warp & 1) == 0)
        ws_produce<STATS, EMPTY, G>(a, win_all[pair], sh, tr, k0, st);
    else
        ws_consume<G>(a, sh, tr, k0);
    if (STATS && (warp & 1) == 0)
        add_hits(a, st);
}

template <bool STATS, bool EMPTY, int PAIRS>
__global__ void __launch_bounds__(2 * PAIRS * CSG_WARP, 24 / (2 * PAIRS)) k_walk64ws(WalkArgs a)
{
    walk64ws_body<STATS, EMPTY, PAIRS, 0>(a);
}

// The FP64 walk split by the root's children (trees built here, few tasks
// for the GPU): partials into a.part, summed by k_walk_sum; the same bits as
// k_walk64ws.
template <bool STATS, int PAIRS, int G>
__global__ void __launch_bounds__(2 * PAIRS * CSG_WARP, 24 / (2 * PAIRS)) k_walk64ws_units(WalkArgs a)
{
    walk64ws_body<STATS, false, PAIRS, G>(a);
}

// Dead bodies get a = 0 (src/octree.c:226-230); alive ones are overwritten by
// the walk.
// Also rewinds the task counter of the persistent walks.
__global__ void k_zero_acc(const double *__restrict__ m, double *ax, double *ay, double *az, int n,
                           DevScalars *sc)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0)
        sc->task_next = 0;
    if (i >= n)
        return;
    if (m[i] <= 0.0) {
        ax[i] = 0.0;
        ay[i] = 0.0;
        az[i] = 0.0;
    }
}

// Interaction lists: the cells each alive body interacts with, in the
// reference's depth-first order (the FP64 walk's interaction set), written
// per caller index: ids[offs[i] .. offs[i] + counts[i]). FILL = false counts,
// FILL = true writes (offs from an exclusive scan of the counts).
template <bool FILL, int WARPS>
__global__ void __launch_bounds__(WARPS * CSG_WARP) k_walk_lists(WalkArgs a, int *counts,
                                                             const int *offs, int *ids, int cap)
{
    __shared__ NodeW32 win_all[WARPS][CSG_WARP];
    NodeW32 *win = win_all[threadIdx.x >> 5];
    for_each_task<WARPS, false>(a, [&](const TaskRange &tr) {
        const int lane = threadIdx.x & 31;
        const bool valid = lane < tr.count;
        const int me = valid ? a.perm[tr.pos0 + lane] : -1;
        const BodyPos b = body_pos(a, me, valid);
        int k = 0;
        const int base = (FILL && valid) ? offs[me] : 0;
        const int lim = (FILL && valid) ? min(counts[me], cap - base) : 0;
        walk_cells<false>(a, win, tr.root, tr.end, me, valid, b,
            [&](bool take, const Cell &, float, float, float, float, int cur) {
                if (take) {
                    if (FILL && k < lim)
                        ids[base + k] = cur;
                    k++;
                }
            },
            [&](int, bool) {});
        if (!FILL && valid)
            counts[me] = k;
    });
}

} // namespace

// ---- host side -------------------------------------------------------------

namespace {

WalkArgs walk_args(csgd_t *d, const csgd_force_params *p)
{
    WalkArgs a;
    a.perm = d->perm;
    a.x = d->x;
    a.y = d->y;
    a.z = d->z;
    a.w64 = d->w64;
    a.w32 = d->w32;
    a.tasks = d->tasks;
    a.roots = d->roots;
    a.sc = d->sc;
    a.wait_polls = csgd_wait_polls(d);
    a.ax = d->ax;
    a.ay = d->ay;
    a.az = d->az;
    a.G = p->G;
    a.eps2 = p->softening * p->softening;
    a.theta2 = p->theta * p->theta;
    a.t2lo = a.theta2 * (1.0 - 0x1p-50);
    a.t2hi = a.theta2 * (1.0 + 0x1p-50);
    a.Gf = (float)p->G;
    a.eps2f = (float)a.eps2;
    // FP32 error band: |d| is exact to ~2^-46 |coordinates| (hi/lo pairs), d^2
    // to a few FP32 ulps, each product below to 2^-23; g = 2^-19 (1 + theta^2)
    // relative covers them with a wide margin. theta = 0 gives acc_k = opn_k =
    // inf: nothing is accepted, every cell with d^2 > 0 opens.
    const double g = 0x1p-19 * (1.0 + a.theta2);
    a.acc_k = (float)((1.0 + g) / a.theta2);
    a.opn_k = (float)((1.0 - g) / a.theta2);
    a.node_cap = d->node_cap;
    a.group = d->walk_group;
    return a;
}

// Kernel variant by (stats, empty cells, persistent); persistent launches
// exist for trees built here only (no empty cells).
#define CSG_LAUNCH_WALK(K, W, grid, s, a)                                                  \
    do {                                                                                    \
        if (persist && stats)                                                               \
            K<true, false, W, true><<<grid, W * CSG_WARP, 0, s>>>(a);                       \
        else if (persist)                                                                   \
            K<false, false, W, true><<<grid, W * CSG_WARP, 0, s>>>(a);                      \
        else if (stats && empty)                                                            \
            K<true, true, W, false><<<grid, W * CSG_WARP, 0, s>>>(a);                       \
        else if (stats)                                                                     \
            K<true, false, W, false><<<grid, W * CSG_WARP, 0, s>>>(a);                      \
        else if (empty)                                                                     \
            K<false, true, W, false><<<grid, W * CSG_WARP, 0, s>>>(a);                      \
        else                                                                                \
            K<false, false, W, false><<<grid, W * CSG_WARP, 0, s>>>(a);                     \
    } while (0)


// One walk launch with the state's launch shape.
void launch_walk(csgd_t *d, const WalkArgs &a, int precision, int exact)
{
    cudaStream_t s = d->stream;
    const int W = d->walk_warps == 4 ? 4 : 8;
    // trees built here have no empty cell below a non-empty root; a caller's
    // pool may (the reference skips those cells)
    const bool empty = d->imported != 0;
    const bool stats = d->stats != 0;
    const bool persist = a.group > 0 && !empty && !exact;
    WalkArgs b = a;
    if (!persist)
        b.group = 0;
    int grid;
    if (persist) {
        grid = d->num_sms * d->walk_bps;
    } else {
        const long long tasks = (long long)d->n / CSG_WARP + d->n_gal + 1; // >= n_tasks
        grid = (int)((tasks + W - 1) / W);
    }
    if (grid < 1)
        grid = 1;
    if (exact) {
        if (stats)
            k_walk64_exact<true><<<grid, 8 * CSG_WARP, 0, s>>>(b);
        else
            k_walk64_exact<false><<<grid, 8 * CSG_WARP, 0, s>>>(b);
    } else if (precision == CSG_PREC_FP32_MIXED && !stats && !empty && csgd_walk_split(d) &&
               d->wpart && d->wpart_cap >= d->n) {
        // few tasks for the GPU: eight warps per task, one per root child,
        // then the partials added in child order (the same bits as below)
        const long long units = ((long long)d->n / CSG_WARP + d->n_gal + 1) * WSEGS;
        k_walk32_units<<<(int)((units + 3) / 4), 4 * CSG_WARP, 0, s>>>(b, d->wpart,
                                                                       (long long)d->wpart_cap);
        d->launches++;
        k_walk_sum<<<csgd_grid(d->n, 256), 256, 0, s>>>(d->wpart, (long long)d->wpart_cap, d->m,
                                                          d->n, b.G, d->ax, d->ay, d->az, nullptr,
                                                          nullptr, 0);
    } else if (precision == CSG_PREC_FP32_MIXED) {
        if (W == 4)
            CSG_LAUNCH_WALK(k_walk32, 4, grid, s, b);
        else
            CSG_LAUNCH_WALK(k_walk32, 8, grid, s, b);
    } else { // FP64: producer/consumer pairs (the task group applies to FP32 only)
        // small systems (split_max bodies or fewer): pairs per (task, root
        // children), partials added by k_walk_sum; the rest a pair per task
        b.sys_n = d->n_gal > 1 ? d->sys_n : nullptr;
        b.n_bodies = d->n;
        b.split_max = (int)csgd_split_max_bodies(d);
        const bool units = !empty && d->wpart && d->wpart_cap >= d->n &&
                           csgd_sys_min_n(d) <= b.split_max;
        b.skip_small = units;
        if (units) {
            // G segments per pair: one while the units fit about four waves of
            // pairs (12 per SM), more (with markers between them) for larger launches
            const long long tasks = (long long)d->n / CSG_WARP + d->n_gal + 1;
            int g = 1;
            while (g < WSEGS && tasks * (WSEGS / g) > 4LL * 12 * d->num_sms)
                g *= 2;
            const long long nu = tasks * (WSEGS / g);
            const int pairs = nu > 8LL * d->num_sms ? 2 : 1;
            const int gw = (int)((nu + pairs - 1) / pairs);
            b.part = d->wpart;
            b.pstride = d->wpart_cap;
#define CSG_U(ST, P, GG) k_walk64ws_units<ST, P, GG><<<gw, 2 * P * CSG_WARP, 0, s>>>(b)
#define CSG_UG(ST, P)                                                                              \
    do {                                                                                          \
        if (g == 1)                                                                               \
            CSG_U(ST, P, 1);                                                                      \
        else if (g == 2)                                                                          \
            CSG_U(ST, P, 2);                                                                      \
        else if (g == 4)                                                                          \
            CSG_U(ST, P, 4);                                                                      \
        else                                                                                      \
            CSG_U(ST, P, 8);                                                                      \
    } while (0)
            if (pairs == 2 && stats)
                CSG_UG(true, 2);
            else if (pairs == 2)
                CSG_UG(false, 2);
            else if (stats)
                CSG_UG(true, 1);
            else
                CSG_UG(false, 1);
#undef CSG_UG
#undef CSG_U
            k_walk_sum<<<csgd_grid(d->n, 256), 256, 0, s>>>(d->wpart, (long long)d->wpart_cap,
                                                              d->m, d->n, b.G, d->ax, d->ay, d->az,
                                                              d->gid, b.sys_n, b.split_max);
            d->launches += 2;
            if (csgd_sys_max_n(d) <= b.split_max)
                return; // every system is small
        }
        const long long tasks = (long long)d->n / CSG_WARP + d->n_gal + 1; // >= n_tasks
        const int pairs = tasks > 8LL * d->num_sms ? 2 : 1;
        const int gw = (int)((tasks + pairs - 1) / pairs);
        const int threads = 2 * pairs * CSG_WARP;
#define CSG_WS(ST, EM)                                                                             \
    do {                                                                                          \
        if (pairs == 2)                                                                           \
            k_walk64ws<ST, EM, 2><<<gw, threads, 0, s>>>(b);                                      \
        else                                                                                      \
            k_walk64ws<ST, EM, 1><<<gw, threads, 0, s>>>(b);                                      \
    } while (0)
        if (stats && empty)
            CSG_WS(true, true);
        else if (stats)
            CSG_WS(true, false);
        else if (empty)
            CSG_WS(false, true);
        else
            CSG_WS(false, false);
#undef CSG_WS
    }
    d->launches++;
}

} // namespace

extern "C" int csgd_gravity_ex(csgd_t *d, const csgd_force_params *p, int exact)
{
    const int n = d->n;
    if (n <= 0)
        return CSG_OK;
    WalkArgs a = walk_args(d, p);
    if (exact) // the parity walk keeps one warp per task, 8 warps per block
        a.group = 0;
    cudaStream_t s = d->stream;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) == cudaSuccess && cap == cudaStreamCaptureStatusNone) {
        const int rc = csgd_prepare_walk(d, p->precision); // a capture prepared it before
        if (rc)
            return rc;
    }
    { k_zero_acc<<<csgd_grid(n, 256), 256, 0, s>>>(d->m, d->ax, d->ay, d->az, n, d->sc); d->launches++; }
    if (exact) {
        const int saved = d->walk_warps;
        d->walk_warps = 8;
        launch_walk(d, a, p->precision, 1);
        d->walk_warps = saved;
    } else {
        launch_walk(d, a, p->precision, 0);
    }
    return csgd_check(d, cudaGetLastError());
}

extern "C" int csgd_gravity(csgd_t *d, const csgd_force_params *p)
{
    return csgd_gravity_ex(d, p, 0);
}

extern "C" int csgd_walk_lists(csgd_t *d, const csgd_force_params *p, int *counts,
                               const int *offs, int *ids, int cap, int fill)
{
    const int n = d->n;
    if (n <= 0)
        return CSG_OK;
    if (d->imported) { // lists are defined on trees built here
        return CSG_ERR_UNSUPPORTED;
    }
    WalkArgs a = walk_args(d, p);
    a.group = 0;
    const long long tasks = (long long)n / CSG_WARP + d->n_gal + 1;
    // few tasks (the adjoint's 10k bodies are ~313): 2-warp blocks spread them
    // over every SM instead of crowding 8 per SM on a quarter of the GPU
    if (tasks < 8LL * d->num_sms) {
        const int grid = (int)((tasks + 1) / 2);
        if (fill)
            { k_walk_lists<true, 2><<<grid, 2 * CSG_WARP, 0, d->stream>>>(a, counts, offs, ids, cap); d->launches++; }
        else
            { k_walk_lists<false, 2><<<grid, 2 * CSG_WARP, 0, d->stream>>>(a, counts, offs, ids, cap); d->launches++; }
    } else {
        const int grid = (int)((tasks + 7) / 8);
        if (fill)
            { k_walk_lists<true, 8><<<grid, 8 * CSG_WARP, 0, d->stream>>>(a, counts, offs, ids, cap); d->launches++; }
        else
            { k_walk_lists<false, 8><<<grid, 8 * CSG_WARP, 0, d->stream>>>(a, counts, offs, ids, cap); d->launches++; }
    }
    return csgd_check(d, cudaGetLastError());
}

// ---- launch shape and its autotuner ------------------------------------------

extern "C" int csgd_set_walk_shape(csgd_t *d, const CsgWalkShape *w)
{
    if (!w || (w->warps_per_block != 4 && w->warps_per_block != 8) || w->task_group < 0 ||
        w->task_group > 64 || (w->task_group > 0 && (w->blocks_per_sm < 1 || w->blocks_per_sm > 32))) {
        return CSG_ERR_BAD_ARG;
    }
    if (d->walk_warps != w->warps_per_block || d->walk_group != w->task_group ||
        d->walk_bps != w->blocks_per_sm)
        csgd_drop_graph(d); // the captured walk launch changes
    d->walk_warps = w->warps_per_block;
    d->walk_group = w->task_group;
    d->walk_bps = w->task_group > 0 ? w->blocks_per_sm : 0;
    return CSG_OK;
}

extern "C" void csgd_get_walk_shape(const csgd_t *d, CsgWalkShape *w)
{
    w->warps_per_block = d->walk_warps;
    w->task_group = d->walk_group;
    w->blocks_per_sm = d->walk_bps;
    w->ms = 0.0f;
}

// Times every candidate launch shape on the current tree (reps walks each,
// the median kept) and keeps the fastest. The walk's results do not depend on
// the shape: every body's sum is formed by one lane in the same order.
extern "C" int csgd_autotune_walk(csgd_t *d, const csgd_force_params *p, int reps,
                                  CsgWalkShape *out, CsgWalkShape *all, int all_cap,
                                  int *n_all)
{
    if (reps < 1 || reps > 64) {
        return CSG_ERR_BAD_ARG;
    }
    // persistent candidates: 8, 16 or 24 resident warps per SM (24 is what
    // their register allocation allows), task groups of 1, 2 or 4
    static const int groups[] = {1, 2, 4};
    static const int resident[] = {8, 16, 24};
    CsgWalkShape cand[2 * (1 + 9)];
    int nc = 0;
    for (int w = 4; w <= 8; w += 4) {
        cand[nc++] = CsgWalkShape{w, 0, 0, 0.0f};
        for (int g : groups)
            for (int rw : resident)
                cand[nc++] = CsgWalkShape{w, g, rw / w, 0.0f};
    }
    CsgWalkShape saved;
    csgd_get_walk_shape(d, &saved);
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess)
        return csgd_check(d, cudaGetLastError());
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return csgd_check(d, cudaGetLastError());
    }
    int rc = CSG_OK;
    int best = -1;
    for (int c = 0; c < nc && rc == CSG_OK; c++) {
        d->walk_warps = cand[c].warps_per_block;
        d->walk_group = cand[c].task_group;
        d->walk_bps = cand[c].blocks_per_sm;
        float t[64];
        for (int r = 0; r <= reps && rc == CSG_OK; r++) { // first run warms up
            cudaEventRecord(e0, d->stream);
            rc = csgd_gravity(d, p);
            cudaEventRecord(e1, d->stream);
            if (rc == CSG_OK)
                rc = csgd_sync(d);
            if (rc == CSG_OK && r > 0)
                cudaEventElapsedTime(&t[r - 1], e0, e1);
        }
        if (rc != CSG_OK)
            break;
        for (int i = 1; i < reps; i++) // insertion sort for the median
            for (int j = i; j > 0 && t[j] < t[j - 1]; j--) {
                float x = t[j];
                t[j] = t[j - 1];
                t[j - 1] = x;
            }
        cand[c].ms = t[reps / 2];
        if (best < 0 || cand[c].ms < cand[best].ms)
            best = c;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    d->walk_warps = saved.warps_per_block;
    d->walk_group = saved.task_group;
    d->walk_bps = saved.blocks_per_sm;
    if (rc != CSG_OK)
        return rc;
    if (n_all)
        *n_all = nc;
    for (int c = 0; all && c < nc && c < all_cap; c++)
        all[c] = cand[c];
    rc = csgd_set_walk_shape(d, &cand[best]);
    if (out)
        *out = cand[best];
    return rc;
}
