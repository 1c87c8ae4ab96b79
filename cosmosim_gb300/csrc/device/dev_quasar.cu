// dev_quasar.cu — the quasar/AGN step (reference src/quasar.c:477-509) on the
// device, as one cooperative launch over the whole GPU.
//
// What the step reproduces (the reference's semantics are the specification):
// accretion onto each SMBH in index order and, per SMBH, of its victims in
// index order, the SMBH's mass, velocity and spin evolving victim by victim;
// accretion rates and luminosities; radiation feedback; jet countdown, with a
// lobe appended for every expiring heavy jet; lobe countdown; recycling of
// jets far from the first live SMBH as infalling gas; jet spawning. Random
// numbers come from one xorshift64 stream (src/quasar.c:11-35) consumed in
// that order — 3 draws per lobe, 2 per recycled jet, 3 per jet spawn — and
// the jet knot phase advances once per step (:224).
//
// How the GPU does it:
//  * Each stage is a grid-wide pass; stages are separated by grid barriers of
//    one cooperative launch, so the step has no host round trip inside.
//  * Where index order matters, a pass sets one bit per selected body in a
//    bitmap, and an ordered compaction (per-block bit counts, prefix over
//    blocks, in-block scan) turns the bits into an ascending list and clears
//    them.
//  * Accretion: only candidates inside the swallow radius or the ISCO can be
//    accreted ("inner"), so only they form a sequential chain: one thread
//    walks them in index order (staged a block-wide chunk at a time in shared
//    memory), updating the SMBH and recording its mass and velocity after
//    every accretion event. Every other candidate ("outer":
//    possibly turned into gas and dragged, never accreted) runs in parallel
//    with the SMBH state that holds at its index, found by binary search in
//    that event table.
//  * Appended and recycled bodies: each one knows its slot from a prefix
//    count and its random numbers from its draw offset; the generator is
//    jumped ahead to that offset (xs_jump), so all of them are written at
//    once.
// Arithmetic keeps the reference's operation order (the file is compiled
// without fused multiply-add); the accretion chain's divisions and square
// roots are the correctly rounded integer-pipe ones of dev_fpint.cuh (same
// bits as the compiler's, at a fraction of a lone thread's FP64 latency);
// sin, cos and log are CUDA's, within 2 ulp of the C library's, so spawned
// and recycled jets agree to ~1e-15 and all other fields exactly.
//
// Fields: positions, velocities, accelerations, mass, type, density,
// pressure, internal energy and smoothing length live in the SoA arrays;
// spin, accretion rate, luminosity and lifetime in the device Body staging
// (csgd::aos), their authoritative copy while the state is resident.
#include <cooperative_groups.h>

#include "dev_fpint.cuh"
#include "dev_internal.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr double QPI = 3.14159265358979323846;
constexpr int QB = 256;              // threads per block
constexpr int QMAX_SMBH = 1024;      // SMBHs one step handles
constexpr int QMAX_SPAWNS = 12;      // spawns per SMBH: up to 8 plus 4 burst knots
constexpr unsigned FULL = 0xffffffffu;

struct QCfg {
    double acc_r, swallow_r, isco_r, alpha, jet_speed, jet_mass, jet_life, fb, eta, edd_k,
        smoothing;
    int jet_cap, ring_count, n_alloc, pad;
};

struct Bodies {
    double *x, *y, *z, *vx, *vy, *vz, *ax, *ay, *az, *m, *rho, *P, *u, *h;
    int *type;
    Body *aos;
};

// Device scratch, one allocation sized for `cap` bodies (layout in qscratch_layout).
struct QScratch {
    unsigned *bits;  // cap bits, all zero between uses
    int *list;       // ordered compaction output, cap
    int *blockcnt;   // per-block counts of a compaction
    int *smbh;       // SMBH indices as found (unordered)
    int *ev_idx;     // accretion event table: victim index (row 0: -1 = initial state)
    double *ev_m, *ev_vx, *ev_vy, *ev_vz; // SMBH mass and velocity after the event
    int *sp_k, *sp_j, *sp_first, *sp_ring, *sp_norm; // jet spawn plan
    double *frame;   // per SMBH: jet frame (perp, perp2, helix offset), 9 doubles
    XsJumpTable *jump;
};

struct Hole { // an SMBH while its victims are processed
    double x, y, z, vx, vy, vz, m, sx, sy, sz;
};

struct Draws { // the step's random stream from a given offset
    unsigned long long s;
    __device__ double uniform()
    {
        s ^= s << 13;
        s ^= s >> 7;
        s ^= s << 17;
        return (double)(s >> 11) * (1.0 / 9007199254740992.0);
    }
    __device__ double gaussian() // Box-Muller, first output (src/quasar.c:29-35)
    {
        double a = uniform();
        const double b = uniform();
        if (a < 1e-15)
            a = 1e-15;
        return sqrt(-2.0 * log(a)) * cos(2.0 * QPI * b);
    }
};

// Exclusive prefix sum of v over the block; *total receives the block's sum.
__device__ int block_exscan(int v, int *total)
{
    __shared__ int s_w[QB / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, x, o);
        if (lane >= o)
            x += y;
    }
    if (lane == 31)
        s_w[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int t = lane < QB / 32 ? s_w[lane] : 0;
        for (int o = 1; o < QB / 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL, t, o);
            if (lane >= o)
                t += y;
        }
        if (lane < QB / 32)
            s_w[lane] = t;
    }
    __syncthreads();
    const int before = wid ? s_w[wid - 1] : 0;
    *total = s_w[QB / 32 - 1];
    __syncthreads(); // s_w is reused by the next call
    return before + x - v;
}

// The positions of the bits set in bits[0, nwords), ascending, into out[];
// the words are cleared. Returns the count (in every block). Holds one grid
// barrier; out[] may be read after the caller's next barrier.
__device__ int grid_compact(cg::grid_group &grid, unsigned *bits, int nwords, int *out,
                            int *blockcnt)
{
    const int per = (nwords + (int)gridDim.x - 1) / (int)gridDim.x;
    const int w0 = min(nwords, (int)blockIdx.x * per), w1 = min(nwords, w0 + per);
    int mine = 0;
    for (int w = w0 + threadIdx.x; w < w1; w += QB)
        mine += __popc(bits[w]);
    int tot;
    block_exscan(mine, &tot);
    if (threadIdx.x == 0)
        blockcnt[blockIdx.x] = tot;
    grid.sync();
    int before = 0, all = 0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += QB) {
        const int v = blockcnt[b];
        all += v;
        if (b < (int)blockIdx.x)
            before += v;
    }
    int base, total;
    block_exscan(before, &base);
    block_exscan(all, &total);
    for (int c0 = w0; c0 < w1; c0 += QB) {
        const int w = c0 + threadIdx.x;
        unsigned word = w < w1 ? bits[w] : 0u;
        int chunk;
        int at = base + block_exscan(__popc(word), &chunk);
        while (word) {
            out[at++] = w * 32 + (__ffs(word) - 1);
            word &= word - 1u;
        }
        if (w < w1)
            bits[w] = 0u;
        base += chunk;
    }
    return total;
}

__device__ __forceinline__ void mark(unsigned *bits, int i)
{
    atomicOr(&bits[i >> 5], 1u << (i & 31));
}

// A body stops: no mass, no velocity, no acceleration.
__device__ __forceinline__ void stop_body(const Bodies &b, int i)
{
    b.m[i] = 0.0;
    b.vx[i] = b.vy[i] = b.vz[i] = 0.0;
    b.ax[i] = b.ay[i] = b.az[i] = 0.0;
}

// A fresh body record at slot i: every field zero, then the given type.
__device__ void fresh_body(const Bodies &b, int i, int type)
{
    b.x[i] = b.y[i] = b.z[i] = 0.0;
    b.vx[i] = b.vy[i] = b.vz[i] = 0.0;
    b.ax[i] = b.ay[i] = b.az[i] = 0.0;
    b.m[i] = 0.0;
    b.rho[i] = b.P[i] = b.u[i] = b.h[i] = 0.0;
    b.type[i] = type;
    b.aos[i] = Body{};
    b.aos[i].type = (BodyType)type;
}

// Hole H takes victim v (src/quasar.c:63-101): momentum-conserving merge,
// spin nudged toward the victim's orbital angular momentum (relative to the
// merged velocity), victim stopped.
__device__ void swallow(Hole &H, const Bodies &b, int v)
{
    const double mv = b.m[v], mt = H.m + mv;
    H.vx = div_rn(H.m * H.vx + mv * b.vx[v], mt);
    H.vy = div_rn(H.m * H.vy + mv * b.vy[v], mt);
    H.vz = div_rn(H.m * H.vz + mv * b.vz[v], mt);
    const double px = b.x[v] - H.x, py = b.y[v] - H.y, pz = b.z[v] - H.z;
    const double qx = b.vx[v] - H.vx, qy = b.vy[v] - H.vy, qz = b.vz[v] - H.vz;
    const double jx = py * qz - pz * qy, jy = pz * qx - px * qz, jz = px * qy - py * qx;
    const double j = sqrt_rn(jx * jx + jy * jy + jz * jz);
    if (j > 1e-15) {
        const double f = div_rn(mv, mt) * 0.01;
        H.sx += div_rn(f * jx, j);
        H.sy += div_rn(f * jy, j);
        H.sz += div_rn(f * jz, j);
        const double sn = sqrt_rn(H.sx * H.sx + H.sy * H.sy + H.sz * H.sz);
        if (sn > 1e-15) {
            H.sx = div_rn(H.sx, sn);
            H.sy = div_rn(H.sy, sn);
            H.sz = div_rn(H.sz, sn);
        }
    }
    H.m = mt;
    stop_body(b, v);
}

// A candidate at offset (dx, dy, dz), distance r from hole H that is not
// swallowed outright (src/quasar.c:156-183): it turns into gas when the
// circularisation radius of its orbit lies outside the ISCO (SPH fields
// seeded if unset); gas feels the accretion disk's radial drag
// (src/quasar.c:103-123). Returns whether the body is gas.
__device__ bool settle(const Bodies &b, const QCfg &c, const Hole &H, int i, double dx, double dy,
                       double dz, double r)
{
    const double qx = b.vx[i] - H.vx, qy = b.vy[i] - H.vy, qz = b.vz[i] - H.vz;
    const double jx = dy * qz - dz * qy, jy = dz * qx - dx * qz, jz = dx * qy - dy * qx;
    const double r_circ = div_rn(jx * jx + jy * jy + jz * jz, H.m * r);
    if (r_circ > c.isco_r && b.type[i] != BODY_GAS) {
        b.type[i] = BODY_GAS;
        if (b.h[i] < 1e-10)
            b.h[i] = c.acc_r * 0.3;
        if (b.u[i] < 1e-10) {
            const double v2 = b.vx[i] * b.vx[i] + b.vy[i] * b.vy[i] + b.vz[i] * b.vz[i];
            b.u[i] = 0.001 * v2 + 0.01;
        }
    }
    if (b.type[i] != BODY_GAS)
        return false;
    const double rx = b.x[i] - H.x, ry = b.y[i] - H.y, rz = b.z[i] - H.z;
    const double rr = sqrt_rn(rx * rx + ry * ry + rz * rz);
    if (rr < 1e-15)
        return true;
    const double wx = b.vx[i] - H.vx, wy = b.vy[i] - H.vy, wz = b.vz[i] - H.vz;
    const double radial = div_rn(wx * rx + wy * ry + wz * rz, rr);
    b.ax[i] -= c.alpha * div_rn(radial * rx, rr);
    b.ay[i] -= c.alpha * div_rn(radial * ry, rr);
    b.az[i] -= c.alpha * div_rn(radial * rz, rr);
    return true;
}

// Row e of the event table: the largest e with ev_idx[e] < i (row 0 holds
// index -1, the state before any event).
__device__ int state_at(const QScratch &w, int n_events, int i)
{
    int lo = 0, hi = n_events; // ev_idx[lo] < i <= ev_idx[hi + 1]
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (w.ev_idx[mid] < i)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(QB) k_quasar_step(Bodies b, QCfg c, QuasarState *q,
                                                    QScratch w, double dt)
{
    cg::grid_group grid = cg::this_grid();
    __shared__ int s_smbh[QMAX_SMBH];
    const int tid = threadIdx.x;
    const long long gtid = (long long)blockIdx.x * QB + tid;
    const long long gsz = (long long)gridDim.x * QB;
    const bool lead = gtid == 0;
    const int n0 = q->n, jc0 = q->jet_count, knot0 = q->knot_phase;
    const unsigned long long rng0 = q->rng;
    const int nwords = (c.n_alloc + 31) >> 5;
    grid.sync(); // every thread has read the inputs before they change
    if (lead) {
        q->n_smbh = 0;
        q->swallowed = 0.0;
        q->expired = 0;
        q->err = 0;
    }
    grid.sync();

    // ---- the SMBHs, sorted by index in every block ----
    for (long long i = gtid; i < n0; i += gsz)
        if (b.type[i] == BODY_SMBH) {
            const int k = atomicAdd(&q->n_smbh, 1);
            if (k < QMAX_SMBH)
                w.smbh[k] = (int)i;
        }
    grid.sync();
    const int ns = q->n_smbh;
    if (ns > QMAX_SMBH) { // uniform over the grid: nothing has changed yet
        if (lead)
            q->err = CSG_ERR_UNSUPPORTED;
        return;
    }
    int span = 1;
    while (span < ns)
        span <<= 1;
    for (int k = tid; k < span; k += QB)
        s_smbh[k] = k < ns ? w.smbh[k] : 0x7fffffff;
    __syncthreads();
    for (int size = 2; size <= span; size <<= 1) // bitonic sort
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int k = tid; k < span; k += QB) {
                const int o = k ^ stride;
                if (o > k) {
                    const int a = s_smbh[k], v = s_smbh[o];
                    if ((a > v) == ((k & size) == 0)) {
                        s_smbh[k] = v;
                        s_smbh[o] = a;
                    }
                }
            }
            __syncthreads();
        }

    // ---- 1. accretion (src/quasar.c:125-190), SMBH by SMBH ----
    const double r_acc_sq = c.acc_r * c.acc_r, r_sw_sq = c.swallow_r * c.swallow_r;
    for (int k = 0; k < ns; k++) {
        const int s = s_smbh[k];
        if (!(b.m[s] > 0.0))
            continue; // the same decision in every block: SMBH masses only grow here
        const double hx = b.x[s], hy = b.y[s], hz = b.z[s];
        // inner candidates -> bitmap
        for (long long i = gtid; i < n0; i += gsz) {
            if (i == s || b.m[i] <= 0.0 || b.type[i] == BODY_SMBH)
                continue;
            const double dx = b.x[i] - hx, dy = b.y[i] - hy, dz = b.z[i] - hz;
            const double d2 = dx * dx + dy * dy + dz * dz;
            if (!(d2 > r_acc_sq) && (d2 < r_sw_sq || sqrt(d2) < c.isco_r))
                mark(w.bits, (int)i);
        }
        grid.sync();
        const int n_inner = grid_compact(grid, w.bits, nwords, w.list, w.blockcnt);
        grid.sync();
        if (blockIdx.x == 0) {
            // The chain of possible accretions, in index order. The whole block
            // stages a chunk of candidates in shared memory, one thread runs
            // the chain over it (the same arithmetic on the staged copies),
            // the block writes the candidates back.
            __shared__ double cf[12][QB];
            __shared__ int ct[QB];
            const Bodies sb{cf[0], cf[1], cf[2], cf[3], cf[4], cf[5], cf[6], cf[7], cf[8], cf[9],
                            nullptr, nullptr, cf[10], cf[11], ct, nullptr};
            Hole H{hx, hy, hz, b.vx[s], b.vy[s], b.vz[s], b.m[s], b.aos[s].spin_x,
                   b.aos[s].spin_y, b.aos[s].spin_z};
            double swallowed = q->swallowed;
            int e = 0;
            if (tid == 0) {
                w.ev_idx[0] = -1;
                w.ev_m[0] = H.m;
                w.ev_vx[0] = H.vx;
                w.ev_vy[0] = H.vy;
                w.ev_vz[0] = H.vz;
            }
            for (int base = 0; base < n_inner; base += QB) {
                const int cnt = min(QB, n_inner - base);
                const int i = tid < cnt ? w.list[base + tid] : 0;
                if (tid < cnt) {
                    sb.x[tid] = b.x[i];
                    sb.y[tid] = b.y[i];
                    sb.z[tid] = b.z[i];
                    sb.vx[tid] = b.vx[i];
                    sb.vy[tid] = b.vy[i];
                    sb.vz[tid] = b.vz[i];
                    sb.ax[tid] = b.ax[i];
                    sb.ay[tid] = b.ay[i];
                    sb.az[tid] = b.az[i];
                    sb.m[tid] = b.m[i];
                    sb.u[tid] = b.u[i];
                    sb.h[tid] = b.h[i];
                    sb.type[tid] = b.type[i];
                }
                __syncthreads();
                if (tid == 0) {
                    for (int t = 0; t < cnt; t++) {
                        const double dx = sb.x[t] - hx, dy = sb.y[t] - hy, dz = sb.z[t] - hz;
                        const double d2 = dx * dx + dy * dy + dz * dz;
                        bool eaten = d2 < r_sw_sq;
                        if (!eaten) {
                            const double r = sqrt_rn(d2);
                            eaten = settle(sb, c, H, t, dx, dy, dz, r) && r < c.isco_r;
                        }
                        if (eaten) {
                            swallowed += sb.m[t];
                            swallow(H, sb, t);
                            e++;
                            w.ev_idx[e] = w.list[base + t];
                            w.ev_m[e] = H.m;
                            w.ev_vx[e] = H.vx;
                            w.ev_vy[e] = H.vy;
                            w.ev_vz[e] = H.vz;
                        }
                    }
                }
                __syncthreads();
                if (tid < cnt) {
                    b.vx[i] = sb.vx[tid];
                    b.vy[i] = sb.vy[tid];
                    b.vz[i] = sb.vz[tid];
                    b.ax[i] = sb.ax[tid];
                    b.ay[i] = sb.ay[tid];
                    b.az[i] = sb.az[tid];
                    b.m[i] = sb.m[tid];
                    b.u[i] = sb.u[tid];
                    b.h[i] = sb.h[tid];
                    b.type[i] = sb.type[tid];
                }
                __syncthreads(); // the next chunk reuses the staging
            }
            if (tid == 0) {
                q->n_events = e;
                q->swallowed = swallowed;
                b.m[s] = H.m;
                b.vx[s] = H.vx;
                b.vy[s] = H.vy;
                b.vz[s] = H.vz;
                b.aos[s].spin_x = H.sx;
                b.aos[s].spin_y = H.sy;
                b.aos[s].spin_z = H.sz;
            }
        }
        grid.sync();
        // outer candidates, each with the SMBH state at its index
        const int n_events = q->n_events;
        for (long long i = gtid; i < n0; i += gsz) {
            if (i == s || b.m[i] <= 0.0 || b.type[i] == BODY_SMBH)
                continue;
            const double dx = b.x[i] - hx, dy = b.y[i] - hy, dz = b.z[i] - hz;
            const double d2 = dx * dx + dy * dy + dz * dz;
            if (d2 > r_acc_sq || d2 < r_sw_sq)
                continue;
            const double r = sqrt(d2);
            if (r < c.isco_r)
                continue; // inner: done by the chain
            const int e = state_at(w, n_events, (int)i);
            const Hole H{hx, hy, hz, w.ev_vx[e], w.ev_vy[e], w.ev_vz[e], w.ev_m[e], 0.0, 0.0, 0.0};
            settle(b, c, H, (int)i, dx, dy, dz, r);
        }
        grid.sync();
    }

    // ---- 2. accretion rate and luminosity of every SMBH (src/quasar.c:482-494) ----
    if (gtid < ns) {
        const int s = s_smbh[gtid];
        Body &A = b.aos[s];
        const double mdot = q->swallowed / dt;
        A.accretion_rate = c.smoothing * A.accretion_rate + (1.0 - c.smoothing) * mdot;
        const double l_edd = c.edd_k * b.m[s];
        A.luminosity = c.eta * A.accretion_rate;
        if (A.luminosity > l_edd)
            A.luminosity = l_edd;
    }
    grid.sync();

    // ---- 3. feedback (src/quasar.c:192-220), 4. jet countdown (:375-382) ----
    const double r_fb_sq = (c.acc_r * 3.0) * (c.acc_r * 3.0);
    for (long long i = gtid; i < n0; i += gsz) {
        if (b.m[i] <= 0.0 || b.type[i] == BODY_SMBH)
            continue;
        for (int k = 0; k < ns; k++) {
            const int s = s_smbh[k];
            const double lum = b.aos[s].luminosity;
            if (lum <= 0.0)
                continue;
            const double dx = b.x[i] - b.x[s], dy = b.y[i] - b.y[s], dz = b.z[i] - b.z[s];
            const double d2 = dx * dx + dy * dy + dz * dz;
            if (d2 > r_fb_sq || d2 < 1e-10)
                continue;
            const double r = sqrt(d2);
            const double f = c.fb * lum / (4.0 * QPI * d2);
            b.ax[i] += f * dx / r;
            b.ay[i] += f * dy / r;
            b.az[i] += f * dz / r;
        }
        if (b.type[i] == BODY_JET) {
            double &life = b.aos[i].lifetime;
            life -= dt;
            if (life <= 0.0) {
                atomicAdd(&q->expired, 1);
                if (b.m[i] > 0.2)
                    mark(w.bits, (int)i); // leaves a lobe, if there is room
            }
        }
    }
    grid.sync();

    // lobes: the k-th heavy expiring jet (index order) fills slot n0 + k
    const int heavy = grid_compact(grid, w.bits, nwords, w.list, w.blockcnt);
    const int lobes = max(0, min(heavy, c.n_alloc - n0));
    grid.sync();
    for (long long k = gtid; k < lobes; k += gsz) {
        const int j = w.list[k], t = n0 + (int)k;
        Draws g{xs_jump(w.jump, rng0, 3ull * (unsigned long long)k)};
        const double mj = b.m[j], xj = b.x[j], yj = b.y[j], zj = b.z[j];
        const double vxj = b.vx[j], vyj = b.vy[j], vzj = b.vz[j];
        fresh_body(b, t, BODY_LOBE);
        b.m[t] = mj * 0.5;
        b.x[t] = xj;
        b.y[t] = yj;
        b.z[t] = zj;
        const double spread = 0.5;
        b.vx[t] = vxj * 0.15 + (g.uniform() - 0.5) * spread;
        b.vy[t] = vyj * 0.15 + (g.uniform() - 0.5) * spread;
        b.vz[t] = vzj * 0.15 + (g.uniform() - 0.5) * spread;
        b.aos[t].lifetime = c.jet_life * 3.0;
    }
    grid.sync();
    // expired jets stop; lobes (the new ones too) count down (src/quasar.c:404-421)
    const int n1 = n0 + lobes;
    for (long long i = gtid; i < n1; i += gsz) {
        if (b.m[i] <= 0.0)
            continue;
        if (b.type[i] == BODY_JET && i < n0 && b.aos[i].lifetime <= 0.0) {
            stop_body(b, (int)i);
        } else if (b.type[i] == BODY_LOBE) {
            double &life = b.aos[i].lifetime;
            life -= dt;
            if (life <= 0.0)
                stop_body(b, (int)i);
        }
    }
    grid.sync();

    // ---- 4b. recycling around the first live SMBH (src/quasar.c:424-475) ----
    int first = -1;
    for (int k = 0; k < ns && first < 0; k++)
        if (b.m[s_smbh[k]] > 0.0)
            first = s_smbh[k];
    int recycled = 0;
    if (first >= 0) {
        const double rr = c.acc_r * 10.0, rr_sq = rr * rr;
        const double fx = b.x[first], fy = b.y[first], fz = b.z[first];
        for (long long i = gtid; i < n1; i += gsz) {
            if (b.type[i] != BODY_JET || b.m[i] <= 0.0)
                continue;
            const double dx = b.x[i] - fx, dy = b.y[i] - fy, dz = b.z[i] - fz;
            if (!(dx * dx + dy * dy + dz * dz < rr_sq))
                mark(w.bits, (int)i);
        }
        grid.sync();
        recycled = grid_compact(grid, w.bits, nwords, w.list, w.blockcnt);
        grid.sync();
        const double fm = b.m[first], fvx = b.vx[first], fvy = b.vy[first], fvz = b.vz[first];
        for (long long k = gtid; k < recycled; k += gsz) {
            const int i = w.list[k];
            Draws g{xs_jump(w.jump, rng0, 3ull * (unsigned long long)lobes + 2ull * (unsigned long long)k)};
            const double phi = 2.0 * QPI * g.uniform();
            const double ct = 2.0 * g.uniform() - 1.0;
            const double st = sqrt(1.0 - ct * ct);
            const double rp = c.acc_r;
            b.x[i] = fx + rp * st * cos(phi);
            b.y[i] = fy + rp * st * sin(phi);
            b.z[i] = fz + rp * ct;
            const double v_in = 0.5 * sqrt(fm / rp);
            const double nx = (b.x[i] - fx) / rp, ny = (b.y[i] - fy) / rp, nz = (b.z[i] - fz) / rp;
            b.vx[i] = fvx - v_in * nx;
            b.vy[i] = fvy - v_in * ny;
            b.vz[i] = fvz - v_in * nz;
            b.ax[i] = b.ay[i] = b.az[i] = 0.0;
            b.type[i] = BODY_GAS;
            b.aos[i].type = BODY_GAS;
            b.aos[i].lifetime = 0.0;
            b.h[i] = c.acc_r * 0.3;
            const double v2 = b.vx[i] * b.vx[i] + b.vy[i] * b.vy[i] + b.vz[i] * b.vz[i];
            b.u[i] = 0.001 * v2 + 0.01;
            b.rho[i] = 0.0;
            b.P[i] = 0.0;
        }
    }

    // ---- 5. jet spawning (src/quasar.c:221-366) ----
    // The plan: spawns in (SMBH, j) order, each with its ring of bodies; a
    // spawn happens while there is room (jet cap and body capacity), and
    // all spawns that happen form a prefix of the plan.
    const int knot = knot0 + 1;
    double speed_mod = 1.0 + 0.6 * sin(knot * 0.10);
    if (speed_mod < 0.5)
        speed_mod = 0.5;
    const double cone = 0.05 + 0.13 * (0.5 + 0.5 * sin(knot * 0.057));
    const double helix = knot * 0.04;
    const int jc1 = jc0 - q->expired - recycled;
    if (blockIdx.x == 0 && tid == 0) {
        const long long room = min((long long)c.jet_cap - jc1, (long long)c.n_alloc - n1);
        long long made = 0;
        int p = 0;
        const double jet_energy = 0.5 * c.jet_mass * c.jet_speed * c.jet_speed;
        for (int k = 0; k < ns && made < room; k++) {
            const int s = s_smbh[k];
            const Body &A = b.aos[s];
            if (A.luminosity <= 0.0 || jet_energy < 1e-15)
                continue;
            int n_norm = (int)(A.luminosity / jet_energy);
            n_norm = n_norm < 2 ? 2 : (n_norm > 8 ? 8 : n_norm);
            // jet frame: perp to the spin axis, perp2 = spin x perp, helical offset
            double px, py, pz;
            if (fabs(A.spin_z) < 0.9) {
                px = -A.spin_y;
                py = A.spin_x;
                pz = 0.0;
            } else {
                px = 0.0;
                py = -A.spin_z;
                pz = A.spin_y;
            }
            const double pm = sqrt(px * px + py * py + pz * pz);
            if (pm > 1e-15) {
                px /= pm;
                py /= pm;
                pz /= pm;
            }
            double qx = A.spin_y * pz - A.spin_z * py;
            double qy = A.spin_z * px - A.spin_x * pz;
            double qz = A.spin_x * py - A.spin_y * px;
            const double qm = sqrt(qx * qx + qy * qy + qz * qz);
            if (qm > 1e-15) {
                qx /= qm;
                qy /= qm;
                qz /= qm;
            }
            const double amp = c.swallow_r * 0.35;
            double *f = w.frame + 9 * k;
            f[0] = px;
            f[1] = py;
            f[2] = pz;
            f[3] = qx;
            f[4] = qy;
            f[5] = qz;
            f[6] = amp * (cos(helix) * px + sin(helix) * qx);
            f[7] = amp * (cos(helix) * py + sin(helix) * qy);
            f[8] = amp * (cos(helix) * pz + sin(helix) * qz);
            const int spawns = n_norm + ((speed_mod > 1.35) ? 4 : 0);
            for (int j = 0; j < spawns && made < room; j++, p++) {
                const int ring = (j >= n_norm) ? 1 : c.ring_count;
                w.sp_k[p] = k;
                w.sp_j[p] = j;
                w.sp_first[p] = (int)made;
                w.sp_ring[p] = ring;
                w.sp_norm[p] = n_norm;
                made += min((long long)max(ring, 0), room - made);
            }
        }
        q->rng = xs_jump(w.jump, rng0, 3ull * lobes + 2ull * recycled + 3ull * p);
        q->knot_phase = knot;
        q->n = n1 + (int)made;
        q->jet_count = jc1 + (int)made;
        q->spawns = p;
        q->spawned = (int)made;
    }
    grid.sync();
    const int spawns = q->spawns, made = q->spawned;
    const unsigned long long base = 3ull * lobes + 2ull * recycled;
    for (long long t = gtid; t < made; t += gsz) {
        int lo = 0, hi = spawns - 1; // the last spawn whose first body is <= t
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (w.sp_first[mid] <= t)
                lo = mid;
            else
                hi = mid - 1;
        }
        const int p = lo, k = w.sp_k[p], j = w.sp_j[p], ring_n = w.sp_ring[p];
        const int r = (int)t - w.sp_first[p];
        const int s = s_smbh[k];
        const Body &A = b.aos[s];
        const double *f = w.frame + 9 * k;
        const bool burst = j >= w.sp_norm[p];
        const double sign = (j % 2 == 0) ? 1.0 : -1.0;
        const double this_cone = burst ? 0.012 : cone;
        const double this_speed = burst ? c.jet_speed * speed_mod * 1.28 : c.jet_speed * speed_mod;
        const double this_mass = burst ? c.jet_mass * 1.9 : c.jet_mass;
        const double this_life = burst ? c.jet_life * 1.4 : c.jet_life;
        const double fwd = burst ? c.swallow_r * 0.6 : 0.0;
        Draws g{xs_jump(w.jump, rng0, base + 3ull * (unsigned long long)p)};
        const double angle = g.uniform() * 2.0 * QPI;
        const double offset = g.gaussian() * this_cone;
        const double ra = (ring_n > 1) ? 2.0 * QPI * r / ring_n + angle : angle;
        const double rr = (ring_n > 1) ? c.swallow_r * 0.15 : 0.0;
        const double ox = rr * (cos(ra) * f[0] + sin(ra) * f[3]);
        const double oy = rr * (cos(ra) * f[1] + sin(ra) * f[4]);
        const double oz = rr * (cos(ra) * f[2] + sin(ra) * f[5]);
        const int o = n1 + (int)t;
        fresh_body(b, o, BODY_JET);
        b.aos[o].lifetime = this_life;
        b.m[o] = (ring_n > 1) ? this_mass * 0.6 : this_mass;
        const double lift = c.swallow_r + fwd;
        b.x[o] = b.x[s] + sign * A.spin_x * lift + offset * (f[0] * cos(angle)) + sign * f[6] + ox;
        b.y[o] = b.y[s] + sign * A.spin_y * lift + offset * (f[1] * cos(angle)) + sign * f[7] + oy;
        b.z[o] = b.z[s] + sign * A.spin_z * lift + offset * (f[2] * sin(angle)) + sign * f[8] + oz;
        const double widen = this_speed * 0.04 * (1.0 + this_life * 0.1);
        b.vx[o] = b.vx[s] + sign * A.spin_x * this_speed + ox * widen / (rr + 1e-15);
        b.vy[o] = b.vy[s] + sign * A.spin_y * this_speed + oy * widen / (rr + 1e-15);
        b.vz[o] = b.vz[s] + sign * A.spin_z * this_speed + oz * widen / (rr + 1e-15);
    }
}

QCfg qcfg(const QuasarConfig *cfg, int n_alloc)
{
    QCfg c;
    c.acc_r = cfg->accretion_radius;
    c.swallow_r = cfg->swallow_radius;
    c.isco_r = cfg->isco_radius;
    c.alpha = cfg->viscosity_alpha;
    c.jet_speed = cfg->jet_speed;
    c.jet_mass = cfg->jet_mass;
    c.jet_life = cfg->jet_lifetime;
    c.fb = cfg->feedback_strength;
    c.eta = cfg->eta_eff;
    c.edd_k = cfg->eddington_k;
    c.smoothing = cfg->accretion_smoothing;
    c.jet_cap = cfg->jet_cap;
    c.ring_count = cfg->jet_ring_count;
    c.n_alloc = n_alloc;
    c.pad = 0;
    return c;
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// Lays out the scratch for cap bodies and grid blocks; returns its size.
size_t qscratch_layout(char *base, int cap, int blocks, QScratch *w)
{
    const size_t words = ((size_t)cap + 31) / 32 + 1;
    const size_t plan = (size_t)QMAX_SMBH * QMAX_SPAWNS;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *p = base ? base + off : nullptr;
        off += align256(bytes);
        return p;
    };
    w->jump = (XsJumpTable *)take(sizeof(XsJumpTable));
    w->bits = (unsigned *)take(words * sizeof(unsigned));
    w->list = (int *)take((size_t)cap * sizeof(int));
    w->blockcnt = (int *)take((size_t)blocks * sizeof(int));
    w->smbh = (int *)take(QMAX_SMBH * sizeof(int));
    w->ev_idx = (int *)take(((size_t)cap + 1) * sizeof(int));
    w->ev_m = (double *)take(((size_t)cap + 1) * sizeof(double));
    w->ev_vx = (double *)take(((size_t)cap + 1) * sizeof(double));
    w->ev_vy = (double *)take(((size_t)cap + 1) * sizeof(double));
    w->ev_vz = (double *)take(((size_t)cap + 1) * sizeof(double));
    w->sp_k = (int *)take(plan * sizeof(int));
    w->sp_j = (int *)take(plan * sizeof(int));
    w->sp_first = (int *)take(plan * sizeof(int));
    w->sp_ring = (int *)take(plan * sizeof(int));
    w->sp_norm = (int *)take(plan * sizeof(int));
    w->frame = (double *)take((size_t)QMAX_SMBH * 9 * sizeof(double));
    return off;
}

// Grid of the cooperative launch: every block resident at once.
int quasar_blocks(csgd_t *d)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_quasar_step, QB, 0) != cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    return (d->num_sms > 0 ? d->num_sms : 1) * min(per_sm, 4);
}

int ensure_scratch(csgd_t *d, int cap, QScratch *w)
{
    const int blocks = quasar_blocks(d);
    if (d->q_scratch && d->q_scratch_cap >= cap) {
        qscratch_layout((char *)d->q_scratch, d->q_scratch_cap, blocks, w);
        return CSG_OK;
    }
    cudaStreamSynchronize(d->stream);
    if (d->q_scratch)
        cudaFree(d->q_scratch);
    d->q_scratch = nullptr;
    d->q_scratch_cap = 0;
    const size_t bytes = qscratch_layout(nullptr, cap, blocks, w);
    if (csgd_malloc(&d->q_scratch, bytes) != cudaSuccess) {
        cudaGetLastError();
        d->q_scratch = nullptr;
        return CSG_ERR_NOMEM;
    }
    qscratch_layout((char *)d->q_scratch, cap, blocks, w);
    cudaMemsetAsync(w->bits, 0, (((size_t)cap + 31) / 32 + 1) * sizeof(unsigned), d->stream);
    cudaMemcpyAsync(w->jump, &xs_jump_table_host(), sizeof(XsJumpTable), cudaMemcpyHostToDevice,
                    d->stream);
    d->q_scratch_cap = cap;
    return csgd_check(d, cudaGetLastError());
}

} // namespace

extern "C" void csgd_quasar_free(csgd_t *d)
{
    if (d->q_scratch)
        cudaFree(d->q_scratch);
    d->q_scratch = nullptr;
    d->q_scratch_cap = 0;
}

extern "C" int csgd_quasar_state(csgd_t *d, unsigned long long rng, int knot_phase)
{
    if (!d->qs && csgd_malloc((void **)&d->qs, sizeof(QuasarState)) != cudaSuccess) {
        cudaGetLastError();
        return CSG_ERR_NOMEM;
    }
    QuasarState h{};
    h.rng = rng ? rng : 1;
    h.knot_phase = knot_phase;
    cudaMemcpyAsync(d->qs, &h, sizeof(h), cudaMemcpyHostToDevice, d->stream);
    return csgd_sync(d); // h is on the stack
}

extern "C" int csgd_quasar_step(csgd_t *d, const QuasarConfig *cfg, int n_alloc, double dt,
                                int *jet_count, int *n_out)
{
    if (!d->qs) {
        int rc = csgd_quasar_state(d, 1, 0);
        if (rc)
            return rc;
    }
    // errors are returned at once and leave nothing for a later sync to report
    if (n_alloc > d->cap || n_alloc < d->n || d->n_gal > 1)
        return d->n_gal > 1 ? CSG_ERR_UNSUPPORTED : CSG_ERR_BAD_ARG;
    QScratch w;
    int rc = ensure_scratch(d, d->cap, &w);
    if (rc)
        return rc;
    cudaStream_t s = d->stream;
    // body count and jet count in; the step may append bodies
    int *hi = d->h_int;
    hi[0] = d->n;
    hi[1] = *jet_count;
    cudaMemcpyAsync(&d->qs->n, &hi[0], sizeof(int), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(&d->qs->jet_count, &hi[1], sizeof(int), cudaMemcpyHostToDevice, s);
    Bodies b{d->x, d->y, d->z, d->vx, d->vy, d->vz, d->ax, d->ay, d->az, d->m,
             d->rho, d->P, d->u, d->h, d->type, d->aos};
    QCfg c = qcfg(cfg, n_alloc);
    QuasarState *q = d->qs;
    void *args[] = {&b, &c, &q, &w, &dt};
    const int blocks = quasar_blocks(d);
    rc = csgd_check(d, cudaLaunchCooperativeKernel((const void *)k_quasar_step, dim3(blocks),
                                                   dim3(QB), args, 0, s));
    d->launches++;
    if (rc)
        return rc;
    cudaMemcpyAsync(&hi[0], &d->qs->n, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&hi[1], &d->qs->jet_count, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&hi[2], &d->qs->err, sizeof(int), cudaMemcpyDeviceToHost, s);
    rc = csgd_sync(d);
    if (rc)
        return rc;
    if (hi[2])
        return hi[2];
    d->n = hi[0];
    *jet_count = hi[1];
    *n_out = hi[0];
    d->geometry_valid = 0;
    d->gas_valid = 0;
    return CSG_OK;
}
