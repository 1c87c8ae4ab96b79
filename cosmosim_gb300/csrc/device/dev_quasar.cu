// dev_quasar.cu — the quasar/AGN step (reference src/quasar.c:477-509) on
// the device: accretion onto SMBHs, accretion rate and luminosity, radiation
// feedback, jet decay into lobes, recycling of distant jets, jet spawning.
//
// The reference runs these loops in index order with a sequential random
// number stream (xorshift64, src/quasar.c:11-35) and state kept across calls
// (the generator state and the jet knot phase, :11 and :224); bodies spawned
// in a step are appended. The device version keeps that order:
//   - wide passes find the bodies a stage touches (candidates within the
//     accretion radius of an SMBH, expiring jets, distant jets) and compact
//     them in index order;
//   - one thread then processes them in that order, exactly as the
//     reference's loop would (the SMBH's mass, velocity and spin evolve
//     victim by victim; random numbers are drawn in the same sequence);
//   - independent per-body updates (feedback kicks, lifetime countdowns) run
//     on every thread.
// The serial parts touch the few bodies near SMBHs and the jets; the O(N)
// scans are parallel. Compiled with -fmad=false and the reference's
// operation order; sin, cos and log are CUDA's (within 2 ulp of the C
// library's), so spawned jets agree to ~1e-15, everything else exactly.
//
// Field layout: positions, velocities, accelerations, mass, type, density,
// pressure, internal energy and smoothing length live in the SoA arrays;
// spin, accretion rate, luminosity and lifetime in the device Body staging
// (csgd::aos), which is their authoritative copy while the state is resident.
#include "dev_internal.cuh"

namespace {

constexpr double QPI = 3.14159265358979323846;
constexpr int QT = 1024; // threads of the single-block stages

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

__device__ __forceinline__ unsigned long long q_next(QuasarState *q)
{
    unsigned long long x = q->rng;
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    q->rng = x;
    return x;
}

__device__ __forceinline__ double q_uniform(QuasarState *q)
{
    return (double)(q_next(q) >> 11) * (1.0 / 9007199254740992.0);
}

__device__ __forceinline__ double q_gaussian(QuasarState *q)
{
    double u1 = q_uniform(q);
    double u2 = q_uniform(q);
    if (u1 < 1e-15)
        u1 = 1e-15;
    return sqrt(-2.0 * log(u1)) * cos(2.0 * QPI * u2);
}

// Ordered compaction of {i < n : pred(i)} into out[] by one block; returns
// the count (every thread gets it).
template <typename Pred>
__device__ int block_compact(int n, Pred pred, int *out)
{
    __shared__ int s_warp[QT / 32];
    __shared__ int s_base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int total = 0;
    for (int base = 0; base < n; base += QT) {
        const int i = base + threadIdx.x;
        const bool f = i < n && pred(i);
        const unsigned bal = __ballot_sync(0xffffffffu, f);
        if (lane == 0)
            s_warp[warp] = __popc(bal);
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0;
            for (int w = 0; w < QT / 32; w++) {
                int c = s_warp[w];
                s_warp[w] = acc;
                acc += c;
            }
            s_base = acc;
        }
        __syncthreads();
        if (f)
            out[total + s_warp[warp] + __popc(bal & ((1u << lane) - 1u))] = i;
        total += s_base;
        __syncthreads();
    }
    return total;
}

__device__ void zero_body(const Bodies &b, int i)
{
    b.x[i] = b.y[i] = b.z[i] = 0.0;
    b.vx[i] = b.vy[i] = b.vz[i] = 0.0;
    b.ax[i] = b.ay[i] = b.az[i] = 0.0;
    b.m[i] = 0.0;
    b.rho[i] = b.P[i] = b.u[i] = b.h[i] = 0.0;
    b.type[i] = BODY_STAR;
    Body &a = b.aos[i];
    a = Body{};
}

// src/quasar.c:63-101 (s: the SMBH, v: the victim)
__device__ void accrete_body(const Bodies &b, int s, int v)
{
    Body &S = b.aos[s];
    double new_mass = b.m[s] + b.m[v];
    b.vx[s] = (b.m[s] * b.vx[s] + b.m[v] * b.vx[v]) / new_mass;
    b.vy[s] = (b.m[s] * b.vy[s] + b.m[v] * b.vy[v]) / new_mass;
    b.vz[s] = (b.m[s] * b.vz[s] + b.m[v] * b.vz[v]) / new_mass;
    double rx = b.x[v] - b.x[s];
    double ry = b.y[v] - b.y[s];
    double rz = b.z[v] - b.z[s];
    double rvx = b.vx[v] - b.vx[s];
    double rvy = b.vy[v] - b.vy[s];
    double rvz = b.vz[v] - b.vz[s];
    double lx = ry * rvz - rz * rvy;
    double ly = rz * rvx - rx * rvz;
    double lz = rx * rvy - ry * rvx;
    double l_mag = sqrt(lx * lx + ly * ly + lz * lz);
    if (l_mag > 1e-15) {
        double weight = b.m[v] / new_mass * 0.01;
        S.spin_x += weight * lx / l_mag;
        S.spin_y += weight * ly / l_mag;
        S.spin_z += weight * lz / l_mag;
        double s_mag = sqrt(S.spin_x * S.spin_x + S.spin_y * S.spin_y + S.spin_z * S.spin_z);
        if (s_mag > 1e-15) {
            S.spin_x /= s_mag;
            S.spin_y /= s_mag;
            S.spin_z /= s_mag;
        }
    }
    b.m[s] = new_mass;
    b.m[v] = 0.0;
    b.vx[v] = b.vy[v] = b.vz[v] = 0.0;
    b.ax[v] = b.ay[v] = b.az[v] = 0.0;
}

// src/quasar.c:103-123
__device__ void disk_drag(const Bodies &b, int s, int g, double alpha)
{
    double rx = b.x[g] - b.x[s];
    double ry = b.y[g] - b.y[s];
    double rz = b.z[g] - b.z[s];
    double r = sqrt(rx * rx + ry * ry + rz * rz);
    if (r < 1e-15)
        return;
    double rvx = b.vx[g] - b.vx[s];
    double rvy = b.vy[g] - b.vy[s];
    double rvz = b.vz[g] - b.vz[s];
    double v_dot_r = (rvx * rx + rvy * ry + rvz * rz) / r;
    double vr_x = v_dot_r * rx / r;
    double vr_y = v_dot_r * ry / r;
    double vr_z = v_dot_r * rz / r;
    b.ax[g] -= alpha * vr_x;
    b.ay[g] -= alpha * vr_y;
    b.az[g] -= alpha * vr_z;
}

// Stage 1-2 (src/quasar.c:125-190 and :482-494): accretion, then accretion
// rate and luminosity of every SMBH. One block. smbh[]: all bodies of type
// SMBH in index order (count in q->n_smbh); cand[]: scratch.
__global__ void __launch_bounds__(QT) k_q_accretion(Bodies b, QCfg c, QuasarState *q, double dt,
                                                    int *smbh, int *cand)
{
    const int n = q->n;
    const int ns = block_compact(n, [&](int i) { return b.type[i] == BODY_SMBH; }, smbh);
    __shared__ double s_swallowed;
    if (threadIdx.x == 0) {
        q->n_smbh = ns;
        s_swallowed = 0.0;
    }
    __syncthreads();
    const double r_acc_sq = c.acc_r * c.acc_r;
    const double r_swallow_sq = c.swallow_r * c.swallow_r;
    for (int k = 0; k < ns; k++) {
        const int s = smbh[k];
        if (!(b.m[s] > 0.0)) // reference: mass <= 0.0 skips this SMBH
            continue;
        const double sx = b.x[s], sy = b.y[s], sz = b.z[s]; // positions do not change here
        const int nc = block_compact(n, [&](int i) {
            if (i == s || b.m[i] <= 0.0 || b.type[i] == BODY_SMBH)
                return false;
            const double dx = b.x[i] - sx, dy = b.y[i] - sy, dz = b.z[i] - sz;
            return !(dx * dx + dy * dy + dz * dz > r_acc_sq);
        }, cand);
        if (threadIdx.x == 0) {
            for (int j = 0; j < nc; j++) {
                const int i = cand[j];
                double dx = b.x[i] - b.x[s];
                double dy = b.y[i] - b.y[s];
                double dz = b.z[i] - b.z[s];
                double dist_sq = dx * dx + dy * dy + dz * dz;
                if (dist_sq < r_swallow_sq) {
                    s_swallowed += b.m[i];
                    accrete_body(b, s, i);
                    continue;
                }
                double r = sqrt(dist_sq);
                double rvx = b.vx[i] - b.vx[s];
                double rvy = b.vy[i] - b.vy[s];
                double rvz = b.vz[i] - b.vz[s];
                double lx = dy * rvz - dz * rvy;
                double ly = dz * rvx - dx * rvz;
                double lz = dx * rvy - dy * rvx;
                double l_sq = lx * lx + ly * ly + lz * lz;
                double r_circ = l_sq / (b.m[s] * r);
                if (r_circ > c.isco_r && b.type[i] != BODY_GAS) {
                    b.type[i] = BODY_GAS;
                    if (b.h[i] < 1e-10)
                        b.h[i] = c.acc_r * 0.3;
                    if (b.u[i] < 1e-10) {
                        double v2 = b.vx[i] * b.vx[i] + b.vy[i] * b.vy[i] + b.vz[i] * b.vz[i];
                        b.u[i] = 0.001 * v2 + 0.01;
                    }
                }
                if (b.type[i] == BODY_GAS) {
                    disk_drag(b, s, i, c.alpha);
                    if (r < c.isco_r) {
                        s_swallowed += b.m[i];
                        accrete_body(b, s, i);
                    }
                }
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double mdot_instant = s_swallowed / dt;
        for (int k = 0; k < ns; k++) {
            Body &S = b.aos[smbh[k]];
            S.accretion_rate = c.smoothing * S.accretion_rate + (1.0 - c.smoothing) * mdot_instant;
            double l_edd = c.edd_k * b.m[smbh[k]];
            S.luminosity = c.eta * S.accretion_rate;
            if (S.luminosity > l_edd)
                S.luminosity = l_edd;
        }
    }
}

// Stage 3 (src/quasar.c:192-220): radiation pressure of every luminous SMBH
// on the bodies within 3 accretion radii, added in SMBH index order.
__global__ void k_q_feedback(Bodies b, QCfg c, const QuasarState *q, const int *smbh)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = q->n, ns = q->n_smbh;
    if (i >= n || b.m[i] <= 0.0 || b.type[i] == BODY_SMBH)
        return;
    const double r_fb_sq = (c.acc_r * 3.0) * (c.acc_r * 3.0);
    for (int k = 0; k < ns; k++) {
        const int s = smbh[k];
        const double lum = b.aos[s].luminosity;
        if (lum <= 0.0)
            continue;
        double dx = b.x[i] - b.x[s];
        double dy = b.y[i] - b.y[s];
        double dz = b.z[i] - b.z[s];
        double dist_sq = dx * dx + dy * dy + dz * dz;
        if (dist_sq > r_fb_sq || dist_sq < 1e-10)
            continue;
        double r = sqrt(dist_sq);
        double f_mag = c.fb * lum / (4.0 * QPI * dist_sq);
        b.ax[i] += f_mag * dx / r;
        b.ay[i] += f_mag * dy / r;
        b.az[i] += f_mag * dz / r;
    }
}

__device__ void spawn_jets(const Bodies &b, const QCfg &c, QuasarState *q, const int *smbh,
                           int ns)
{
    q->knot_phase++;
    const int knot_phase = q->knot_phase;
    double phase_rad = knot_phase * 0.10;
    double phase_rad2 = knot_phase * 0.057;
    double speed_mod = 1.0 + 0.6 * sin(phase_rad);
    if (speed_mod < 0.5)
        speed_mod = 0.5;
    double cone_angle = 0.05 + 0.13 * (0.5 + 0.5 * sin(phase_rad2));
    double helix_phase = knot_phase * 0.04;
    for (int k = 0; k < ns; k++) {
        const int s = smbh[k];
        const Body &S = b.aos[s];
        if (S.luminosity <= 0.0)
            continue;
        double jet_energy = 0.5 * c.jet_mass * c.jet_speed * c.jet_speed;
        if (jet_energy < 1e-15)
            continue;
        int n_spawn = (int)(S.luminosity / jet_energy);
        if (n_spawn < 2)
            n_spawn = 2;
        if (n_spawn > 8)
            n_spawn = 8;
        double perp_x, perp_y, perp_z;
        if (fabs(S.spin_z) < 0.9) {
            perp_x = -S.spin_y;
            perp_y = S.spin_x;
            perp_z = 0.0;
        } else {
            perp_x = 0.0;
            perp_y = -S.spin_z;
            perp_z = S.spin_y;
        }
        double pmag = sqrt(perp_x * perp_x + perp_y * perp_y + perp_z * perp_z);
        if (pmag > 1e-15) {
            perp_x /= pmag;
            perp_y /= pmag;
            perp_z /= pmag;
        }
        double perp2_x = S.spin_y * perp_z - S.spin_z * perp_y;
        double perp2_y = S.spin_z * perp_x - S.spin_x * perp_z;
        double perp2_z = S.spin_x * perp_y - S.spin_y * perp_x;
        double pmag2 = sqrt(perp2_x * perp2_x + perp2_y * perp2_y + perp2_z * perp2_z);
        if (pmag2 > 1e-15) {
            perp2_x /= pmag2;
            perp2_y /= pmag2;
            perp2_z /= pmag2;
        }
        double helix_amp = c.swallow_r * 0.35;
        double hx = helix_amp * (cos(helix_phase) * perp_x + sin(helix_phase) * perp2_x);
        double hy = helix_amp * (cos(helix_phase) * perp_y + sin(helix_phase) * perp2_y);
        double hz = helix_amp * (cos(helix_phase) * perp_z + sin(helix_phase) * perp2_z);
        double actual_speed = c.jet_speed * speed_mod;
        int burst_extra = (speed_mod > 1.35) ? 4 : 0;
        int total_spawn = n_spawn + burst_extra;
        for (int j = 0; j < total_spawn && q->jet_count < c.jet_cap; j++) {
            if (q->n >= c.n_alloc)
                break;
            int is_burst = (j >= n_spawn);
            double sign = (j % 2 == 0) ? 1.0 : -1.0;
            double this_cone = is_burst ? 0.012 : cone_angle;
            double this_speed = is_burst ? actual_speed * 1.28 : actual_speed;
            double this_mass = is_burst ? c.jet_mass * 1.9 : c.jet_mass;
            double this_life = is_burst ? c.jet_life * 1.4 : c.jet_life;
            double axial_fwd = is_burst ? c.swallow_r * 0.6 : 0.0;
            double angle = q_uniform(q) * 2.0 * QPI;
            double offset = q_gaussian(q) * this_cone;
            int ring_n = c.ring_count;
            if (is_burst)
                ring_n = 1;
            for (int r = 0; r < ring_n; r++) {
                if (q->n >= c.n_alloc || q->jet_count >= c.jet_cap)
                    break;
                const int jt = q->n;
                zero_body(b, jt);
                b.type[jt] = BODY_JET;
                b.aos[jt].type = BODY_JET;
                b.aos[jt].lifetime = this_life;
                double ring_angle = (ring_n > 1) ? 2.0 * QPI * r / ring_n + angle : angle;
                double ring_r = (ring_n > 1) ? c.swallow_r * 0.15 : 0.0;
                double rx = ring_r * (cos(ring_angle) * perp_x + sin(ring_angle) * perp2_x);
                double ry = ring_r * (cos(ring_angle) * perp_y + sin(ring_angle) * perp2_y);
                double rz = ring_r * (cos(ring_angle) * perp_z + sin(ring_angle) * perp2_z);
                b.m[jt] = (ring_n > 1) ? this_mass * 0.6 : this_mass;
                b.x[jt] = b.x[s] + sign * S.spin_x * (c.swallow_r + axial_fwd) +
                          offset * (perp_x * cos(angle)) + sign * hx + rx;
                b.y[jt] = b.y[s] + sign * S.spin_y * (c.swallow_r + axial_fwd) +
                          offset * (perp_y * cos(angle)) + sign * hy + ry;
                b.z[jt] = b.z[s] + sign * S.spin_z * (c.swallow_r + axial_fwd) +
                          offset * (perp_z * sin(angle)) + sign * hz + rz;
                double expand_v = this_speed * 0.04 * (1.0 + b.aos[jt].lifetime * 0.1);
                b.vx[jt] = b.vx[s] + sign * S.spin_x * this_speed + rx * expand_v / (ring_r + 1e-15);
                b.vy[jt] = b.vy[s] + sign * S.spin_y * this_speed + ry * expand_v / (ring_r + 1e-15);
                b.vz[jt] = b.vz[s] + sign * S.spin_z * this_speed + rz * expand_v / (ring_r + 1e-15);
                q->n++;
                q->jet_count++;
            }
        }
    }
}

// Stages 4, 4b and 5 (src/quasar.c:375-475 and :301-373): jet decay into
// lobes, lobe decay, recycling of distant jets, jet spawning. One block.
__global__ void __launch_bounds__(QT) k_q_jets(Bodies b, QCfg c, QuasarState *q, double dt,
                                               const int *smbh, int *list)
{
    const int n0 = q->n, ns = q->n_smbh;
    // 4. jets: count down; expiring ones (in index order) spawn lobes
    for (int i = threadIdx.x; i < n0; i += QT)
        if (b.type[i] == BODY_JET && b.m[i] > 0.0)
            b.aos[i].lifetime -= dt;
    __syncthreads();
    const int ne = block_compact(n0, [&](int i) {
        return b.type[i] == BODY_JET && b.m[i] > 0.0 && b.aos[i].lifetime <= 0.0;
    }, list);
    if (threadIdx.x == 0) {
        for (int k = 0; k < ne; k++) {
            const int i = list[k];
            if (q->n < c.n_alloc && b.m[i] > 0.2) {
                const int lb = q->n;
                zero_body(b, lb);
                b.type[lb] = BODY_LOBE;
                b.aos[lb].type = BODY_LOBE;
                b.m[lb] = b.m[i] * 0.5;
                b.x[lb] = b.x[i];
                b.y[lb] = b.y[i];
                b.z[lb] = b.z[i];
                double spread = 0.5;
                b.vx[lb] = b.vx[i] * 0.15 + (q_uniform(q) - 0.5) * spread;
                b.vy[lb] = b.vy[i] * 0.15 + (q_uniform(q) - 0.5) * spread;
                b.vz[lb] = b.vz[i] * 0.15 + (q_uniform(q) - 0.5) * spread;
                b.aos[lb].lifetime = c.jet_life * 3.0;
                q->n++;
            }
            b.m[i] = 0.0;
            b.vx[i] = b.vy[i] = b.vz[i] = 0.0;
            b.ax[i] = b.ay[i] = b.az[i] = 0.0;
            q->jet_count--;
        }
    }
    __syncthreads();
    const int n1 = q->n;
    // lobes (those spawned just now too)
    for (int i = threadIdx.x; i < n1; i += QT) {
        if (b.type[i] != BODY_LOBE || b.m[i] <= 0.0)
            continue;
        b.aos[i].lifetime -= dt;
        if (b.aos[i].lifetime <= 0.0) {
            b.m[i] = 0.0;
            b.vx[i] = b.vy[i] = b.vz[i] = 0.0;
            b.ax[i] = b.ay[i] = b.az[i] = 0.0;
        }
    }
    __syncthreads();
    // 4b. jets beyond 10 accretion radii of the first live SMBH come back as gas
    __shared__ int s_first;
    if (threadIdx.x == 0) {
        s_first = -1;
        for (int k = 0; k < ns; k++)
            if (b.m[smbh[k]] > 0.0) {
                s_first = smbh[k];
                break;
            }
    }
    __syncthreads();
    const int s = s_first;
    if (s >= 0) {
        const double recycle_r = c.acc_r * 10.0;
        const double recycle_r_sq = recycle_r * recycle_r;
        const double sx = b.x[s], sy = b.y[s], sz = b.z[s];
        const int nr = block_compact(n1, [&](int i) {
            if (b.type[i] != BODY_JET || b.m[i] <= 0.0)
                return false;
            const double dx = b.x[i] - sx, dy = b.y[i] - sy, dz = b.z[i] - sz;
            return !(dx * dx + dy * dy + dz * dz < recycle_r_sq);
        }, list);
        if (threadIdx.x == 0) {
            for (int k = 0; k < nr; k++) {
                const int i = list[k];
                double angle = 2.0 * QPI * q_uniform(q);
                double cos_phi = 2.0 * q_uniform(q) - 1.0;
                double sin_phi = sqrt(1.0 - cos_phi * cos_phi);
                double r_place = c.acc_r;
                b.x[i] = b.x[s] + r_place * sin_phi * cos(angle);
                b.y[i] = b.y[s] + r_place * sin_phi * sin(angle);
                b.z[i] = b.z[s] + r_place * cos_phi;
                double v_inward = 0.5 * sqrt(b.m[s] / r_place);
                double nx = (b.x[i] - b.x[s]) / r_place;
                double ny = (b.y[i] - b.y[s]) / r_place;
                double nz = (b.z[i] - b.z[s]) / r_place;
                b.vx[i] = b.vx[s] - v_inward * nx;
                b.vy[i] = b.vy[s] - v_inward * ny;
                b.vz[i] = b.vz[s] - v_inward * nz;
                b.ax[i] = b.ay[i] = b.az[i] = 0.0;
                b.type[i] = BODY_GAS;
                b.aos[i].type = BODY_GAS;
                b.aos[i].lifetime = 0.0;
                b.h[i] = c.acc_r * 0.3;
                double v2 = b.vx[i] * b.vx[i] + b.vy[i] * b.vy[i] + b.vz[i] * b.vz[i];
                b.u[i] = 0.001 * v2 + 0.01;
                b.rho[i] = 0.0;
                b.P[i] = 0.0;
                q->jet_count--;
            }
        }
        __syncthreads();
    }
    // 5. spawning
    if (threadIdx.x == 0)
        spawn_jets(b, c, q, smbh, ns);
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

} // namespace

extern "C" int csgd_quasar_state(csgd_t *d, unsigned long long rng, int knot_phase)
{
    if (!d->qs && cudaMalloc((void **)&d->qs, sizeof(QuasarState)) != cudaSuccess) {
        cudaGetLastError();
        csgd_set_err(d, CSG_ERR_NOMEM);
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
    if (n_alloc > d->cap || d->n_gal > 1) {
        csgd_set_err(d, d->n_gal > 1 ? CSG_ERR_UNSUPPORTED : CSG_ERR_BAD_ARG);
        return d->n_gal > 1 ? CSG_ERR_UNSUPPORTED : CSG_ERR_BAD_ARG;
    }
    cudaStream_t s = d->stream;
    // body count and jet count in, the step may append bodies
    int *hi = d->h_int;
    hi[0] = d->n;
    hi[1] = *jet_count;
    cudaMemcpyAsync(&d->qs->n, &hi[0], sizeof(int), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(&d->qs->jet_count, &hi[1], sizeof(int), cudaMemcpyHostToDevice, s);
    Bodies b{d->x, d->y, d->z, d->vx, d->vy, d->vz, d->ax, d->ay, d->az, d->m,
             d->rho, d->P, d->u, d->h, d->type, d->aos};
    QCfg c = qcfg(cfg, n_alloc);
    int *smbh = d->cnt, *list = d->base; // tree scratch: free between builds
    { k_q_accretion<<<1, QT, 0, s>>>(b, c, d->qs, dt, smbh, list); d->launches++; }
    { k_q_feedback<<<csgd_grid(n_alloc > 0 ? n_alloc : 1, 256), 256, 0, s>>>(b, c, d->qs, smbh); d->launches++; }
    { k_q_jets<<<1, QT, 0, s>>>(b, c, d->qs, dt, smbh, list); d->launches++; }
    cudaMemcpyAsync(&hi[2], &d->qs->n, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&hi[3], &d->qs->jet_count, sizeof(int), cudaMemcpyDeviceToHost, s);
    int rc = csgd_sync(d);
    if (rc)
        return rc;
    d->n = hi[2];
    *jet_count = hi[3];
    *n_out = hi[2];
    d->geometry_valid = 0;
    d->gas_valid = 0;
    return CSG_OK;
}
