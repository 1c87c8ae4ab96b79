/*
 * orc.c — CPU oracle (test infrastructure only; see orc.h).
 *
 * A restatement, written for this project, of cosmosim's double-precision
 * Barnes-Hut / SPH / leapfrog path. Recursion in the reference is replaced by
 * explicit stacks that visit cells in the same depth-first octant order, so
 * accumulation order — and with -ffp-contract=off every rounding — matches the
 * reference. Each function names the reference lines it follows.
 */
#include "orc.h"

#include <float.h>
#include <math.h>
#include <stddef.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAX_DEPTH 64 /* reference src/octree.c:5 */
#define ORC_STACK 520    /* > 64 levels x 7 pending siblings + 8 */
#define ORC_PI 3.14159265358979323846

int orc_set_threads(int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
    return omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

/* ---- tree construction: reference src/octree.c:7-169 ---------------------- */

static int orc_new_cell(OctreeNode *pool, int *pool_size, double x, double y, double z, double hs)
{
    int id = *pool_size;
    *pool_size = id + 1;
    OctreeNode *c = pool + id;
    c->cx = c->cy = c->cz = 0.0;
    c->total_mass = 0.0;
    c->center_x = x;
    c->center_y = y;
    c->center_z = z;
    c->half_size = hs;
    c->body_index = -1;
    for (int q = 0; q < 8; q++)
        c->children[q] = -1;
    return id;
}

/* Octant code of a point in a cell: +1 east (x >= c), +2 south (y < c),
   +4 bottom (z < c) — reference src/octree.c:30-40. */
static int orc_octant(const OctreeNode *c, double x, double y, double z)
{
    return (x >= c->center_x ? 1 : 0) | (y < c->center_y ? 2 : 0) | (z < c->center_z ? 4 : 0);
}

/* Creates the child cell of octant q — geometry of reference src/octree.c:42-50,
   87-90 and 105-108: child centre = centre +/- 0.5 * half_size per axis. */
static int orc_make_child(OctreeNode *pool, int *pool_size, int parent, int q)
{
    const OctreeNode *p = pool + parent;
    double ox = (q & 1) ? 0.5 : -0.5;
    double oy = (q & 2) ? -0.5 : 0.5;
    double oz = (q & 4) ? -0.5 : 0.5;
    double hs = p->half_size * 0.5;
    double x = p->center_x + ox * p->half_size;
    double y = p->center_y + oy * p->half_size;
    double z = p->center_z + oz * p->half_size;
    int id = orc_new_cell(pool, pool_size, x, y, z, hs);
    pool[parent].children[q] = id;
    return id;
}

/* Running mass-weighted centre update, reference src/octree.c:73-77, 95-100. */
static void orc_absorb(OctreeNode *c, double x, double y, double z, double m)
{
    double mt = c->total_mass + m;
    c->cx = (c->cx * c->total_mass + x * m) / mt;
    c->cy = (c->cy * c->total_mass + y * m) / mt;
    c->cz = (c->cz * c->total_mass + z * m) / mt;
    c->total_mass = mt;
}

static void orc_put(OctreeNode *c, const Body *b, int bi)
{
    c->body_index = bi;
    c->cx = b->x;
    c->cy = b->y;
    c->cz = b->z;
    c->total_mass = b->mass;
}

/* Iterative form of the reference's recursive insert (src/octree.c:52-112). */
static void orc_insert(OctreeNode *pool, int *pool_size, const Body *bodies, int bi)
{
    const Body *b = bodies + bi;
    int cell = 0;
    for (int depth = 0;; depth++) {
        OctreeNode *c = pool + cell;
        if (c->total_mass == 0.0 && c->body_index == -1) {
            orc_put(c, b, bi);
            return;
        }
        if (depth >= ORC_MAX_DEPTH) {
            orc_absorb(c, b->x, b->y, b->z, b->mass);
            return;
        }
        if (c->body_index >= 0) {
            /* split a leaf: its body moves one level down first */
            int old = c->body_index;
            c->body_index = -1;
            const Body *o = bodies + old;
            int q_old = orc_octant(c, o->x, o->y, o->z);
            int child = orc_make_child(pool, pool_size, cell, q_old);
            orc_put(pool + child, o, old);
            c = pool + cell;
        }
        orc_absorb(c, b->x, b->y, b->z, b->mass);
        int q = orc_octant(c, b->x, b->y, b->z);
        int next = c->children[q];
        if (next < 0)
            next = orc_make_child(pool, pool_size, cell, q);
        cell = next;
    }
}

void orc_octree_build(OctreeNode *pool, int *pool_size, const Body *bodies, int n)
{
    *pool_size = 0;
    double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX};
    double hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
    int alive = 0;
    for (int i = 0; i < n; i++) {
        const Body *b = bodies + i;
        if (b->mass <= 0.0)
            continue;
        alive++;
        double p[3] = {b->x, b->y, b->z};
        for (int a = 0; a < 3; a++) {
            if (p[a] < lo[a])
                lo[a] = p[a];
            if (p[a] > hi[a])
                hi[a] = p[a];
        }
    }
    if (alive == 0) { /* reference src/octree.c:141-144 */
        orc_new_cell(pool, pool_size, 0.0, 0.0, 0.0, 1.0);
        return;
    }
    /* root cube, reference src/octree.c:146-159 */
    double ext = hi[0] - lo[0];
    if (hi[1] - lo[1] > ext)
        ext = hi[1] - lo[1];
    if (hi[2] - lo[2] > ext)
        ext = hi[2] - lo[2];
    double hs = ext * 0.5 * 1.01;
    if (hs < 1e-10)
        hs = 1.0;
    orc_new_cell(pool, pool_size, (lo[0] + hi[0]) * 0.5, (lo[1] + hi[1]) * 0.5,
                 (lo[2] + hi[2]) * 0.5, hs);
    for (int i = 0; i < n; i++)
        if (bodies[i].mass > 0.0)
            orc_insert(pool, pool_size, bodies, i);
}

/* ---- force walk: reference src/octree.c:171-234 --------------------------- */

/* Depth-first walk of one body; children pushed 7..0 so they pop 0..7. */
static void orc_walk_body(const OctreeNode *pool, int root, Body *b, int bi, double G,
                          double eps2, double theta2, int64_t *count)
{
    int stack[ORC_STACK];
    int sp = 0;
    double ax = 0.0, ay = 0.0, az = 0.0;
    int64_t hits = 0;
    stack[sp++] = root;
    while (sp > 0) {
        const OctreeNode *c = pool + stack[--sp];
        if (c->total_mass == 0.0)
            continue;
        double dx = c->cx - b->x;
        double dy = c->cy - b->y;
        double dz = c->cz - b->z;
        double d2 = dx * dx + dy * dy + dz * dz;
        int take;
        if (c->body_index >= 0) {
            take = (c->body_index != bi);
            if (!take)
                continue;
        } else {
            double s = 2.0 * c->half_size;
            take = (d2 > 0.0 && (s * s) / d2 < theta2);
        }
        if (take) {
            double r2 = d2 + eps2;
            double inv_r3 = 1.0 / (r2 * sqrt(r2));
            ax += G * c->total_mass * dx * inv_r3;
            ay += G * c->total_mass * dy * inv_r3;
            az += G * c->total_mass * dz * inv_r3;
            hits++;
            continue;
        }
        for (int q = 7; q >= 0; q--)
            if (c->children[q] >= 0)
                stack[sp++] = c->children[q];
    }
    b->ax = ax;
    b->ay = ay;
    b->az = az;
    if (count)
        *count = hits;
}

void orc_octree_compute_forces(const OctreeNode *pool, int root, Body *bodies, int n, double G,
                               double softening, double theta)
{
    double eps2 = softening * softening;
    double theta2 = theta * theta;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < n; i++) {
        bodies[i].ax = 0.0;
        bodies[i].ay = 0.0;
        bodies[i].az = 0.0;
        if (bodies[i].mass <= 0.0)
            continue;
        orc_walk_body(pool, root, bodies + i, i, G, eps2, theta2, NULL);
    }
}

int64_t orc_octree_count_interactions(const OctreeNode *pool, int root, const Body *bodies,
                                      int n, double theta, int32_t *per_body)
{
    double theta2 = theta * theta;
    int64_t total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
    for (int i = 0; i < n; i++) {
        int64_t hits = 0;
        if (bodies[i].mass > 0.0) {
            Body tmp = bodies[i];
            orc_walk_body(pool, root, &tmp, i, 1.0, 1.0, theta2, &hits);
        }
        if (per_body)
            per_body[i] = (int32_t)hits;
        total += hits;
    }
    return total;
}

/* ---- neighbour search: reference src/octree.c:236-318 --------------------- */

int orc_octree_find_neighbors(const OctreeNode *pool, int root, const Body *bodies, int n,
                              double cx, double cy, double cz, double radius, int *buf,
                              int capacity)
{
    (void)n;
    double r2 = radius * radius;
    int stack[ORC_STACK];
    int sp = 0, count = 0;
    stack[sp++] = root;
    while (sp > 0 && count < capacity) {
        const OctreeNode *c = pool + stack[--sp];
        double gx = fmax(0.0, fabs(cx - c->center_x) - c->half_size);
        double gy = fmax(0.0, fabs(cy - c->center_y) - c->half_size);
        double gz = fmax(0.0, fabs(cz - c->center_z) - c->half_size);
        if (gx * gx + gy * gy + gz * gz > r2)
            continue;
        if (c->body_index >= 0) {
            const Body *b = bodies + c->body_index;
            if (b->mass <= 0.0)
                continue;
            double bx = b->x - cx;
            double by = b->y - cy;
            double bz = b->z - cz;
            if (bx * bx + by * by + bz * bz <= r2)
                buf[count++] = c->body_index;
            continue;
        }
        for (int q = 7; q >= 0; q--)
            if (c->children[q] >= 0)
                stack[sp++] = c->children[q];
    }
    return count;
}

/* ---- SPH: reference src/sph.c ---------------------------------------------- */

/* M4 cubic spline, reference src/sph.c:11-25 */
static double orc_W(double r, double h)
{
    if (h < 1e-10)
        return 0.0;
    double q = r / h;
    if (q > 1.0)
        return 0.0;
    double norm = 8.0 / (ORC_PI * h * h * h);
    if (q <= 0.5)
        return norm * (1.0 - 6.0 * q * q + 6.0 * q * q * q);
    double t = 1.0 - q;
    return norm * 2.0 * t * t * t;
}

/* its radial derivative, reference src/sph.c:27-41 */
static double orc_dWdr(double r, double h)
{
    if (h < 1e-10)
        return 0.0;
    double q = r / h;
    if (q > 1.0 || r < 1e-15)
        return 0.0;
    double norm = 8.0 / (ORC_PI * h * h * h);
    if (q <= 0.5)
        return norm * (-12.0 * q + 18.0 * q * q) / h;
    double t = 1.0 - q;
    return norm * (-6.0 * t * t) / h;
}

/* reference src/sph.c:45-97 */
void orc_sph_compute_density(Body *bodies, int n, const OctreeNode *tree)
{
#pragma omp parallel for schedule(dynamic)
    for (int i = 0; i < n; i++) {
        Body *bi = bodies + i;
        if (bi->type != BODY_GAS || bi->mass <= 0.0)
            continue;
        int nb[CSG_SPH_MAX_NEIGHBORS];
        double h = bi->smoothing_h;
        int nn = orc_octree_find_neighbors(tree, 0, bodies, n, bi->x, bi->y, bi->z, h, nb,
                                           CSG_SPH_MAX_NEIGHBORS);
        if (nn < 20 && h < 50.0)
            bi->smoothing_h = h * 1.2;
        else if (nn > 48 && h > 0.1)
            bi->smoothing_h = h * 0.8;
        double rho = 0.0;
        for (int k = 0; k < nn; k++) {
            const Body *bj = bodies + nb[k];
            if (bj->mass <= 0.0)
                continue;
            double dx = bi->x - bj->x;
            double dy = bi->y - bj->y;
            double dz = bi->z - bj->z;
            double r = sqrt(dx * dx + dy * dy + dz * dz);
            rho += bj->mass * orc_W(r, h);
        }
        if (rho < 1e-15 || isnan(rho))
            rho = 1e-15;
        bi->density = rho;
        double u = bi->internal_energy;
        if (u < 1e-15)
            u = 1e-15;
        bi->pressure = (CSG_SPH_GAMMA - 1.0) * rho * u;
    }
}

/* reference src/sph.c:101-196 */
void orc_sph_compute_forces(Body *bodies, int n, const OctreeNode *tree)
{
#pragma omp parallel for schedule(dynamic)
    for (int i = 0; i < n; i++) {
        Body *bi = bodies + i;
        if (bi->type != BODY_GAS || bi->mass <= 0.0)
            continue;
        int nb[CSG_SPH_MAX_NEIGHBORS];
        double h_i = bi->smoothing_h;
        double rho_i = bi->density;
        double P_i = bi->pressure;
        double c_i = sqrt(CSG_SPH_GAMMA * P_i / (rho_i + 1e-15));
        int nn = orc_octree_find_neighbors(tree, 0, bodies, n, bi->x, bi->y, bi->z, h_i, nb,
                                           CSG_SPH_MAX_NEIGHBORS);
        double sx = 0.0, sy = 0.0, sz = 0.0;
        for (int k = 0; k < nn; k++) {
            int j = nb[k];
            const Body *bj = bodies + j;
            if (j == i || bj->mass <= 0.0 || bj->type != BODY_GAS)
                continue;
            double dx = bi->x - bj->x;
            double dy = bi->y - bj->y;
            double dz = bi->z - bj->z;
            double r = sqrt(dx * dx + dy * dy + dz * dz);
            if (r < 1e-15)
                continue;
            double h_avg = 0.5 * (h_i + bj->smoothing_h);
            double rho_j = bj->density;
            double P_j = bj->pressure;
            double dvx = bi->vx - bj->vx;
            double dvy = bi->vy - bj->vy;
            double dvz = bi->vz - bj->vz;
            double vr = dvx * dx + dvy * dy + dvz * dz;
            double visc = 0.0;
            if (vr < 0.0) {
                double mu = h_avg * vr / (r * r + 0.01 * h_avg * h_avg);
                double c_j = sqrt(CSG_SPH_GAMMA * P_j / (rho_j + 1e-15));
                double c_avg = 0.5 * (c_i + c_j);
                double rho_avg = 0.5 * (rho_i + rho_j);
                visc = (-1.0 * c_avg * mu + 2.0 * mu * mu) / (rho_avg + 1e-15);
            }
            double g = orc_dWdr(r, h_avg);
            double gx = g * dx / r;
            double gy = g * dy / r;
            double gz = g * dz / r;
            double f = bj->mass * (P_i / (rho_i * rho_i + 1e-15) + P_j / (rho_j * rho_j + 1e-15) +
                                   visc);
            sx -= f * gx;
            sy -= f * gy;
            sz -= f * gz;
        }
        if (isnan(sx))
            sx = 0.0;
        if (isnan(sy))
            sy = 0.0;
        if (isnan(sz))
            sz = 0.0;
        bi->ax += sx * 0.1;
        bi->ay += sy * 0.1;
        bi->az += sz * 0.1;
    }
}

/* reference src/sph.c:200-231 */
void orc_sph_apply_cooling(Body *bodies, int n, double dt)
{
    const double lambda0 = 0.05;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        Body *b = bodies + i;
        if (b->type != BODY_GAS || b->mass <= 0.0)
            continue;
        double u = b->internal_energy;
        double rho = b->density;
        if (u < 1e-15 || rho < 1e-15)
            continue;
        double u_new = u / (1.0 + dt * lambda0 * rho * 0.5 / sqrt(u));
        if (u_new < 0.01)
            u_new = 0.01;
        b->internal_energy = u_new;
        b->pressure = (CSG_SPH_GAMMA - 1.0) * rho * u_new;
    }
}

/* ---- leapfrog: reference src/integrator.c ---------------------------------- */

void orc_integrator_init_accelerations(Body *bodies, int n, double G, double softening,
                                       double theta, OctreeNode *pool)
{
    int ps = 0;
    orc_octree_build(pool, &ps, bodies, n);
    orc_octree_compute_forces(pool, 0, bodies, n, G, softening, theta);
}

void orc_integrator_step(Body *bodies, int n, double dt, double G, double softening,
                         double theta, OctreeNode *pool, int sph_enabled)
{
    for (int i = 0; i < n; i++) { /* half kick + drift, :22-31 */
        Body *b = bodies + i;
        if (b->mass <= 0.0)
            continue;
        b->vx += 0.5 * b->ax * dt;
        b->vy += 0.5 * b->ay * dt;
        b->vz += 0.5 * b->az * dt;
        b->x += b->vx * dt;
        b->y += b->vy * dt;
        b->z += b->vz * dt;
    }
    int ps = 0;
    orc_octree_build(pool, &ps, bodies, n);
    orc_octree_compute_forces(pool, 0, bodies, n, G, softening, theta);
    if (sph_enabled) {
        orc_sph_compute_density(bodies, n, pool);
        orc_sph_compute_forces(bodies, n, pool);
    }
    for (int i = 0; i < n; i++) { /* half kick, :45-51 */
        Body *b = bodies + i;
        if (b->mass <= 0.0)
            continue;
        b->vx += 0.5 * b->ax * dt;
        b->vy += 0.5 * b->ay * dt;
        b->vz += 0.5 * b->az * dt;
    }
    if (sph_enabled)
        orc_sph_apply_cooling(bodies, n, dt);
}

/* ---- checks: reference tests/test_physics.c:34-71 -------------------------- */

void orc_direct_forces(const Body *bodies, int n, const int32_t *idx, int m, double G,
                       double softening, double *acc)
{
    double eps2 = softening * softening;
    int cnt = idx ? m : n;
#pragma omp parallel for schedule(dynamic, 16)
    for (int k = 0; k < cnt; k++) {
        int i = idx ? idx[k] : k;
        const Body *bi = bodies + i;
        double ax = 0.0, ay = 0.0, az = 0.0;
        for (int j = 0; j < n; j++) {
            if (j == i)
                continue;
            const Body *bj = bodies + j;
            double dx = bj->x - bi->x;
            double dy = bj->y - bi->y;
            double dz = bj->z - bi->z;
            double r2 = dx * dx + dy * dy + dz * dz + eps2;
            double inv_r3 = 1.0 / (r2 * sqrt(r2));
            ax += G * bj->mass * dx * inv_r3;
            ay += G * bj->mass * dy * inv_r3;
            az += G * bj->mass * dz * inv_r3;
        }
        acc[3 * k + 0] = ax;
        acc[3 * k + 1] = ay;
        acc[3 * k + 2] = az;
    }
}

double orc_total_energy(const Body *bodies, int n, double G, double softening)
{
    double ke = 0.0;
    for (int i = 0; i < n; i++) {
        const Body *b = bodies + i;
        ke += 0.5 * b->mass * (b->vx * b->vx + b->vy * b->vy + b->vz * b->vz);
    }
    double pe = 0.0;
    for (int i = 0; i < n; i++) {
        for (int j = i + 1; j < n; j++) {
            double dx = bodies[j].x - bodies[i].x;
            double dy = bodies[j].y - bodies[i].y;
            double dz = bodies[j].z - bodies[i].z;
            double r = sqrt(dx * dx + dy * dy + dz * dz + softening * softening);
            pe -= G * bodies[i].mass * bodies[j].mass / r;
        }
    }
    return ke + pe;
}

/* ---- quasar step (reference src/quasar.c) ----------------------------------- */

static uint64_t q_state = 1;  /* src/quasar.c:11 */
static int q_knot_phase = 0; /* src/quasar.c:224 */

void orc_quasar_seed(uint64_t rng_state, int knot_phase)
{
    q_state = rng_state ? rng_state : 1;
    q_knot_phase = knot_phase;
}

static double q_uni(void) /* src/quasar.c:13-27: xorshift64 13/7/17, 53-bit uniform */
{
    uint64_t x = q_state;
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    q_state = x;
    return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

static double q_gauss(void) /* src/quasar.c:29-35: Box-Muller, first output */
{
    double u1 = q_uni(), u2 = q_uni();
    if (u1 < 1e-15)
        u1 = 1e-15;
    return sqrt(-2.0 * log(u1)) * cos(2.0 * ORC_PI * u2);
}

static void q_kill(Body *b)
{
    b->mass = 0.0;
    b->vx = b->vy = b->vz = 0.0;
    b->ax = b->ay = b->az = 0.0;
}

/* src/quasar.c:63-101: momentum-conserving merge, spin nudged by the
   victim's specific angular momentum direction. */
static void q_swallow(Body *s, Body *v)
{
    double mt = s->mass + v->mass;
    s->vx = (s->mass * s->vx + v->mass * v->vx) / mt;
    s->vy = (s->mass * s->vy + v->mass * v->vy) / mt;
    s->vz = (s->mass * s->vz + v->mass * v->vz) / mt;
    double rx = v->x - s->x, ry = v->y - s->y, rz = v->z - s->z;
    double ux = v->vx - s->vx, uy = v->vy - s->vy, uz = v->vz - s->vz;
    double lx = ry * uz - rz * uy, ly = rz * ux - rx * uz, lz = rx * uy - ry * ux;
    double lm = sqrt(lx * lx + ly * ly + lz * lz);
    if (lm > 1e-15) {
        double w = v->mass / mt * 0.01;
        s->spin_x += w * lx / lm;
        s->spin_y += w * ly / lm;
        s->spin_z += w * lz / lm;
        double sm = sqrt(s->spin_x * s->spin_x + s->spin_y * s->spin_y + s->spin_z * s->spin_z);
        if (sm > 1e-15) {
            s->spin_x /= sm;
            s->spin_y /= sm;
            s->spin_z /= sm;
        }
    }
    s->mass = mt;
    q_kill(v);
}

/* src/quasar.c:103-123: drag on the radial velocity component */
static void q_drag(const Body *s, Body *g, double alpha)
{
    double rx = g->x - s->x, ry = g->y - s->y, rz = g->z - s->z;
    double r = sqrt(rx * rx + ry * ry + rz * rz);
    if (r < 1e-15)
        return;
    double ux = g->vx - s->vx, uy = g->vy - s->vy, uz = g->vz - s->vz;
    double vr = (ux * rx + uy * ry + uz * rz) / r;
    g->ax -= alpha * (vr * rx / r);
    g->ay -= alpha * (vr * ry / r);
    g->az -= alpha * (vr * rz / r);
}

/* src/quasar.c:125-190 */
static double q_accrete(Body *b, int n, const QuasarConfig *c)
{
    double swallowed = 0.0;
    double ra2 = c->accretion_radius * c->accretion_radius;
    double rs2 = c->swallow_radius * c->swallow_radius;
    for (int s = 0; s < n; s++) {
        if (b[s].type != BODY_SMBH || b[s].mass <= 0.0)
            continue;
        Body *S = &b[s];
        for (int i = 0; i < n; i++) {
            if (i == s || b[i].mass <= 0.0 || b[i].type == BODY_SMBH)
                continue;
            double dx = b[i].x - S->x, dy = b[i].y - S->y, dz = b[i].z - S->z;
            double d2 = dx * dx + dy * dy + dz * dz;
            if (d2 > ra2)
                continue;
            if (d2 < rs2) {
                swallowed += b[i].mass;
                q_swallow(S, &b[i]);
                continue;
            }
            double r = sqrt(d2);
            double ux = b[i].vx - S->vx, uy = b[i].vy - S->vy, uz = b[i].vz - S->vz;
            double lx = dy * uz - dz * uy, ly = dz * ux - dx * uz, lz = dx * uy - dy * ux;
            double rc = (lx * lx + ly * ly + lz * lz) / (S->mass * r);
            if (rc > c->isco_radius && b[i].type != BODY_GAS) {
                b[i].type = BODY_GAS;
                if (b[i].smoothing_h < 1e-10)
                    b[i].smoothing_h = c->accretion_radius * 0.3;
                if (b[i].internal_energy < 1e-10) {
                    double v2 = b[i].vx * b[i].vx + b[i].vy * b[i].vy + b[i].vz * b[i].vz;
                    b[i].internal_energy = 0.001 * v2 + 0.01;
                }
            }
            if (b[i].type == BODY_GAS) {
                q_drag(S, &b[i], c->viscosity_alpha);
                if (r < c->isco_radius) {
                    swallowed += b[i].mass;
                    q_swallow(S, &b[i]);
                }
            }
        }
    }
    return swallowed;
}

/* src/quasar.c:192-220 */
static void q_feedback(Body *b, int n, const QuasarConfig *c)
{
    double rf2 = (c->accretion_radius * 3.0) * (c->accretion_radius * 3.0);
    for (int s = 0; s < n; s++) {
        if (b[s].type != BODY_SMBH || b[s].luminosity <= 0.0)
            continue;
        for (int i = 0; i < n; i++) {
            if (i == s || b[i].mass <= 0.0 || b[i].type == BODY_SMBH)
                continue;
            double dx = b[i].x - b[s].x, dy = b[i].y - b[s].y, dz = b[i].z - b[s].z;
            double d2 = dx * dx + dy * dy + dz * dz;
            if (d2 > rf2 || d2 < 1e-10)
                continue;
            double r = sqrt(d2);
            double f = c->feedback_strength * b[s].luminosity / (4.0 * ORC_PI * d2);
            b[i].ax += f * dx / r;
            b[i].ay += f * dy / r;
            b[i].az += f * dz / r;
        }
    }
}

/* src/quasar.c:222-373: knots (speed/cone modulation), helical offset, rings */
static void q_spawn(Body *b, int *n, int n_alloc, QuasarConfig *c)
{
    q_knot_phase++;
    double ph1 = q_knot_phase * 0.10, ph2 = q_knot_phase * 0.057;
    double speed_mod = 1.0 + 0.6 * sin(ph1);
    if (speed_mod < 0.5)
        speed_mod = 0.5;
    double cone = 0.05 + 0.13 * (0.5 + 0.5 * sin(ph2));
    double helix = q_knot_phase * 0.04;
    for (int s = 0; s < *n; s++) {
        if (b[s].type != BODY_SMBH || b[s].luminosity <= 0.0)
            continue;
        const Body *S = &b[s];
        double e_jet = 0.5 * c->jet_mass * c->jet_speed * c->jet_speed;
        if (e_jet < 1e-15)
            continue;
        int ns = (int)(S->luminosity / e_jet);
        ns = ns < 2 ? 2 : (ns > 8 ? 8 : ns);
        double px, py, pz;
        if (fabs(S->spin_z) < 0.9) {
            px = -S->spin_y;
            py = S->spin_x;
            pz = 0.0;
        } else {
            px = 0.0;
            py = -S->spin_z;
            pz = S->spin_y;
        }
        double pm = sqrt(px * px + py * py + pz * pz);
        if (pm > 1e-15) {
            px /= pm;
            py /= pm;
            pz /= pm;
        }
        double qx = S->spin_y * pz - S->spin_z * py;
        double qy = S->spin_z * px - S->spin_x * pz;
        double qz = S->spin_x * py - S->spin_y * px;
        double qm = sqrt(qx * qx + qy * qy + qz * qz);
        if (qm > 1e-15) {
            qx /= qm;
            qy /= qm;
            qz /= qm;
        }
        double amp = c->swallow_radius * 0.35;
        double hx = amp * (cos(helix) * px + sin(helix) * qx);
        double hy = amp * (cos(helix) * py + sin(helix) * qy);
        double hz = amp * (cos(helix) * pz + sin(helix) * qz);
        double speed = c->jet_speed * speed_mod;
        int total = ns + ((speed_mod > 1.35) ? 4 : 0);
        for (int j = 0; j < total && c->jet_count < c->jet_cap; j++) {
            if (*n >= n_alloc)
                break;
            int burst = j >= ns;
            double sign = (j % 2 == 0) ? 1.0 : -1.0;
            double jcone = burst ? 0.012 : cone;
            double jspeed = burst ? speed * 1.28 : speed;
            double jmass = burst ? c->jet_mass * 1.9 : c->jet_mass;
            double jlife = burst ? c->jet_lifetime * 1.4 : c->jet_lifetime;
            double fwd = burst ? c->swallow_radius * 0.6 : 0.0;
            double angle = q_uni() * 2.0 * ORC_PI;
            double offset = q_gauss() * jcone;
            int ring = burst ? 1 : c->jet_ring_count;
            for (int r = 0; r < ring; r++) {
                if (*n >= n_alloc || c->jet_count >= c->jet_cap)
                    break;
                Body *J = &b[*n];
                memset(J, 0, sizeof(Body));
                J->type = BODY_JET;
                J->lifetime = jlife;
                double ra = (ring > 1) ? 2.0 * ORC_PI * r / ring + angle : angle;
                double rr = (ring > 1) ? c->swallow_radius * 0.15 : 0.0;
                double rx = rr * (cos(ra) * px + sin(ra) * qx);
                double ry = rr * (cos(ra) * py + sin(ra) * qy);
                double rz = rr * (cos(ra) * pz + sin(ra) * qz);
                J->mass = (ring > 1) ? jmass * 0.6 : jmass;
                J->x = S->x + sign * S->spin_x * (c->swallow_radius + fwd) +
                       offset * (px * cos(angle)) + sign * hx + rx;
                J->y = S->y + sign * S->spin_y * (c->swallow_radius + fwd) +
                       offset * (py * cos(angle)) + sign * hy + ry;
                J->z = S->z + sign * S->spin_z * (c->swallow_radius + fwd) +
                       offset * (pz * sin(angle)) + sign * hz + rz;
                double ev = jspeed * 0.04 * (1.0 + J->lifetime * 0.1);
                J->vx = S->vx + sign * S->spin_x * jspeed + rx * ev / (rr + 1e-15);
                J->vy = S->vy + sign * S->spin_y * jspeed + ry * ev / (rr + 1e-15);
                J->vz = S->vz + sign * S->spin_z * jspeed + rz * ev / (rr + 1e-15);
                (*n)++;
                c->jet_count++;
            }
        }
    }
}

/* src/quasar.c:375-420: jets count down and leave a lobe; lobes count down */
static void q_decay(Body *b, int *n, int n_alloc, QuasarConfig *c, double dt)
{
    int n0 = *n;
    for (int i = 0; i < n0; i++) {
        if (b[i].type != BODY_JET || b[i].mass <= 0.0)
            continue;
        b[i].lifetime -= dt;
        if (b[i].lifetime > 0.0)
            continue;
        if (*n < n_alloc && b[i].mass > 0.2) {
            Body *L = &b[*n];
            memset(L, 0, sizeof(Body));
            L->type = BODY_LOBE;
            L->mass = b[i].mass * 0.5;
            L->x = b[i].x;
            L->y = b[i].y;
            L->z = b[i].z;
            L->vx = b[i].vx * 0.15 + (q_uni() - 0.5) * 0.5;
            L->vy = b[i].vy * 0.15 + (q_uni() - 0.5) * 0.5;
            L->vz = b[i].vz * 0.15 + (q_uni() - 0.5) * 0.5;
            L->lifetime = c->jet_lifetime * 3.0;
            (*n)++;
        }
        q_kill(&b[i]);
        c->jet_count--;
    }
    for (int i = 0; i < *n; i++) {
        if (b[i].type != BODY_LOBE || b[i].mass <= 0.0)
            continue;
        b[i].lifetime -= dt;
        if (b[i].lifetime <= 0.0)
            q_kill(&b[i]);
    }
}

/* src/quasar.c:422-475: jets beyond 10 accretion radii of the first SMBH
   return as infalling gas on the accretion sphere */
static void q_recycle(Body *b, int n, QuasarConfig *c)
{
    int s = -1;
    for (int i = 0; i < n && s < 0; i++)
        if (b[i].type == BODY_SMBH && b[i].mass > 0.0)
            s = i;
    if (s < 0)
        return;
    const Body *S = &b[s];
    double R = c->accretion_radius * 10.0;
    for (int i = 0; i < n; i++) {
        if (b[i].type != BODY_JET || b[i].mass <= 0.0)
            continue;
        double dx = b[i].x - S->x, dy = b[i].y - S->y, dz = b[i].z - S->z;
        if (dx * dx + dy * dy + dz * dz < R * R)
            continue;
        double angle = 2.0 * ORC_PI * q_uni();
        double cp = 2.0 * q_uni() - 1.0;
        double sp = sqrt(1.0 - cp * cp);
        double rp = c->accretion_radius;
        b[i].x = S->x + rp * sp * cos(angle);
        b[i].y = S->y + rp * sp * sin(angle);
        b[i].z = S->z + rp * cp;
        double vin = 0.5 * sqrt(S->mass / rp);
        double nx = (b[i].x - S->x) / rp, ny = (b[i].y - S->y) / rp, nz = (b[i].z - S->z) / rp;
        b[i].vx = S->vx - vin * nx;
        b[i].vy = S->vy - vin * ny;
        b[i].vz = S->vz - vin * nz;
        b[i].ax = b[i].ay = b[i].az = 0.0;
        b[i].type = BODY_GAS;
        b[i].lifetime = 0.0;
        b[i].smoothing_h = c->accretion_radius * 0.3;
        double v2 = b[i].vx * b[i].vx + b[i].vy * b[i].vy + b[i].vz * b[i].vz;
        b[i].internal_energy = 0.001 * v2 + 0.01;
        b[i].density = 0.0;
        b[i].pressure = 0.0;
        c->jet_count--;
    }
}

void orc_quasar_step(Body *bodies, int *n, int n_alloc, QuasarConfig *cfg, double dt)
{
    double swallowed = q_accrete(bodies, *n, cfg);
    for (int i = 0; i < *n; i++) { /* src/quasar.c:482-494 */
        if (bodies[i].type != BODY_SMBH)
            continue;
        Body *S = &bodies[i];
        S->accretion_rate = cfg->accretion_smoothing * S->accretion_rate +
                            (1.0 - cfg->accretion_smoothing) * (swallowed / dt);
        S->luminosity = cfg->eta_eff * S->accretion_rate;
        if (S->luminosity > cfg->eddington_k * S->mass)
            S->luminosity = cfg->eddington_k * S->mass;
    }
    q_feedback(bodies, *n, cfg);
    q_decay(bodies, n, n_alloc, cfg, dt);
    q_recycle(bodies, *n, cfg);
    q_spawn(bodies, n, n_alloc, cfg);
}
