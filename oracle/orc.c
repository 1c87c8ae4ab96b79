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
