/*
 * ics.c — seeded initial conditions.
 *
 * The reference draws its galaxies with a time-seeded xorshift64 generator
 * (src/initial_conditions.c:8-38). Here the same published generator
 * (Marsaglia xorshift, shifts 13/7/17; 53-bit uniforms; Box-Muller normals)
 * is seeded explicitly so every run is reproducible.
 *
 * Two families:
 *   csg_ref_spiral / csg_ref_merger: the reference's own galaxy recipe
 *     (src/initial_conditions.c:40-144), used by cosmosim_create when the
 *     application does not link the reference's generators;
 *   csg_generate_ics kinds 0-6: the benchmark configurations (exponential
 *     disks with the given scale lengths and masses, a Plummer bulge drawn by
 *     the Aarseth-Henon-Wielen (1974) rejection method, a tilted merger).
 */
#include "capi_internal.h"

#include <math.h>
#include <stdint.h>
#include <string.h>

#define CSG_PI 3.14159265358979323846

typedef struct {
    uint64_t s;
} Rng;

static void rng_seed(Rng *r, uint64_t seed) { r->s = seed ? seed : 1; }

static uint64_t rng_next(Rng *r)
{
    uint64_t x = r->s;
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    r->s = x;
    return x;
}

static double rng_uniform(Rng *r) { return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0); }

static double rng_normal(Rng *r)
{
    double u1 = rng_uniform(r);
    double u2 = rng_uniform(r);
    if (u1 < 1e-15)
        u1 = 1e-15;
    return sqrt(-2.0 * log(u1)) * cos(2.0 * CSG_PI * u2);
}

static void clear_body(Body *b)
{
    memset(b, 0, sizeof(*b));
    b->type = BODY_STAR;
}

/* ---- the reference recipe (src/initial_conditions.c:40-144) -------------- */

void csg_ref_spiral(Body *bodies, int n, double cx, double cy, double galaxy_mass,
                    double disk_radius, double vx_bulk, double vy_bulk, uint64_t seed)
{
    Rng r;
    rng_seed(&r, seed);
    double rs = disk_radius / 4.0;
    double zh = disk_radius * 0.02;
    clear_body(&bodies[0]);
    bodies[0].x = cx;
    bodies[0].y = cy;
    bodies[0].vx = vx_bulk;
    bodies[0].vy = vy_bulk;
    bodies[0].mass = galaxy_mass * 0.01;
    for (int i = 1; i < n; i++) {
        Body *b = &bodies[i];
        clear_body(b);
        double u = rng_uniform(&r);
        if (u < 1e-15)
            u = 1e-15;
        double rad = -rs * log(1.0 - u * (1.0 - exp(-disk_radius / rs)));
        double th0 = 2.0 * CSG_PI * rng_uniform(&r);
        double arm = log(rad / rs + 0.1) / 0.27;
        double th = th0 + 0.35 * exp(-rad / (disk_radius * 0.8)) * sin(2.0 * (th0 - arm));
        b->x = cx + rad * cos(th);
        b->y = cy + rad * sin(th);
        b->z = rng_normal(&r) * zh;
        b->mass = (rng_uniform(&r) < 0.01) ? 10.0 + rng_uniform(&r) * 90.0 : 1.0;
        double menc = galaxy_mass * (1.0 - exp(-rad / rs) * (1.0 + rad / rs)) + bodies[0].mass;
        if (rad < 1e-10)
            rad = 1e-10;
        double vc = sqrt(menc / rad);
        double disp = 0.05 * vc;
        double vt = vc + rng_normal(&r) * disp;
        double vr = rng_normal(&r) * disp;
        b->vx = vx_bulk - vt * sin(th) + vr * cos(th);
        b->vy = vy_bulk + vt * cos(th) + vr * sin(th);
        b->vz = rng_normal(&r) * disp * 0.1;
    }
}

void csg_ref_merger(Body *bodies, int n, double separation, double approach_vel, uint64_t seed)
{
    int n1 = n / 2;
    int n2 = n - n1;
    double disk_radius = separation * 0.15;
    double gm = (double)n1 * 2.0;
    csg_ref_spiral(bodies, n1, -separation * 0.5, 0.0, gm, disk_radius, approach_vel,
                   approach_vel * 0.3, seed);
    csg_ref_spiral(bodies + n1, n2, separation * 0.5, 0.0, gm * 0.7, disk_radius * 0.8,
                   -approach_vel, -approach_vel * 0.3, seed + 12345);
}

/* The reference's quasar galaxy (src/initial_conditions.c:146-196): a spiral
   whose central body becomes an SMBH of mass smbh_mass_frac x galaxy_mass,
   spin (0, 0.7071, 0.7071), seeded accretion; the inner 20% of the disk
   radius is gas with SPH fields. */
void csg_ref_quasar_galaxy(Body *bodies, int n, double cx, double cy, double galaxy_mass,
                           double disk_radius, double vx_bulk, double vy_bulk,
                           double smbh_mass_frac, uint64_t seed)
{
    csg_ref_spiral(bodies, n, cx, cy, galaxy_mass, disk_radius, vx_bulk, vy_bulk, seed);
    if (n < 1)
        return;
    bodies[0].mass = galaxy_mass * smbh_mass_frac;
    bodies[0].type = BODY_SMBH;
    bodies[0].spin_x = 0.0;
    bodies[0].spin_y = 0.7071;
    bodies[0].spin_z = 0.7071;
    bodies[0].accretion_rate = galaxy_mass * 0.001;
    bodies[0].luminosity = 0.1 * bodies[0].accretion_rate;
    double inner_sq = (disk_radius * 0.2) * (disk_radius * 0.2);
    double spacing = disk_radius / sqrt((double)n);
    for (int i = 1; i < n; i++) {
        double dx = bodies[i].x - cx, dy = bodies[i].y - cy;
        if (dx * dx + dy * dy < inner_sq)
            bodies[i].type = BODY_GAS;
    }
    for (int i = 1; i < n; i++) {
        if (bodies[i].type != BODY_GAS)
            continue;
        double dx = bodies[i].x - cx, dy = bodies[i].y - cy;
        double r = sqrt(dx * dx + dy * dy);
        if (r < 1e-10)
            r = 1e-10;
        double m_enc = galaxy_mass * (1.0 - exp(-r / (disk_radius / 4.0)));
        double vloc = sqrt(m_enc / r);
        bodies[i].internal_energy = 0.5 * vloc * vloc / (CSG_SPH_GAMMA - 1.0);
        bodies[i].smoothing_h = spacing * 2.0;
    }
}

/* The reference's quasar merger (src/initial_conditions.c:268-348): two quasar
   galaxies, masses 1 : 1.2, the second 30% larger and tilted 50 deg about x,
   on a grazing orbit (tangential 0.2 v_circ, radial approach_vel). */
void csg_ref_quasar_merger(Body *bodies, int n, double separation, double approach_vel,
                           double smbh_mass_frac, uint64_t seed)
{
    int n1 = n / 2, n2 = n - n1;
    double disk_radius = separation * 0.15;
    double galaxy_mass = (double)n1 * 2.0;
    double total_mass = galaxy_mass + galaxy_mass * 1.2;
    double v_orbit = sqrt(total_mass / separation) * 0.2;
    csg_ref_quasar_galaxy(bodies, n1, -separation * 0.5, 0.0, galaxy_mass, disk_radius,
                          approach_vel, v_orbit, smbh_mass_frac, seed);
    bodies[0].spin_x = 0.0;
    bodies[0].spin_y = 0.7071;
    bodies[0].spin_z = 0.7071;
    csg_ref_quasar_galaxy(bodies + n1, n2, separation * 0.5, 0.0, galaxy_mass * 1.2,
                          disk_radius * 1.3, -approach_vel, -v_orbit * 0.85, smbh_mass_frac,
                          seed + 12345);
    double t = 50.0 * CSG_PI / 180.0, ct = cos(t), st = sin(t);
    for (int i = n1; i < n; i++) {
        double y0 = bodies[i].y, z0 = bodies[i].z;
        bodies[i].y = y0 * ct - z0 * st;
        bodies[i].z = y0 * st + z0 * ct;
        double vy0 = bodies[i].vy, vz0 = bodies[i].vz;
        bodies[i].vy = vy0 * ct - vz0 * st;
        bodies[i].vz = vy0 * st + vz0 * ct;
    }
    if (n2 > 0) {
        double sy = 0.7071 * ct - 0.7071 * st, sz = 0.7071 * st + 0.7071 * ct;
        double smag = sqrt(sy * sy + sz * sz);
        bodies[n1].spin_x = 0.0;
        bodies[n1].spin_y = sy / smag;
        bodies[n1].spin_z = sz / smag;
    }
}

/* The reference's merger dust (src/initial_conditions.c:198-266): a tidal
   bridge between the two centres and an outer halo around each disk. */
void csg_ref_merger_dust(Body *bodies, int start_idx, int n_dust, double separation,
                         uint64_t seed)
{
    Rng r;
    rng_seed(&r, seed);
    double disk_radius = separation * 0.15;
    double gm1 = (double)(start_idx / 2) * 2.0, gm2 = gm1 * 1.2;
    double disk_r2 = disk_radius * 1.3;
    double cx1 = -separation * 0.5, cx2 = separation * 0.5;
    int n_tidal = n_dust / 3;
    int n_halo1 = (n_dust - n_tidal) / 2;
    int n_halo2 = n_dust - n_tidal - n_halo1;
    for (int i = 0; i < n_tidal; i++) {
        Body *b = &bodies[start_idx + i];
        clear_body(b);
        double t = rng_uniform(&r);
        double bx = cx1 + t * (cx2 - cx1);
        double by = rng_normal(&r) * separation * 0.06;
        b->x = bx + rng_normal(&r) * separation * 0.04;
        b->y = by;
        b->z = rng_normal(&r) * separation * 0.015;
        b->mass = 0.4 + rng_uniform(&r) * 0.6;
        b->type = BODY_DUST;
        double rr = sqrt(bx * bx + by * by);
        if (rr < 1e-10)
            rr = 1e-10;
        double v_c = sqrt(gm1 / rr) * 0.25;
        b->vx = -v_c * by / rr + rng_normal(&r) * 0.4;
        b->vy = v_c * bx / rr + rng_normal(&r) * 0.4;
        b->vz = rng_normal(&r) * 0.2;
    }
    for (int half = 0; half < 2; half++) {
        int cnt = half ? n_halo2 : n_halo1;
        int off = start_idx + n_tidal + (half ? n_halo1 : 0);
        double rad0 = half ? disk_r2 : disk_radius, cx = half ? cx2 : cx1;
        double gm = half ? gm2 : gm1;
        for (int i = 0; i < cnt; i++) {
            Body *b = &bodies[off + i];
            clear_body(b);
            double rr = rad0 * (0.7 + 0.9 * sqrt(rng_uniform(&r)));
            double th = 2.0 * CSG_PI * rng_uniform(&r);
            b->x = cx + rr * cos(th);
            b->y = rr * sin(th);
            b->z = rng_normal(&r) * rad0 * 0.08;
            b->mass = 0.4 + rng_uniform(&r) * 0.6;
            b->type = BODY_DUST;
            double v_c = sqrt(gm / rr) * 0.75;
            double disp = v_c * 0.08;
            b->vx = -v_c * sin(th) + rng_normal(&r) * disp;
            b->vy = v_c * cos(th) + rng_normal(&r) * disp;
            b->vz = rng_normal(&r) * disp * 0.3;
        }
    }
}

/* The reference's quasar defaults (src/quasar.c:37-57). */
CSG_EXPORT QuasarConfig csg_quasar_default_config(void)
{
    QuasarConfig c;
    memset(&c, 0, sizeof(c));
    c.accretion_radius = 3.0;
    c.swallow_radius = 0.3;
    c.isco_radius = 0.5;
    c.viscosity_alpha = 0.05;
    c.jet_speed = 20.0;
    c.jet_mass = 0.5;
    c.jet_lifetime = 5.0;
    c.feedback_strength = 1.0;
    c.eta_eff = 0.1;
    c.eddington_k = 0.5;
    c.accretion_smoothing = 0.95;
    c.jet_cap = 2000;
    c.jet_ring_count = 4;
    return c;
}

/* ---- benchmark configurations --------------------------------------------- */

typedef struct {
    double mass;       /* disk mass (excluding the central body) */
    double rd;         /* scale length */
    double zh;         /* vertical Gaussian scale */
    double smbh;       /* central mass (0: none) */
    double gas_frac;   /* inner fraction drawn as SPH gas */
    double bulge_mass; /* Plummer bulge mass inside the disk (enclosed-mass term) */
    double bulge_a;
} DiskSpec;

static double plummer_menc(double m, double a, double r)
{
    if (m <= 0.0)
        return 0.0;
    return m * r * r * r / pow(r * r + a * a, 1.5);
}

/* One exponential disk centred at the origin, in its own frame, following the
   reference recipe (truncated radial draw to 4 scale lengths, two-arm spiral
   perturbation, circular speed from the enclosed mass, 5% dispersion in the
   plane and 0.5% vertically). Body 0 is the central mass when spec->smbh > 0.
   Disk bodies share spec->mass equally. */
static void disk(Body *out, int n, const DiskSpec *spec, Rng *r)
{
    int first = 0;
    if (spec->smbh > 0.0 && n > 0) {
        clear_body(&out[0]);
        out[0].mass = spec->smbh;
        out[0].type = BODY_SMBH;
        first = 1;
    }
    int nd = n - first;
    double mi = nd > 0 ? spec->mass / nd : 0.0;
    double rmax = 4.0 * spec->rd;
    double spacing = rmax / sqrt((double)(n > 0 ? n : 1));
    for (int i = first; i < n; i++) {
        Body *b = &out[i];
        clear_body(b);
        double u = rng_uniform(r);
        if (u < 1e-15)
            u = 1e-15;
        double rad = -spec->rd * log(1.0 - u * (1.0 - exp(-rmax / spec->rd)));
        double th0 = 2.0 * CSG_PI * rng_uniform(r);
        double arm = log(rad / spec->rd + 0.1) / 0.27;
        double th = th0 + 0.35 * exp(-rad / (rmax * 0.8)) * sin(2.0 * (th0 - arm));
        b->x = rad * cos(th);
        b->y = rad * sin(th);
        b->z = rng_normal(r) * spec->zh;
        b->mass = mi;
        double x = rad / spec->rd;
        double menc = spec->mass * (1.0 - exp(-x) * (1.0 + x)) + spec->smbh +
                      plummer_menc(spec->bulge_mass, spec->bulge_a, rad);
        if (rad < 1e-10)
            rad = 1e-10;
        double vc = sqrt(menc / rad);
        double disp = 0.05 * vc;
        double vt = vc + rng_normal(r) * disp;
        double vr = rng_normal(r) * disp;
        b->vx = -vt * sin(th) + vr * cos(th);
        b->vy = vt * cos(th) + vr * sin(th);
        b->vz = rng_normal(r) * disp * 0.1;
        if (u < spec->gas_frac) { /* inner bodies are gas, src/initial_conditions.c:170-194 */
            b->type = BODY_GAS;
            double mg = spec->mass * (1.0 - exp(-x));
            double vloc = sqrt(mg / rad);
            b->internal_energy = 0.5 * vloc * vloc / (CSG_SPH_GAMMA - 1.0);
            b->smoothing_h = spacing * 2.0;
        }
    }
}

/* Plummer sphere of mass m, scale a, truncated at 20a; velocities by the
   Aarseth-Henon-Wielen rejection method. */
static void plummer(Body *out, int n, double m, double a, Rng *r)
{
    double mi = n > 0 ? m / n : 0.0;
    for (int i = 0; i < n; i++) {
        Body *b = &out[i];
        clear_body(b);
        double rad;
        do {
            double u = rng_uniform(r);
            if (u < 1e-12)
                u = 1e-12;
            rad = a / sqrt(pow(u, -2.0 / 3.0) - 1.0);
        } while (!(rad < 20.0 * a));
        double cz = 2.0 * rng_uniform(r) - 1.0;
        double ph = 2.0 * CSG_PI * rng_uniform(r);
        double sz = sqrt(1.0 - cz * cz);
        b->x = rad * sz * cos(ph);
        b->y = rad * sz * sin(ph);
        b->z = rad * cz;
        double q, g;
        do {
            q = rng_uniform(r);
            g = 0.1 * rng_uniform(r);
        } while (g > q * q * pow(1.0 - q * q, 3.5));
        double ve = sqrt(2.0 * m / sqrt(rad * rad + a * a));
        double v = q * ve;
        double vz = 2.0 * rng_uniform(r) - 1.0;
        double vph = 2.0 * CSG_PI * rng_uniform(r);
        double vs = sqrt(1.0 - vz * vz);
        b->vx = v * vs * cos(vph);
        b->vy = v * vs * sin(vph);
        b->vz = v * vz;
        b->mass = mi;
    }
}

static void shift(Body *b, int n, double x, double y, double z, double vx, double vy, double vz)
{
    for (int i = 0; i < n; i++) {
        b[i].x += x;
        b[i].y += y;
        b[i].z += z;
        b[i].vx += vx;
        b[i].vy += vy;
        b[i].vz += vz;
    }
}

static void tilt_x(Body *b, int n, double deg)
{
    double t = deg * CSG_PI / 180.0, c = cos(t), s = sin(t);
    for (int i = 0; i < n; i++) {
        double y = b[i].y, z = b[i].z;
        b[i].y = y * c - z * s;
        b[i].z = y * s + z * c;
        double vy = b[i].vy, vz = b[i].vz;
        b[i].vy = vy * c - vz * s;
        b[i].vz = vy * s + vz * c;
    }
}

/* Two disks, mass ratio 1:1.2, the second tilted 50 deg about x; separation
   30 scale lengths; nearly radial approach at 0.3 v_circ (tangential/radial
   0.17, as the reference's merger comment gives); each with an SMBH of
   0.005 x its disk mass. */
static void merger(Body *out, int n, double gas_frac, Rng *r)
{
    int n1 = n / 2, n2 = n - n1;
    DiskSpec g1 = {1.0, 1.0, 0.1, 0.005 * 1.0, gas_frac, 0.0, 0.0};
    DiskSpec g2 = {1.2, 1.3, 0.13, 0.005 * 1.2, gas_frac, 0.0, 0.0};
    disk(out, n1, &g1, r);
    disk(out + n1, n2, &g2, r);
    tilt_x(out + n1, n2, 50.0);
    double m1 = g1.mass + g1.smbh, m2 = g2.mass + g2.smbh, mt = m1 + m2;
    double sep = 30.0;
    double vcirc = sqrt(mt / sep);
    double vrel = 0.3 * vcirc;
    double vrad = vrel / sqrt(1.0 + 0.17 * 0.17), vtan = 0.17 * vrad;
    shift(out, n1, -sep * m2 / mt, 0.0, 0.0, vrad * m2 / mt, vtan * m2 / mt, 0.0);
    shift(out + n1, n2, sep * m1 / mt, 0.0, 0.0, -vrad * m1 / mt, -vtan * m1 / mt, 0.0);
}

/* The disk of kinds 0, 3, 5, 6 as a plan for the device generator: its
   DiskSpec and the generator state before its first body's draws (kind 3
   draws its scale length and SMBH fraction first). Returns 0, or -1 for a
   kind that is not a single disk. */
int csg_disk_plan(int kind, uint64_t seed, csgd_disk_plan *plan)
{
    Rng r;
    rng_seed(&r, seed);
    DiskSpec s;
    switch (kind) {
    case 0:
        s = (DiskSpec){1.0, 1.0, 0.1, 0.01, 0.0, 0.0, 0.0};
        break;
    case 3: {
        double rd = 0.5 + 1.5 * rng_uniform(&r);
        double f = 0.001 + 0.019 * rng_uniform(&r);
        s = (DiskSpec){1.0, rd, 0.1 * rd, f, 0.0, 0.0, 0.0};
        break;
    }
    case 5:
        s = (DiskSpec){1.0, 1.0, 0.1, 0.005 * 1.0, 0.0, 0.0, 0.0};
        break;
    case 6:
        s = (DiskSpec){1.2, 1.3, 0.13, 0.005 * 1.2, 0.0, 0.0, 0.0};
        break;
    default:
        return -1;
    }
    memset(plan, 0, sizeof(*plan));
    plan->mass = s.mass;
    plan->rd = s.rd;
    plan->zh = s.zh;
    plan->smbh = s.smbh;
    plan->gas_frac = s.gas_frac;
    plan->bulge_mass = s.bulge_mass;
    plan->bulge_a = s.bulge_a;
    plan->seed = r.s;
    return 0;
}

int csg_generate_ics_impl(int kind, int n, uint64_t seed, Body *out)
{
    if (n < 0 || (n > 0 && !out))
        return -1;
    Rng r;
    rng_seed(&r, seed);
    switch (kind) {
    case 0: { /* single disk: R_d 1, z 0.1, mass 1, SMBH 0.01 */
        DiskSpec s = {1.0, 1.0, 0.1, 0.01, 0.0, 0.0, 0.0};
        disk(out, n, &s, &r);
        break;
    }
    case 1:
        merger(out, n, 0.10, &r);
        break;
    case 2: { /* Plummer bulge 30% (a 0.5) + disk 70%, equal masses, total 1 */
        int nb = (int)(0.3 * (double)n);
        int nd = n - nb;
        double mb = (double)nb / (double)n, md = (double)nd / (double)n;
        plummer(out, nb, mb, 0.5, &r);
        DiskSpec s = {md, 1.0, 0.1, 0.0, 0.0, mb, 0.5};
        disk(out + nb, nd, &s, &r);
        break;
    }
    case 3: { /* ensemble member: R_d in [0.5, 2], SMBH fraction in [0.001, 0.02] */
        double rd = 0.5 + 1.5 * rng_uniform(&r);
        double f = 0.001 + 0.019 * rng_uniform(&r);
        DiskSpec s = {1.0, rd, 0.1 * rd, f, 0.0, 0.0, 0.0};
        disk(out, n, &s, &r);
        break;
    }
    case 4:
        merger(out, n, 0.0, &r);
        break;
    case 5: { /* the merger's first disk alone, stars only, in its own frame */
        DiskSpec s = {1.0, 1.0, 0.1, 0.005 * 1.0, 0.0, 0.0, 0.0};
        disk(out, n, &s, &r);
        break;
    }
    case 6: { /* the merger's second disk alone (untilted), stars only, own frame */
        DiskSpec s = {1.2, 1.3, 0.13, 0.005 * 1.2, 0.0, 0.0, 0.0};
        disk(out, n, &s, &r);
        break;
    }
    default:
        return -1;
    }
    return n;
}

CSG_EXPORT int csg_generate_ics(int kind, int n, uint64_t seed, Body *out)
{
    return csg_generate_ics_impl(kind, n, seed, out);
}

CSG_EXPORT int csg_generate_ics_device(int kind, int n, uint64_t seed, Body *device_out,
                                       void *stream)
{
    csgd_disk_plan p;
    if (n < 0 || (n > 0 && !device_out) || csg_disk_plan(kind, seed, &p))
        return -1;
    if (n == 0)
        return 0;
    return csgd_generate_disks(stream, &p, &n, 1, device_out) ? -1 : n;
}
