/*
 * orc_ics.c — seeded benchmark initial conditions for the CPU side.
 *
 * TEST INFRASTRUCTURE ONLY (part of liborc.so). The timed CPU baseline and
 * the reference arm draw their bodies here, so that they never load the
 * product library; tests/test_oracle_ics.py checks that every kind equals the
 * library's csg_generate_ics byte for byte.
 *
 * The recipes follow the reference's generator (src/initial_conditions.c):
 *   - xorshift64 with shifts 13/7/17, 53-bit uniforms, Box-Muller normals
 *     with u1 clamped at 1e-15 (:8-38), but seeded explicitly instead of
 *     from time(NULL) (:49);
 *   - the exponential disk: truncated radial inversion, two-arm spiral
 *     offset with pitch 0.27, circular speed from the enclosed mass, 5%
 *     in-plane and 0.5% vertical dispersion (:64-110);
 *   - gas fields of the inner disk (:170-194), the 50 degree tilt about x of
 *     the merger's second galaxy (:321-347);
 * with the benchmark configurations' parameters (disk mass, scale length,
 * SMBH mass, equal disk masses; a Plummer bulge drawn by the
 * Aarseth-Henon-Wielen 1974 rejection method, truncated at 20 a).
 * The floating-point operations run in the same order as the library's
 * generator; built with -ffp-contract=off like it.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "orc.h"

#define ORC_PI 3.14159265358979323846
#define ORC_GAMMA (5.0 / 3.0)

typedef struct {
    uint64_t s;
} orc_rng;

static uint64_t orc_draw(orc_rng *g) /* src/initial_conditions.c:15-23 */
{
    g->s ^= g->s << 13;
    g->s ^= g->s >> 7;
    g->s ^= g->s << 17;
    return g->s;
}

static double orc_unit(orc_rng *g) /* :25-28, [0, 1) with 53 bits */
{
    return (double)(orc_draw(g) >> 11) * (1.0 / 9007199254740992.0);
}

static double orc_gauss(orc_rng *g) /* :31-38 */
{
    double a = orc_unit(g);
    double b = orc_unit(g);
    if (a < 1e-15)
        a = 1e-15;
    return sqrt(-2.0 * log(a)) * cos(2.0 * ORC_PI * b);
}

static void orc_blank(Body *b)
{
    memset(b, 0, sizeof(*b));
    b->type = BODY_STAR;
}

/* An exponential disk (scale length rd, truncated at 4 rd, Gaussian
   thickness zh) of disk mass md shared equally, around an optional central
   mass smbh at index 0; gas_frac of the radial quantiles are SPH gas; an
   optional Plummer bulge (mb, ab) adds to the enclosed mass. */
typedef struct {
    double md, rd, zh, smbh, gas_frac, mb, ab;
} orc_disk_spec;

static double orc_plummer_mass_within(double m, double a, double r)
{
    return m > 0.0 ? m * r * r * r / pow(r * r + a * a, 1.5) : 0.0;
}

static void orc_disk(Body *b, int n, const orc_disk_spec *d, orc_rng *g)
{
    int i0 = 0;
    if (d->smbh > 0.0 && n > 0) {
        orc_blank(b);
        b->mass = d->smbh;
        b->type = BODY_SMBH;
        i0 = 1;
    }
    const double m_each = (n - i0) > 0 ? d->md / (n - i0) : 0.0;
    const double r_max = 4.0 * d->rd;
    const double h_gas = 2.0 * (r_max / sqrt((double)(n > 0 ? n : 1)));
    for (int i = i0; i < n; i++) {
        Body *p = b + i;
        orc_blank(p);
        double u = orc_unit(g);
        if (u < 1e-15)
            u = 1e-15;
        double r = -d->rd * log(1.0 - u * (1.0 - exp(-r_max / d->rd)));
        const double phi0 = 2.0 * ORC_PI * orc_unit(g);
        const double arm = log(r / d->rd + 0.1) / 0.27;
        const double phi = phi0 + 0.35 * exp(-r / (r_max * 0.8)) * sin(2.0 * (phi0 - arm));
        p->x = r * cos(phi);
        p->y = r * sin(phi);
        p->z = orc_gauss(g) * d->zh;
        p->mass = m_each;
        const double s = r / d->rd;
        const double m_in = d->md * (1.0 - exp(-s) * (1.0 + s)) + d->smbh +
                            orc_plummer_mass_within(d->mb, d->ab, r);
        if (r < 1e-10)
            r = 1e-10;
        const double vc = sqrt(m_in / r);
        const double sig = 0.05 * vc;
        const double vt = vc + orc_gauss(g) * sig;
        const double vr = orc_gauss(g) * sig;
        p->vx = -vt * sin(phi) + vr * cos(phi);
        p->vy = vt * cos(phi) + vr * sin(phi);
        p->vz = orc_gauss(g) * sig * 0.1;
        if (u < d->gas_frac) {
            const double vg = sqrt(d->md * (1.0 - exp(-s)) / r);
            p->type = BODY_GAS;
            p->internal_energy = 0.5 * vg * vg / (ORC_GAMMA - 1.0);
            p->smoothing_h = h_gas;
        }
    }
}

/* Plummer sphere, mass m, scale a, radii below 20 a; speeds q v_esc with q
   drawn from q^2 (1 - q^2)^(7/2) by rejection (Aarseth, Henon & Wielen 1974). */
static void orc_plummer(Body *b, int n, double m, double a, orc_rng *g)
{
    const double m_each = n > 0 ? m / n : 0.0;
    for (int i = 0; i < n; i++) {
        Body *p = b + i;
        orc_blank(p);
        double r;
        for (;;) {
            double u = orc_unit(g);
            if (u < 1e-12)
                u = 1e-12;
            r = a / sqrt(pow(u, -2.0 / 3.0) - 1.0);
            if (r < 20.0 * a)
                break;
        }
        const double c = 2.0 * orc_unit(g) - 1.0;
        const double ph = 2.0 * ORC_PI * orc_unit(g);
        const double sn = sqrt(1.0 - c * c);
        p->x = r * sn * cos(ph);
        p->y = r * sn * sin(ph);
        p->z = r * c;
        double q;
        for (;;) {
            q = orc_unit(g);
            const double y = 0.1 * orc_unit(g);
            if (!(y > q * q * pow(1.0 - q * q, 3.5)))
                break;
        }
        const double v = q * sqrt(2.0 * m / sqrt(r * r + a * a));
        const double vc = 2.0 * orc_unit(g) - 1.0;
        const double vph = 2.0 * ORC_PI * orc_unit(g);
        const double vs = sqrt(1.0 - vc * vc);
        p->vx = v * vs * cos(vph);
        p->vy = v * vs * sin(vph);
        p->vz = v * vc;
        p->mass = m_each;
    }
}

static void orc_move(Body *b, int n, const double dx[3], const double dv[3])
{
    for (int i = 0; i < n; i++) {
        b[i].x += dx[0];
        b[i].y += dx[1];
        b[i].z += dx[2];
        b[i].vx += dv[0];
        b[i].vy += dv[1];
        b[i].vz += dv[2];
    }
}

/* Rotation by deg about the x axis (src/initial_conditions.c:321-347). */
static void orc_tilt(Body *b, int n, double deg)
{
    const double t = deg * ORC_PI / 180.0, c = cos(t), s = sin(t);
    for (int i = 0; i < n; i++) {
        const double y = b[i].y, z = b[i].z, vy = b[i].vy, vz = b[i].vz;
        b[i].y = y * c - z * s;
        b[i].z = y * s + z * c;
        b[i].vy = vy * c - vz * s;
        b[i].vz = vy * s + vz * c;
    }
}

/* Two disks 1 : 1.2 (scale lengths 1 and 1.3), SMBHs 0.005 of each disk
   mass, the second tilted 50 deg; separation 30, relative speed 0.3 v_circ,
   tangential / radial 0.17; both moved so the centre of mass is at rest at
   the origin. */
static void orc_merger(Body *b, int n, double gas_frac, orc_rng *g)
{
    const int na = n / 2, nb = n - na;
    const orc_disk_spec A = {1.0, 1.0, 0.1, 0.005 * 1.0, gas_frac, 0.0, 0.0};
    const orc_disk_spec B = {1.2, 1.3, 0.13, 0.005 * 1.2, gas_frac, 0.0, 0.0};
    orc_disk(b, na, &A, g);
    orc_disk(b + na, nb, &B, g);
    orc_tilt(b + na, nb, 50.0);
    const double ma = A.md + A.smbh, mb = B.md + B.smbh, mt = ma + mb;
    const double sep = 30.0;
    const double vrel = 0.3 * sqrt(mt / sep);
    const double vrad = vrel / sqrt(1.0 + 0.17 * 0.17), vtan = 0.17 * vrad;
    const double xa[3] = {-sep * mb / mt, 0.0, 0.0}, va[3] = {vrad * mb / mt, vtan * mb / mt, 0.0};
    const double xb[3] = {sep * ma / mt, 0.0, 0.0}, vb[3] = {-vrad * ma / mt, -vtan * ma / mt, 0.0};
    orc_move(b, na, xa, va);
    orc_move(b + na, nb, xb, vb);
}

int orc_generate_ics(int kind, int n, uint64_t seed, Body *out)
{
    if (n < 0 || (n > 0 && !out))
        return -1;
    orc_rng g = {seed ? seed : 1};
    switch (kind) {
    case 0: { /* exponential disk: R_d 1, z 0.1, mass 1, SMBH 0.01 */
        const orc_disk_spec d = {1.0, 1.0, 0.1, 0.01, 0.0, 0.0, 0.0};
        orc_disk(out, n, &d, &g);
        return n;
    }
    case 1: /* merger, 10% gas */
        orc_merger(out, n, 0.10, &g);
        return n;
    case 2: { /* Plummer bulge 30% (a 0.5), disk 70%, equal masses, total 1 */
        const int nbulge = (int)(0.3 * (double)n);
        const double mbulge = (double)nbulge / (double)n;
        const double mdisk = (double)(n - nbulge) / (double)n;
        orc_plummer(out, nbulge, mbulge, 0.5, &g);
        const orc_disk_spec d = {mdisk, 1.0, 0.1, 0.0, 0.0, mbulge, 0.5};
        orc_disk(out + nbulge, n - nbulge, &d, &g);
        return n;
    }
    case 3: { /* ensemble galaxy: R_d in [0.5, 2], SMBH fraction in [0.001, 0.02] */
        const double rd = 0.5 + 1.5 * orc_unit(&g);
        const double f = 0.001 + 0.019 * orc_unit(&g);
        const orc_disk_spec d = {1.0, rd, 0.1 * rd, f, 0.0, 0.0, 0.0};
        orc_disk(out, n, &d, &g);
        return n;
    }
    case 4: /* merger, stars only */
        orc_merger(out, n, 0.0, &g);
        return n;
    case 5: { /* the merger's first disk alone, own frame */
        const orc_disk_spec d = {1.0, 1.0, 0.1, 0.005 * 1.0, 0.0, 0.0, 0.0};
        orc_disk(out, n, &d, &g);
        return n;
    }
    case 6: { /* the merger's second disk alone, untilted, own frame */
        const orc_disk_spec d = {1.2, 1.3, 0.13, 0.005 * 1.2, 0.0, 0.0, 0.0};
        orc_disk(out, n, &d, &g);
        return n;
    }
    default:
        return -1;
    }
}
