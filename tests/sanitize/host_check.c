/*
 * host_check.c — the host code of this repository under AddressSanitizer and
 * UndefinedBehaviorSanitizer (built and run by tests/test_sanitize_host.py).
 *
 * Covers what runs on the CPU without a GPU: the library's seeded initial
 * conditions (csrc/host/ics.c) against the oracle's, the pool scan that
 * guards every caller-supplied tree (csg_pool_extent: reachable extent,
 * cycles, shared children) and the oracle itself (tree, forces, neighbour
 * search, SPH, leapfrog, quasar step, direct sum, energy). The device entry
 * points the host files refer to are stubbed: no device here.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../cosmosim_gb300/csrc/host/capi_internal.h"
#include "../../oracle/orc.h"

/* ---- stubs of the device layer (no GPU in this check) ---- */
csgd_t *csgd_create(void) { return NULL; }
void csgd_destroy(csgd_t *d) { (void)d; }
int csgd_has_device(void) { return 0; }
const char *csgd_error_string(int code) { return code ? "error" : "ok"; }
void csgd_set_export_order(csgd_t *d, int on) { (void)d; (void)on; }
void csgd_set_wait_limit(csgd_t *d, int polls) { (void)d; (void)polls; }
int csgd_check_device_wait(csgd_t *d, int polls, int *status) { (void)d; (void)polls; *status = 0; return 0; }
int csgd_set_phase_timing(csgd_t *d, int on) { (void)d; (void)on; return 0; }
int csgd_phase_times(const csgd_t *d, double ms[12], long long *substeps)
{
    (void)d;
    memset(ms, 0, 12 * sizeof(double));
    *substeps = 0;
    return 0;
}
int csgd_generate_disks(void *stream, const csgd_disk_plan *plans, const int *counts, int n_sys,
                        Body *out)
{
    (void)stream; (void)plans; (void)counts; (void)n_sys; (void)out;
    return CSG_ERR_NO_DEVICE;
}

static int failures = 0;
#define CHECK(c)                                                                                   \
    do {                                                                                           \
        if (!(c)) {                                                                                \
            fprintf(stderr, "check failed: %s (line %d)\n", #c, __LINE__);                         \
            failures++;                                                                            \
        }                                                                                          \
    } while (0)

int main(void)
{
    /* initial conditions: library == oracle, byte for byte, every kind */
    const int sizes[] = {0, 1, 2, 3, 777};
    for (int kind = 0; kind < 7; kind++)
        for (int s = 0; s < 5; s++) {
            const int n = sizes[s];
            Body *a = calloc(n + 1, sizeof(Body)), *b = calloc(n + 1, sizeof(Body));
            CHECK(csg_generate_ics_impl(kind, n, 1234 + kind, a) == n);
            CHECK(orc_generate_ics(kind, n, 1234 + kind, b) == n);
            CHECK(memcmp(a, b, sizeof(Body) * (size_t)n) == 0);
            free(a);
            free(b);
        }
    CHECK(csg_generate_ics_impl(9, 10, 1, NULL) == -1);
    CHECK(orc_generate_ics(0, -1, 1, NULL) == -1);

    /* a 3000-body merger with gas: the oracle's tree, walk, SPH and steps */
    const int n = 3000;
    Body *b = calloc(n, sizeof(Body));
    orc_generate_ics(1, n, 99, b);
    OctreeNode *pool = calloc((size_t)8 * n, sizeof(OctreeNode));
    int ps = 0;
    orc_octree_build(pool, &ps, b, n);
    CHECK(ps > n && ps <= 8 * n);
    int extent = 0;
    CHECK(csg_pool_extent(pool, 0, &extent) == CSG_OK && extent == ps);
    orc_integrator_init_accelerations(b, n, 1.0, 0.01, 0.5, pool);
    for (int k = 0; k < 3; k++)
        orc_integrator_step(b, n, 1e-3, 1.0, 0.01, 0.5, pool, 1);
    int buf[128];
    const int nb = orc_octree_find_neighbors(pool, 0, b, n, b[5].x, b[5].y, b[5].z, 0.3, buf, 128);
    CHECK(nb >= 0 && nb <= 128);
    int32_t *per = calloc(n, sizeof(int32_t));
    CHECK(orc_octree_count_interactions(pool, 0, b, n, 0.5, per) > 0);
    int32_t idx[64];
    for (int k = 0; k < 64; k++)
        idx[k] = (k * 37) % n;
    double *acc = calloc(3 * 64, sizeof(double));
    orc_direct_forces(b, n, idx, 64, 1.0, 0.01, acc);
    const double e = orc_total_energy(b, n, 1.0, 0.01);
    CHECK(e == e);

    /* the pool scan refuses what is not a tree (the steps rebuilt the pool:
       take its current extent) */
    CHECK(csg_pool_extent(pool, 0, &ps) == CSG_OK && ps > n && ps <= 8 * n);
    OctreeNode *bad = calloc((size_t)ps, sizeof(OctreeNode));
    memcpy(bad, pool, sizeof(OctreeNode) * (size_t)ps);
    int child = -1;
    for (int q = 0; q < 8 && child < 0; q++)
        child = bad[0].children[q];
    for (int q = 0; q < 8; q++)
        if (bad[child].children[q] < 0) { /* a cycle back to the root */
            bad[child].children[q] = 0;
            break;
        }
    CHECK(csg_pool_extent(bad, 0, &extent) == CSG_ERR_BAD_POOL);
    memcpy(bad, pool, sizeof(OctreeNode) * (size_t)ps);
    int other = -1; /* a second child of the root, shared with the first below */
    for (int q = 0; q < 8; q++)
        if (bad[0].children[q] >= 0 && bad[0].children[q] != child)
            other = bad[0].children[q];
    CHECK(other >= 0);
    for (int q = 0; q < 8 && other >= 0; q++)
        if (bad[child].children[q] < 0) {
            bad[child].children[q] = other;
            break;
        }
    CHECK(csg_pool_extent(bad, 0, &extent) == CSG_ERR_BAD_POOL);
    CHECK(csg_pool_extent(pool, -1, &extent) == CSG_ERR_BAD_POOL);

    /* quasar step: accretion, jets, lobes, recycling over a few steps */
    const int nq = 2000, nalloc = 2600;
    Body *q = calloc(nalloc, sizeof(Body));
    orc_generate_ics(1, nq, 5, q);
    q[0].type = BODY_SMBH;
    q[0].luminosity = 400.0;
    q[nq / 2].type = BODY_SMBH;
    QuasarConfig cfg = csg_quasar_default_config();
    cfg.jet_cap = 300;
    int nn = nq;
    orc_quasar_seed(1, 0);
    for (int k = 0; k < 20; k++)
        orc_quasar_step(q, &nn, nalloc, &cfg, 0.05);
    CHECK(nn >= nq && nn <= nalloc);

    /* the thread context without a device: a clean error, nothing else */
    CHECK(csg_thread_dev() == NULL && csg_last_error() == CSG_ERR_NO_DEVICE);
    csg_release_thread_state();

    free(b);
    free(pool);
    free(per);
    free(acc);
    free(bad);
    free(q);
    if (failures)
        fprintf(stderr, "%d checks failed\n", failures);
    else
        printf("host code clean under ASan/UBSan\n");
    return failures ? 1 : 0;
}
