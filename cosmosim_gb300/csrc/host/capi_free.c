/*
 * capi_free.c — the reference's free functions (octree.h, integrator.h,
 * sph.h) over host arrays: upload, run on the device, copy results back.
 *
 * Semantics kept from the reference:
 *   - the caller owns bodies and the pool; pool holds the built tree after
 *     octree_build / integrator_* (root at index 0, reference numbering);
 *   - octree_compute_forces / sph_* / octree_find_neighbors use the tree the
 *     given pool holds (it is uploaded, whoever built it);
 *   - void functions report failures through csg_last_error(), never abort.
 * On failure the caller's arrays are left as they were.
 */
#include "capi_internal.h"

#include <string.h>

static csgd_force_params force_params(double G, double softening, double theta)
{
    csgd_force_params p;
    p.G = G;
    p.softening = softening;
    p.theta = theta;
    p.precision = csg_thread_precision();
    return p;
}

/* Uploads bodies and the pool's tree. */
static int load_pool(csgd_t *d, const OctreeNode *pool, int root, const Body *bodies, int n)
{
    int nn = 0;
    int rc = csg_pool_extent(pool, root, &nn);
    if (rc)
        return rc;
    rc = csgd_upload_bodies(d, bodies, n);
    if (!rc)
        rc = csgd_import_pool(d, pool, nn, root);
    if (!rc)
        rc = csgd_sync(d); /* a bad pool must be reported before any walk */
    return rc;
}

/* Writes the device tree into the caller's pool (capacity 8n, the reference
   contract; the root alone for n < 1). */
static int store_pool(csgd_t *d, OctreeNode *pool, int *pool_size, int n)
{
    int ps = 0;
    int cap = 8 * (n > 1 ? n : 1);
    int rc = csgd_export_pool(d, pool, cap, &ps);
    if (rc)
        return rc;
    if (pool_size)
        *pool_size = ps;
    return CSG_OK;
}

/* Records a free function's status for csg_last_error. A failed call also
   waits for its queued work and discards what it left for a later sync (a
   device error flag, a parked host error), so the next call starts clean. */
static void finish(csgd_t *d, int rc)
{
    if (rc)
        (void)csgd_sync(d);
    csg_thread_set_error(rc);
}

CSG_EXPORT void octree_build(OctreeNode *pool, int *pool_size, const Body *bodies, int n)
{
    csgd_t *d = csg_thread_dev();
    if (!d)
        return;
    if (!pool || !pool_size || (n > 0 && !bodies) || n < 0) {
        csg_thread_set_error(CSG_ERR_BAD_ARG);
        return;
    }
    int rc = csgd_upload_bodies(d, bodies, n);
    if (!rc)
        rc = csgd_build_tree(d, 1);
    if (!rc)
        rc = store_pool(d, pool, pool_size, n);
    finish(d, rc);
}

static void compute_forces(const OctreeNode *pool, int root, Body *bodies, int n, double G,
                           double softening, double theta, int exact)
{
    csgd_t *d = csg_thread_dev();
    if (!d)
        return;
    if (!pool || (n > 0 && !bodies) || n < 0) {
        csg_thread_set_error(CSG_ERR_BAD_ARG);
        return;
    }
    if (n == 0) {
        csg_thread_set_error(CSG_OK);
        return;
    }
    int rc = load_pool(d, pool, root, bodies, n);
    csgd_force_params p = force_params(G, softening, theta);
    if (!rc)
        rc = csgd_gravity_ex(d, &p, exact);
    if (!rc)
        rc = csgd_download_bodies(d, bodies, n);
    if (!rc)
        rc = csgd_sync(d);
    finish(d, rc);
}

CSG_EXPORT void octree_compute_forces(const OctreeNode *pool, int root, Body *bodies, int n,
                                      double G, double softening, double theta)
{
    compute_forces(pool, root, bodies, n, G, softening, theta, 0);
}

CSG_EXPORT void csg_octree_compute_forces_exact(const OctreeNode *pool, int root, Body *bodies,
                                                int n, double G, double softening, double theta)
{
    compute_forces(pool, root, bodies, n, G, softening, theta, 1);
}

CSG_EXPORT int octree_find_neighbors(const OctreeNode *pool, int root, const Body *bodies, int n,
                                     double cx, double cy, double cz, double radius,
                                     int *neighbor_buf, int buf_capacity)
{
    csgd_t *d = csg_thread_dev();
    if (!d)
        return 0;
    if (!pool || n < 0 || (n > 0 && !bodies) || (buf_capacity > 0 && !neighbor_buf)) {
        csg_thread_set_error(CSG_ERR_BAD_ARG);
        return 0;
    }
    int count = 0;
    int rc = load_pool(d, pool, root, bodies, n);
    if (!rc)
        rc = csgd_find_neighbors(d, cx, cy, cz, radius, neighbor_buf, buf_capacity, &count);
    finish(d, rc);
    return rc ? 0 : count;
}

CSG_EXPORT void integrator_init_accelerations(Body *bodies, int n, double G, double softening,
                                              double theta, OctreeNode *pool)
{
    csgd_t *d = csg_thread_dev();
    if (!d)
        return;
    if (!pool || n < 0 || (n > 0 && !bodies)) {
        csg_thread_set_error(CSG_ERR_BAD_ARG);
        return;
    }
    csgd_force_params p = force_params(G, softening, theta);
    int rc = csgd_upload_bodies(d, bodies, n);
    if (!rc)
        rc = csgd_build_tree(d, 1);
    if (!rc)
        rc = csgd_gravity(d, &p);
    if (!rc)
        rc = store_pool(d, pool, NULL, n); /* syncs */
    if (!rc)
        rc = csgd_download_bodies(d, bodies, n);
    if (!rc)
        rc = csgd_sync(d);
    finish(d, rc);
}

CSG_EXPORT void integrator_step(Body *bodies, int n, double dt, double G, double softening,
                                double theta, OctreeNode *pool, int sph_enabled)
{
    csgd_t *d = csg_thread_dev();
    if (!d)
        return;
    if (!pool || n < 0 || (n > 0 && !bodies)) {
        csg_thread_set_error(CSG_ERR_BAD_ARG);
        return;
    }
    csgd_force_params p = force_params(G, softening, theta);
    int rc = csgd_upload_bodies(d, bodies, n);
    /* a mapped (pinned) pool is filled by the export kernels beside the walk;
       any other pool after the substep */
    OctreeNode *pool_view = n > 0 ? (OctreeNode *)csgd_host_view(pool) : NULL;
    if (pool_view && !csgd_set_substep_export(d, pool_view, 8 * (n > 1 ? n : 1)))
        pool_view = NULL;
    /* one substep, replayed from the thread state's captured graph while n
       and the parameters stay the same (bit-identical to direct launches) */
    if (!rc)
        rc = csgd_substeps(d, 1, dt, &p, sph_enabled ? 1 : 0);
    csgd_set_substep_export(d, NULL, 0);
    if (!rc && !pool_view)
        rc = store_pool(d, pool, NULL, n);
    if (!rc)
        rc = csgd_download_step_fields(d, bodies, n, sph_enabled ? 1 : 0);
    if (!rc)
        rc = csgd_sync(d);
    finish(d, rc);
}

static void sph_pass(Body *bodies, int n, const OctreeNode *tree, int which)
{
    csgd_t *d = csg_thread_dev();
    if (!d)
        return;
    if (!tree || n < 0 || (n > 0 && !bodies)) {
        csg_thread_set_error(CSG_ERR_BAD_ARG);
        return;
    }
    if (n == 0) {
        csg_thread_set_error(CSG_OK);
        return;
    }
    int rc = load_pool(d, tree, 0, bodies, n);
    if (!rc)
        rc = which == 0 ? csgd_sph_density(d) : csgd_sph_forces(d, 0);
    if (!rc)
        rc = csgd_download_bodies(d, bodies, n);
    if (!rc)
        rc = csgd_sync(d);
    finish(d, rc);
}

CSG_EXPORT void sph_compute_density(Body *bodies, int n, const OctreeNode *tree)
{
    sph_pass(bodies, n, tree, 0);
}

CSG_EXPORT void sph_compute_forces(Body *bodies, int n, const OctreeNode *tree)
{
    sph_pass(bodies, n, tree, 1);
}

CSG_EXPORT void sph_apply_cooling(Body *bodies, int n, double dt)
{
    csgd_t *d = csg_thread_dev();
    if (!d)
        return;
    if (n < 0 || (n > 0 && !bodies)) {
        csg_thread_set_error(CSG_ERR_BAD_ARG);
        return;
    }
    int rc = csgd_upload_bodies(d, bodies, n);
    if (!rc)
        rc = csgd_sph_cooling(d, dt);
    if (!rc)
        rc = csgd_download_bodies(d, bodies, n);
    if (!rc)
        rc = csgd_sync(d);
    finish(d, rc);
}

/* ---- quasar step (reference src/quasar.c:477-509) on the GPU ---------------- */

CSG_EXPORT void csg_quasar_step(Body *bodies, int *n, int n_alloc, QuasarConfig *cfg, double dt)
{
    csgd_t *d = csg_thread_dev();
    if (!d)
        return;
    if (!bodies || !n || !cfg || *n < 0 || n_alloc < *n) {
        csg_thread_set_error(CSG_ERR_BAD_ARG);
        return;
    }
    int new_n = *n, jets = cfg->jet_count;
    int rc = csgd_reserve(d, n_alloc > 0 ? n_alloc : 1); /* room for appended jets */
    if (!rc)
        rc = csgd_upload_bodies(d, bodies, *n);
    if (!rc)
        rc = csgd_quasar_step(d, cfg, n_alloc, dt, &jets, &new_n);
    if (!rc)
        rc = csgd_download_bodies(d, bodies, new_n);
    if (!rc)
        rc = csgd_sync(d);
    if (!rc) {
        *n = new_n;
        cfg->jet_count = jets;
    }
    finish(d, rc);
}

CSG_EXPORT int csg_sort_keys(const uint64_t *keys, int n, int bits, uint64_t *out_keys,
                             int *out_index)
{
    csgd_t *d = csg_thread_dev();
    if (!d)
        return CSG_ERR_NO_DEVICE;
    int rc = csgd_sort_keys(d, (const unsigned long long *)keys, n, bits,
                            (unsigned long long *)out_keys, out_index);
    finish(d, rc);
    return rc;
}

CSG_EXPORT void csg_quasar_seed(uint64_t rng_state, int knot_phase)
{
    csgd_t *d = csg_thread_dev();
    if (!d)
        return;
    csg_thread_set_error(csgd_quasar_state(d, (unsigned long long)rng_state, knot_phase));
}
