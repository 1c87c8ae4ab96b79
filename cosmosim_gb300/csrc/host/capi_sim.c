/*
 * capi_sim.c — the embeddable handle API (reference src/cosmosim_api.c) with
 * bodies resident on the GPU between steps.
 *
 * A handle owns one device state (its own CUDA stream) and a host Body array
 * that cosmosim_get_bodies refreshes only when the device holds newer data.
 * Quasar mode runs the quasar step (src/quasar.c:477-509) on the device after
 * each substep and compacts dead bodies on the device every 60 steps
 * (src/cosmosim_api.c:121-141): the bodies stay resident. Initial conditions
 * and quasar defaults come from the reference's generators when the
 * application links them, else from this library's seeded restatement of the
 * same recipes.
 */
#include "capi_internal.h"

#include <stdlib.h>
#include <string.h>

/* Compile-time physics of the reference API, src/cosmosim_api.c:10-17. */
#define REF_G 1.0
#define REF_SOFTENING 1.5
#define REF_GALAXY_MASS 100.0
#define REF_DISK_RADIUS 15.0
#define REF_SEPARATION 40.0
#define REF_APPROACH_VEL 0.15
#define CSG_DEFAULT_SEED 0x5EED0000ull

/* The reference's CPU-side translation units, when the application links
   them (they are not part of this library). */
extern QuasarConfig quasar_default_config(void) __attribute__((weak));
extern void generate_spiral_galaxy(Body *bodies, int n, double cx, double cy, double galaxy_mass,
                                   double disk_radius, double vx_bulk, double vy_bulk)
    __attribute__((weak));
extern void generate_merger(Body *bodies, int n, double separation, double approach_vel)
    __attribute__((weak));
extern void generate_quasar_galaxy(Body *bodies, int n, double cx, double cy, double galaxy_mass,
                                   double disk_radius, double vx_bulk, double vy_bulk,
                                   double smbh_mass_frac) __attribute__((weak));
extern void generate_quasar_merger(Body *bodies, int n, double separation, double approach_vel,
                                   double smbh_mass_frac) __attribute__((weak));
extern void generate_merger_dust(Body *bodies, int start_idx, int n_dust, double separation)
    __attribute__((weak));


typedef struct {
    csgd_t *dev;
    Body *host;
    int n_alloc;
    int current_n;
    CosmosimConfig config;
    CsgSimParams params;
    QuasarConfig qcfg;
    int quasar;
    double sim_time;
    int compact_counter;
    int host_stale;
    int last_error;
} SimState;

static csgd_force_params fparams(const SimState *s)
{
    csgd_force_params p;
    p.G = s->params.G;
    p.softening = s->params.softening;
    p.theta = s->params.theta;
    p.precision = s->params.precision;
    return p;
}

static int set_err(SimState *s, int rc)
{
    s->last_error = rc;
    return rc;
}

static void destroy_state(SimState *s)
{
    if (!s)
        return;
    if (s->dev)
        csgd_destroy(s->dev);
    free(s->host);
    free(s);
}

/* Uploads host[0..current_n), declares the systems (n_sys > 1: an
   ensemble) and sets the initial accelerations (src/integrator.c:4-10: tree +
   gravity, no SPH). */
static SimState *start_systems(SimState *s, int n_sys, const int *counts)
{
    s->dev = csgd_create();
    if (!s->dev) {
        csg_thread_set_error(csgd_has_device() ? CSG_ERR_NOMEM : CSG_ERR_NO_DEVICE);
        destroy_state(s);
        return NULL;
    }
    csgd_force_params p = fparams(s);
    int rc = csgd_reserve(s->dev, s->n_alloc);
    if (!rc)
        rc = csgd_upload_bodies(s->dev, s->host, s->current_n);
    if (!rc && n_sys > 1)
        rc = csgd_set_systems(s->dev, n_sys, counts);
    if (!rc)
        rc = csgd_build_tree(s->dev, 0);
    if (!rc)
        rc = csgd_gravity(s->dev, &p);
    if (!rc)
        rc = csgd_download_bodies(s->dev, s->host, s->current_n);
    if (!rc)
        rc = csgd_sync(s->dev);
    if (rc) {
        csg_thread_set_error(rc);
        destroy_state(s);
        return NULL;
    }
    csg_thread_set_error(CSG_OK);
    return s;
}

static SimState *start(SimState *s) { return start_systems(s, 1, NULL); }

CSG_EXPORT CosmosimConfig cosmosim_default_config(void)
{
    CosmosimConfig c; /* src/cosmosim_api.c:30-45 */
    memset(&c, 0, sizeof(c));
    c.n_bodies = 20000;
    c.merger = 0;
    c.quasar = 0;
    c.dt = 0.005;
    c.theta = 0.5;
    c.smbh_mass_frac = 0.05;
    c.accretion_radius = 6.0;
    c.jet_speed = 15.0;
    c.feedback_strength = 0.3;
    c.substeps = 2;
    return c;
}

CSG_EXPORT SimHandle cosmosim_create_ex(CosmosimConfig config, double G, double softening,
                                        int precision)
{
    int n = config.n_bodies < 2 ? 2 : config.n_bodies; /* src/cosmosim_api.c:50-51 */
    int n_dust = (config.merger && config.quasar) ? n / 5 : 0;
    int n_alloc = config.quasar ? n + n_dust + n / 4 : n;
    SimState *s = (SimState *)calloc(1, sizeof(SimState));
    Body *bodies = (Body *)calloc((size_t)n_alloc, sizeof(Body));
    if (!s || !bodies) {
        free(s);
        free(bodies);
        csg_thread_set_error(CSG_ERR_NOMEM);
        return NULL;
    }
    if (config.quasar) { /* src/cosmosim_api.c:66-75 */
        if (config.merger) {
            if (generate_quasar_merger)
                generate_quasar_merger(bodies, n, REF_SEPARATION, REF_APPROACH_VEL,
                                       config.smbh_mass_frac);
            else
                csg_ref_quasar_merger(bodies, n, REF_SEPARATION, REF_APPROACH_VEL,
                                      config.smbh_mass_frac, CSG_DEFAULT_SEED);
            if (n_dust > 0) {
                if (generate_merger_dust)
                    generate_merger_dust(bodies, n, n_dust, REF_SEPARATION);
                else
                    csg_ref_merger_dust(bodies, n, n_dust, REF_SEPARATION,
                                        CSG_DEFAULT_SEED + 99999ull);
            }
        } else {
            if (generate_quasar_galaxy)
                generate_quasar_galaxy(bodies, n, 0.0, 0.0, (double)n * 2.0, REF_DISK_RADIUS,
                                       0.0, 0.0, config.smbh_mass_frac);
            else
                csg_ref_quasar_galaxy(bodies, n, 0.0, 0.0, (double)n * 2.0, REF_DISK_RADIUS,
                                      0.0, 0.0, config.smbh_mass_frac, CSG_DEFAULT_SEED);
        }
    } else if (config.merger) {
        if (generate_merger)
            generate_merger(bodies, n, REF_SEPARATION, REF_APPROACH_VEL);
        else
            csg_ref_merger(bodies, n, REF_SEPARATION, REF_APPROACH_VEL, CSG_DEFAULT_SEED);
    } else {
        if (generate_spiral_galaxy)
            generate_spiral_galaxy(bodies, n, 0.0, 0.0, REF_GALAXY_MASS, REF_DISK_RADIUS, 0.0,
                                   0.0);
        else
            csg_ref_spiral(bodies, n, 0.0, 0.0, REF_GALAXY_MASS, REF_DISK_RADIUS, 0.0, 0.0,
                           CSG_DEFAULT_SEED);
    }
    s->host = bodies;
    s->n_alloc = n_alloc;
    s->current_n = n + n_dust;
    s->config = config;
    s->params.G = G;
    s->params.softening = softening;
    s->params.theta = config.theta;
    s->params.dt = config.dt;
    s->params.substeps = config.substeps;
    s->params.sph = config.quasar ? 1 : 0; /* the reference passes quasar as sph_enabled */
    s->params.precision = precision;
    s->quasar = config.quasar ? 1 : 0;
    if (s->quasar) { /* src/cosmosim_api.c:87-94 */
        s->qcfg = quasar_default_config ? quasar_default_config() : csg_quasar_default_config();
        s->qcfg.accretion_radius = config.accretion_radius;
        s->qcfg.jet_speed = config.jet_speed;
        s->qcfg.feedback_strength = config.feedback_strength;
        s->qcfg.jet_cap = n / 10;
        s->qcfg.max_bodies = n_alloc;
    }
    return (SimHandle)start(s);
}

CSG_EXPORT SimHandle cosmosim_create(CosmosimConfig config)
{
    return cosmosim_create_ex(config, REF_G, REF_SOFTENING, CSG_PREC_FP64);
}

CSG_EXPORT SimHandle cosmosim_create_from_bodies(const Body *bodies, int n,
                                                 const CsgSimParams *params)
{
    if (n < 0 || (n > 0 && !bodies) || !params) {
        csg_thread_set_error(CSG_ERR_BAD_ARG);
        return NULL;
    }
    SimState *s = (SimState *)calloc(1, sizeof(SimState));
    Body *host = (Body *)calloc((size_t)(n > 0 ? n : 1), sizeof(Body));
    if (!s || !host) {
        free(s);
        free(host);
        csg_thread_set_error(CSG_ERR_NOMEM);
        return NULL;
    }
    if (n > 0)
        memcpy(host, bodies, sizeof(Body) * (size_t)n);
    s->host = host;
    s->n_alloc = n;
    s->current_n = n;
    s->params = *params;
    s->config = cosmosim_default_config();
    s->config.n_bodies = n;
    s->config.dt = params->dt;
    s->config.theta = params->theta;
    s->config.substeps = params->substeps;
    return (SimHandle)start(s);
}

CSG_EXPORT SimHandle cosmosim_create_ensemble(const Body *bodies, int n, int n_sys,
                                              const int *counts, const CsgSimParams *params)
{
    if (n < 1 || !bodies || n_sys < 1 || n_sys > CSG_MAX_SYSTEMS || !counts || !params) {
        csg_thread_set_error(CSG_ERR_BAD_ARG);
        return NULL;
    }
    if (params->sph) {
        csg_thread_set_error(CSG_ERR_UNSUPPORTED);
        return NULL;
    }
    long long total = 0;
    for (int g = 0; g < n_sys; g++) {
        if (counts[g] < 0) {
            csg_thread_set_error(CSG_ERR_BAD_ARG);
            return NULL;
        }
        total += counts[g];
    }
    if (total != n) {
        csg_thread_set_error(CSG_ERR_BAD_ARG);
        return NULL;
    }
    SimState *s = (SimState *)calloc(1, sizeof(SimState));
    Body *host = (Body *)calloc((size_t)n, sizeof(Body));
    if (!s || !host) {
        free(s);
        free(host);
        csg_thread_set_error(CSG_ERR_NOMEM);
        return NULL;
    }
    memcpy(host, bodies, sizeof(Body) * (size_t)n);
    s->host = host;
    s->n_alloc = n;
    s->current_n = n;
    s->params = *params;
    s->config = cosmosim_default_config();
    s->config.n_bodies = n;
    s->config.dt = params->dt;
    s->config.theta = params->theta;
    s->config.substeps = params->substeps;
    return (SimHandle)start_systems(s, n_sys, counts);
}

CSG_EXPORT SimHandle cosmosim_create_ensemble_ics(int kind, int n_sys, const int *counts,
                                                  uint64_t seed0, const CsgSimParams *params)
{
    if (n_sys < 1 || n_sys > CSG_MAX_SYSTEMS || !counts || !params) {
        csg_thread_set_error(CSG_ERR_BAD_ARG);
        return NULL;
    }
    if (params->sph) {
        csg_thread_set_error(CSG_ERR_UNSUPPORTED);
        return NULL;
    }
    long long total = 0;
    csgd_disk_plan *plans = (csgd_disk_plan *)calloc((size_t)n_sys, sizeof(csgd_disk_plan));
    if (!plans) {
        csg_thread_set_error(CSG_ERR_NOMEM);
        return NULL;
    }
    for (int g = 0; g < n_sys; g++) {
        if (counts[g] < 0 || csg_disk_plan(kind, seed0 + (uint64_t)g, &plans[g])) {
            free(plans);
            csg_thread_set_error(CSG_ERR_BAD_ARG);
            return NULL;
        }
        total += counts[g];
    }
    if (total < 1 || total > 0x7fffffff) {
        free(plans);
        csg_thread_set_error(CSG_ERR_BAD_ARG);
        return NULL;
    }
    const int n = (int)total;
    SimState *s = (SimState *)calloc(1, sizeof(SimState));
    Body *host = (Body *)calloc((size_t)n, sizeof(Body));
    csgd_t *d = csgd_create();
    int rc = (!s || !host) ? CSG_ERR_NOMEM
             : (!d ? (csgd_has_device() ? CSG_ERR_NOMEM : CSG_ERR_NO_DEVICE) : CSG_OK);
    if (!rc)
        rc = csgd_reserve(d, n);
    if (!rc) /* generated straight into the device Body staging */
        rc = csgd_generate_disks(csgd_stream(d), plans, counts, n_sys, csgd_aos(d));
    if (!rc)
        rc = csgd_unpack_aos(d);
    if (!rc)
        rc = csgd_set_systems(d, n_sys, counts);
    csgd_force_params p;
    if (s)
        s->params = *params;
    if (!rc) {
        p.G = params->G;
        p.softening = params->softening;
        p.theta = params->theta;
        p.precision = params->precision;
        rc = csgd_build_tree(d, 0);
    }
    if (!rc)
        rc = csgd_gravity(d, &p);
    if (!rc)
        rc = csgd_download_bodies(d, host, n);
    if (!rc)
        rc = csgd_sync(d);
    free(plans);
    if (rc) {
        if (d)
            csgd_destroy(d);
        free(host);
        free(s);
        csg_thread_set_error(rc);
        return NULL;
    }
    s->dev = d;
    s->host = host;
    s->n_alloc = n;
    s->current_n = n;
    s->config = cosmosim_default_config();
    s->config.n_bodies = n;
    s->config.dt = params->dt;
    s->config.theta = params->theta;
    s->config.substeps = params->substeps;
    csg_thread_set_error(CSG_OK);
    return (SimHandle)s;
}

CSG_EXPORT int cosmosim_system_count(SimHandle handle)
{
    if (!handle)
        return 0;
    return csgd_system_count(((SimState *)handle)->dev);
}

CSG_EXPORT int cosmosim_set_walk_shape(SimHandle handle, const CsgWalkShape *shape)
{
    if (!handle || !shape)
        return CSG_ERR_BAD_ARG;
    SimState *s = (SimState *)handle;
    int rc = csgd_set_walk_shape(s->dev, shape);
    if (rc)
        csgd_sync(s->dev); /* clears the recorded argument error */
    return set_err(s, rc);
}

CSG_EXPORT int cosmosim_get_walk_shape(SimHandle handle, CsgWalkShape *shape)
{
    if (!handle || !shape)
        return CSG_ERR_BAD_ARG;
    csgd_get_walk_shape(((SimState *)handle)->dev, shape);
    return CSG_OK;
}

CSG_EXPORT int cosmosim_autotune_walk(SimHandle handle, int reps, CsgWalkShape *best,
                                      CsgWalkShape *all, int all_cap, int *n_all)
{
    if (!handle || reps < 1 || reps > 64 || all_cap < 0)
        return CSG_ERR_BAD_ARG;
    SimState *s = (SimState *)handle;
    csgd_force_params p = fparams(s);
    /* the walks overwrite the accelerations; keep the handle's own */
    int rc = csgd_sync(s->dev);
    Body *keep = NULL;
    if (!rc) {
        keep = (Body *)malloc(sizeof(Body) * (size_t)(s->current_n > 0 ? s->current_n : 1));
        if (!keep)
            rc = CSG_ERR_NOMEM;
    }
    if (!rc)
        rc = csgd_download_bodies(s->dev, keep, s->current_n);
    if (!rc)
        rc = csgd_build_tree(s->dev, 0);
    if (!rc)
        rc = csgd_autotune_walk(s->dev, &p, reps, best, all, all_cap, n_all);
    if (!rc)
        rc = csgd_upload_bodies(s->dev, keep, s->current_n);
    if (!rc)
        rc = csgd_sync(s->dev);
    free(keep);
    return set_err(s, rc);
}

/* The quasar step between substeps (src/cosmosim_api.c:130-132), on the
   device; it may append jets and lobes. */
static int quasar_substep(SimState *s)
{
    int n = s->current_n;
    int rc = csgd_quasar_step(s->dev, &s->qcfg, s->n_alloc, s->config.dt, &s->qcfg.jet_count, &n);
    if (!rc)
        s->current_n = n;
    return rc;
}

CSG_EXPORT int cosmosim_substeps_async(SimHandle handle, int k)
{
    if (!handle)
        return CSG_ERR_BAD_ARG;
    SimState *s = (SimState *)handle;
    csgd_force_params p = fparams(s);
    int rc = csgd_substeps(s->dev, k, s->params.dt, &p, s->params.sph);
    s->host_stale = 1;
    return set_err(s, rc);
}

CSG_EXPORT void cosmosim_step(SimHandle handle)
{
    if (!handle) /* src/cosmosim_api.c:117-118 */
        return;
    SimState *s = (SimState *)handle;
    csgd_force_params p = fparams(s);
    int rc = CSG_OK;
    if (!s->quasar) {
        rc = csgd_substeps(s->dev, s->params.substeps, s->params.dt, &p, s->params.sph);
    } else {
        for (int sub = 0; sub < s->params.substeps && !rc; sub++) {
            rc = csgd_substep(s->dev, s->params.dt, &p, s->params.sph);
            if (!rc)
                rc = quasar_substep(s);
        }
    }
    if (!rc && s->quasar && ++s->compact_counter >= 60) { /* src/cosmosim_api.c:133-142 */
        int n = s->current_n; /* quasar_compact's semantics, on the device */
        rc = csgd_compact(s->dev, &n);
        if (!rc)
            s->current_n = n;
        s->compact_counter = 0;
    }
    if (!rc)
        rc = csgd_sync(s->dev);
    s->host_stale = 1;
    if (!rc)
        s->sim_time += s->config.dt * s->config.substeps;
    set_err(s, rc);
}

CSG_EXPORT int cosmosim_sync(SimHandle handle)
{
    if (!handle)
        return CSG_ERR_BAD_ARG;
    SimState *s = (SimState *)handle;
    return set_err(s, csgd_sync(s->dev));
}

CSG_EXPORT const Body *cosmosim_get_bodies(SimHandle handle)
{
    if (!handle)
        return NULL;
    SimState *s = (SimState *)handle;
    if (s->host_stale) {
        int rc = csgd_download_bodies(s->dev, s->host, s->current_n);
        if (!rc)
            rc = csgd_sync(s->dev);
        set_err(s, rc);
        if (!rc)
            s->host_stale = 0;
    }
    return s->host;
}

CSG_EXPORT int cosmosim_copy_bodies(SimHandle handle, Body *out, int n)
{
    if (!handle || !out)
        return CSG_ERR_BAD_ARG;
    SimState *s = (SimState *)handle;
    if (n != s->current_n)
        return set_err(s, CSG_ERR_BAD_ARG);
    int rc = csgd_download_bodies(s->dev, out, n);
    if (!rc)
        rc = csgd_sync(s->dev);
    return set_err(s, rc);
}

CSG_EXPORT int cosmosim_set_bodies(SimHandle handle, const Body *bodies, int n)
{
    if (!handle || !bodies)
        return CSG_ERR_BAD_ARG;
    SimState *s = (SimState *)handle;
    if (n != s->current_n)
        return set_err(s, CSG_ERR_BAD_ARG);
    int rc = csgd_upload_bodies(s->dev, bodies, n);
    s->host_stale = 1;
    return set_err(s, rc);
}

CSG_EXPORT int cosmosim_snapshot_f32(SimHandle handle, int format, float *out, int out_is_device,
                                     int max_bodies)
{
    if (!handle)
        return -1;
    SimState *s = (SimState *)handle;
    int count = 0;
    int rc = csgd_snapshot_f32(s->dev, format, out, out_is_device, max_bodies, &count);
    if (rc)
        csgd_sync(s->dev); /* clears a recorded argument error */
    set_err(s, rc);
    return rc ? -1 : count;
}

CSG_EXPORT int cosmosim_compact(SimHandle handle)
{
    if (!handle)
        return -1;
    SimState *s = (SimState *)handle;
    int n = s->current_n;
    int rc = csgd_compact(s->dev, &n);
    if (!rc) {
        s->current_n = n;
        s->host_stale = 1;
    }
    set_err(s, rc);
    return rc ? -1 : n;
}

CSG_EXPORT int cosmosim_get_count(SimHandle handle)
{
    if (!handle)
        return 0;
    return ((SimState *)handle)->current_n;
}

CSG_EXPORT int cosmosim_get_active_count(SimHandle handle)
{
    if (!handle)
        return 0;
    SimState *s = (SimState *)handle;
    int c = 0;
    int rc = csgd_alive_count(s->dev, &c);
    set_err(s, rc);
    return rc ? 0 : c;
}

CSG_EXPORT double cosmosim_get_sim_time(SimHandle handle)
{
    if (!handle)
        return 0.0;
    return ((SimState *)handle)->sim_time;
}

CSG_EXPORT void cosmosim_destroy(SimHandle handle)
{
    if (!handle)
        return;
    destroy_state((SimState *)handle);
}

CSG_EXPORT int cosmosim_last_error(SimHandle handle)
{
    if (!handle)
        return csg_last_error();
    return ((SimState *)handle)->last_error;
}

CSG_EXPORT int cosmosim_set_stream(SimHandle handle, void *cuda_stream)
{
    if (!handle)
        return CSG_ERR_BAD_ARG;
    SimState *s = (SimState *)handle;
    int rc = csgd_sync(s->dev);
    csgd_set_stream(s->dev, cuda_stream);
    return set_err(s, rc);
}

CSG_EXPORT int cosmosim_enable_phase_timing(SimHandle handle, int on)
{
    if (!handle)
        return CSG_ERR_BAD_ARG;
    SimState *s = (SimState *)handle;
    int rc = csgd_sync(s->dev);
    if (!rc)
        rc = csgd_set_phase_timing(s->dev, on);
    return set_err(s, rc);
}

CSG_EXPORT int cosmosim_phase_times(SimHandle handle, CsgPhaseTimes *out)
{
    if (!handle)
        return CSG_ERR_BAD_ARG;
    SimState *s = (SimState *)handle;
    return set_err(s, csg_fill_phase_times(s->dev, out));
}

CSG_EXPORT int cosmosim_set_wait_limit(SimHandle handle, int polls)
{
    if (!handle)
        return CSG_ERR_BAD_ARG;
    SimState *s = (SimState *)handle;
    csgd_set_wait_limit(s->dev, polls);
    return set_err(s, CSG_OK);
}

CSG_EXPORT int cosmosim_build_tree_async(SimHandle handle)
{
    if (!handle)
        return CSG_ERR_BAD_ARG;
    SimState *s = (SimState *)handle;
    return set_err(s, csgd_build_tree(s->dev, s->params.sph));
}

CSG_EXPORT int cosmosim_gravity_async(SimHandle handle)
{
    if (!handle)
        return CSG_ERR_BAD_ARG;
    SimState *s = (SimState *)handle;
    csgd_force_params p = fparams(s);
    s->host_stale = 1;
    return set_err(s, csgd_gravity(s->dev, &p));
}

CSG_EXPORT int cosmosim_enable_stats(SimHandle handle, int on)
{
    if (!handle)
        return CSG_ERR_BAD_ARG;
    SimState *s = (SimState *)handle;
    csgd_enable_stats(s->dev, on);
    return set_err(s, csgd_reset_stats(s->dev));
}

CSG_EXPORT int cosmosim_interactions(SimHandle handle, int64_t *total)
{
    if (!handle || !total)
        return CSG_ERR_BAD_ARG;
    SimState *s = (SimState *)handle;
    return set_err(s, csgd_interactions(s->dev, total));
}

CSG_EXPORT int cosmosim_walk_stats(SimHandle handle, int64_t *interactions, int64_t *warp_steps,
                                   int64_t *active_lane_steps)
{
    if (!handle || !interactions || !warp_steps || !active_lane_steps)
        return CSG_ERR_BAD_ARG;
    SimState *s = (SimState *)handle;
    return set_err(s, csgd_walk_stats(s->dev, interactions, warp_steps, active_lane_steps));
}

CSG_EXPORT int cosmosim_node_count(SimHandle handle, int *n_nodes)
{
    if (!handle || !n_nodes)
        return CSG_ERR_BAD_ARG;
    SimState *s = (SimState *)handle;
    return set_err(s, csgd_node_count(s->dev, n_nodes));
}

CSG_EXPORT int cosmosim_set_precision(SimHandle handle, int precision)
{
    if (!handle)
        return CSG_ERR_BAD_ARG;
    SimState *s = (SimState *)handle;
    s->params.precision =
        (precision == CSG_PREC_FP32_MIXED) ? CSG_PREC_FP32_MIXED : CSG_PREC_FP64;
    return set_err(s, CSG_OK);
}

CSG_EXPORT int cosmosim_direct_forces(SimHandle handle, const int *idx, int m, double *out)
{
    if (!handle || (m > 0 && (!idx || !out)) || m < 0)
        return CSG_ERR_BAD_ARG;
    SimState *s = (SimState *)handle;
    for (int k = 0; k < m; k++)
        if (idx[k] < 0 || idx[k] >= s->current_n)
            return set_err(s, CSG_ERR_BAD_ARG);
    return set_err(s, csgd_direct_forces(s->dev, idx, m, s->params.G, s->params.softening, out));
}

CSG_EXPORT int cosmosim_energy(SimHandle handle, double *kinetic, double *potential)
{
    if (!handle || !kinetic || !potential)
        return CSG_ERR_BAD_ARG;
    SimState *s = (SimState *)handle;
    return set_err(s, csgd_energy(s->dev, s->params.G, s->params.softening, kinetic, potential));
}

CSG_EXPORT int64_t cosmosim_launch_count(SimHandle handle)
{
    if (!handle)
        return 0;
    return (int64_t)csgd_launch_count(((SimState *)handle)->dev);
}

CSG_EXPORT int cosmosim_enable_graphs(SimHandle handle, int on)
{
    if (!handle)
        return CSG_ERR_BAD_ARG;
    csgd_enable_graphs(((SimState *)handle)->dev, on);
    return CSG_OK;
}
