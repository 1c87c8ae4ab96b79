/*
 * capi_context.c — per-thread device state, error channel and pool extent
 * for the reference-compatible free functions.
 */
#include "capi_internal.h"

#include <stdlib.h>
#include <string.h>

static _Thread_local csgd_t *tl_dev;
static _Thread_local int tl_error;
static _Thread_local int tl_precision = CSG_PREC_FP64;

csgd_t *csg_thread_dev(void)
{
    if (!tl_dev) {
        tl_dev = csgd_create();
        if (tl_dev) /* the free functions export the tree into the caller's pool */
            csgd_set_export_order(tl_dev, 1);
        if (!tl_dev)
            tl_error = csgd_has_device() ? CSG_ERR_NOMEM : CSG_ERR_NO_DEVICE;
    }
    return tl_dev;
}

CSG_EXPORT void csg_release_thread_state(void)
{
    if (tl_dev)
        csgd_destroy(tl_dev);
    tl_dev = NULL;
    tl_error = CSG_OK;
}

CSG_EXPORT void csg_set_wait_limit(int polls)
{
    csgd_t *d = csg_thread_dev();
    if (!d)
        return;
    csgd_set_wait_limit(d, polls);
    tl_error = CSG_OK;
}

CSG_EXPORT int csg_check_device_wait(int polls, int *status)
{
    csgd_t *d = csg_thread_dev();
    if (!d)
        return tl_error;
    tl_error = csgd_check_device_wait(d, polls, status);
    return tl_error;
}

void csg_thread_set_error(int code) { tl_error = code; }

int csg_thread_precision(void) { return tl_precision; }

CSG_EXPORT int csg_last_error(void) { return tl_error; }

CSG_EXPORT const char *csg_error_string(int code) { return csgd_error_string(code); }

CSG_EXPORT void csg_set_precision(int precision)
{
    tl_precision = (precision == CSG_PREC_FP32_MIXED) ? CSG_PREC_FP32_MIXED : CSG_PREC_FP64;
}

int csg_pool_extent(const OctreeNode *pool, int root, int *n_nodes)
{
    /* The pool carries no size: walk it from the root, reading exactly the
       cells the reference's own walk would read, and find the highest
       reachable index. A cycle or a repeated child makes it not a tree. */
    if (root < 0)
        return CSG_ERR_BAD_POOL;
    size_t cap = 1024;
    int *stack = (int *)malloc(cap * sizeof(int));
    size_t seen_cap = 0;
    unsigned char *seen = NULL;
    if (!stack)
        return CSG_ERR_NOMEM;
    size_t sp = 0;
    int hi = root;
    stack[sp++] = root;
    int rc = CSG_OK;
    long long visits = 0;
    while (sp > 0) {
        int c = stack[--sp];
        if ((size_t)c >= seen_cap) {
            size_t nc = seen_cap ? seen_cap : 4096;
            while (nc <= (size_t)c)
                nc *= 2;
            unsigned char *ns = (unsigned char *)realloc(seen, nc);
            if (!ns) {
                rc = CSG_ERR_NOMEM;
                break;
            }
            memset(ns + seen_cap, 0, nc - seen_cap);
            seen = ns;
            seen_cap = nc;
        }
        if (seen[c]) {
            rc = CSG_ERR_BAD_POOL;
            break;
        }
        seen[c] = 1;
        if (c > hi)
            hi = c;
        if (++visits > 0x7ffffff0LL) {
            rc = CSG_ERR_BAD_POOL;
            break;
        }
        for (int q = 0; q < 8; q++) {
            int ch = pool[c].children[q];
            if (ch < 0)
                continue;
            if (sp == cap) {
                size_t ncap = cap * 2;
                int *ns = (int *)realloc(stack, ncap * sizeof(int));
                if (!ns) {
                    rc = CSG_ERR_NOMEM;
                    break;
                }
                stack = ns;
                cap = ncap;
            }
            stack[sp++] = ch;
        }
        if (rc)
            break;
    }
    free(stack);
    free(seen);
    if (rc == CSG_OK)
        *n_nodes = hi + 1;
    return rc;
}

int csg_fill_phase_times(const csgd_t *d, CsgPhaseTimes *out)
{
    double ms[12];
    long long k = 0;
    if (!out)
        return CSG_ERR_BAD_ARG;
    csgd_phase_times(d, ms, &k);
    out->kick_drift_ms = ms[0];
    out->build_ms = ms[1];
    out->gravity_ms = ms[2];
    out->sph_ms = ms[3];
    out->kick_ms = ms[4];
    out->cooling_ms = ms[5];
    out->substep_ms = ms[6];
    out->substeps = k;
    out->build_keys_ms = ms[7];
    out->build_sort_ms = ms[8];
    out->build_cells_ms = ms[9];
    out->build_moments_ms = ms[10];
    out->build_rest_ms = ms[11];
    return CSG_OK;
}

CSG_EXPORT int csg_enable_phase_timing(int on)
{
    csgd_t *d = csg_thread_dev();
    if (!d)
        return tl_error;
    tl_error = csgd_set_phase_timing(d, on);
    return tl_error;
}

CSG_EXPORT int csg_phase_times(CsgPhaseTimes *out)
{
    csgd_t *d = csg_thread_dev();
    if (!d)
        return tl_error;
    return csg_fill_phase_times(d, out);
}
