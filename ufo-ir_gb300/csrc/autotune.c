/*
 * autotune.c - search of the tiled forward projector's launch shapes.
 *
 * For a geometry (n_dets, n_angles, step, axis) and a slice count, every
 * launch shape the kernels support is timed on scratch data of that
 * geometry (zeros: the kernel has no data-dependent branches, its chunk
 * forms depend on the geometry only) with CUDA events: one warm-up run,
 * then the best of two. The fixed rules' shape is always a candidate and is
 * kept unless another is at least 2 % faster. The result is cached per
 * context and recorded on the projector, whose later forward projections
 * with that slice count use it (ufoir__fp_shape). Shapes cannot change
 * results: each ray's arithmetic is the same whichever CTA, lane or chunk
 * size carries it.
 *
 * Search space (pruned to what can pay): angles per tile A in {8, 4, 2}
 * with the detector pairs per thread J of an existing kernel variant, rows
 * per chunk K in {32, 16, 8} (shared memory permitting), and, only when the
 * tiles alone cannot fill the GPU twice over, 2, 4 or 8 CTAs per tile with
 * and without column windows.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "host.h"

struct ufoir__tune_entry {
    unsigned int n, na;
    float step, axis;
    int arithmetic;          /* the shape carries the kernel's arithmetic (cfg.fm) */
    int slices;
    udev_fp_cfg cfg;
    ufoir_fp_tuning info;
};

void ufoir__tune_free(ufoir_ctx *ctx)
{
    free(ctx->tune);
    ctx->tune = NULL;
    ctx->n_tune = ctx->cap_tune = 0;
}

static struct ufoir__tune_entry *tune_find(ufoir_ctx *ctx, const ufoir_projector *p, int slices)
{
    const float axis = ufoir__axis(p);
    for (int i = 0; i < ctx->n_tune; i++) {
        struct ufoir__tune_entry *e = &ctx->tune[i];
        if (e->n == p->n_dets && e->na == p->n_angles && e->step == p->lut_step && e->axis == axis &&
            e->arithmetic == p->prm.arithmetic && e->slices == slices)
            return e;
    }
    return NULL;
}

static void info_of(const udev_fp_cfg *c, ufoir_fp_tuning *t)
{
    t->J = c->J;
    t->A = c->A;
    t->win = c->win;
    t->K = c->K;
    t->dsplit = c->dsplit;
    t->threads = c->threads;
}

/* One forward projection with shape c: best of two timed runs after one
 * warm-up, in milliseconds. */
static int time_shape(ufoir_projector *p, const udev_fp_cfg *c, const float *P, const float *TP, float *sino,
                      int slices, float *ms)
{
    udev *d = p->ctx->dev;
    udev_geom g;
    ufoir__projector_geom(p, &g);
    const void *tiles = NULL;
    int n_tiles = 0;
    int rc = ufoir__projector_tiles(p, c->A, &tiles, &n_tiles, NULL);
    if (rc)
        return rc;
    float best = 1e30f;
    for (int r = 0; r < 3; r++) {
        float t = 0.0f;
        if ((rc = udev_timer_begin(d)) ||
            (rc = udev_fp_tiles_cfg(d, &g, c, tiles, n_tiles, P, TP, sino, NULL, 0, sino, -1.0f, slices)) ||
            (rc = udev_timer_end(d, &t)))
            return rc;
        if (r > 0 && t < best)
            best = t;
    }
    *ms = best;
    return udev_take_kernel_error(d);
}

static int same_shape(const udev_fp_cfg *a, const udev_fp_cfg *b)
{
    return a->J == b->J && a->A == b->A && a->win == b->win && a->K == b->K && a->dsplit == b->dsplit;
}

int ufoir__fp_tune(ufoir_projector *p, int n_slices, ufoir_fp_tuning *out)
{
    ufoir_ctx *ctx = p->ctx;
    udev *d = ctx->dev;
    int rc;
    if (out)
        memset(out, 0, sizeof(*out));
    if (!p->have_geometry)
        return ufoir__fail(ctx, UFOIR_ERR_STATE, "autotune: the projector has no geometry yet");
    if (n_slices < 1)
        return UFOIR_ERR_INVALID;
    udev_geom g;
    ufoir__projector_geom(p, &g);
    const int A0 = udev_fp_tile_angles(d, (int) p->n_dets);
    if (A0 <= 0)
        return UFOIR_OK;              /* the row kernel serves this size; nothing to tune */

    struct ufoir__tune_entry *hit = tune_find(ctx, p, n_slices);
    if (hit) {
        p->fp_cfg = hit->cfg;
        p->fp_cfg_slices = n_slices;
        p->fp_cfg_valid = 1;
        if (out)
            *out = hit->info;
        return ufoir__projector_tiles(p, hit->cfg.A, NULL, NULL, NULL);
    }

    const size_t n = p->n_dets, na = p->n_angles, pitch = (size_t) udev_fp_pitch((int) n);
    /* the search runs on as many slices as fill the GPU twice with tiles
     * (at least 8) or on n_slices if fewer: with more, the GPU is as full */
    int S = n_slices;
    {
        int n_tiles0 = 0;
        rc = ufoir__projector_tiles(p, A0, NULL, &n_tiles0, NULL);
        if (rc)
            return rc;
        int fill = (2 * udev_sm_count(d) + n_tiles0 - 1) / (n_tiles0 > 0 ? n_tiles0 : 1);
        fill = fill > 8 ? fill : 8;
        S = S < fill ? S : fill;
    }
    float *P = NULL, *TP = NULL, *sino = NULL;
    udev_fp_cfg def, best;
    ufoir_fp_tuning info;
    memset(&info, 0, sizeof(info));
    UFOIR_TRY(ufoir__alloc(ctx, &P, n * pitch * (size_t) S));
    UFOIR_TRY(ufoir__alloc(ctx, &TP, n * pitch * (size_t) S));
    UFOIR_TRY(ufoir__alloc(ctx, &sino, na * n * (size_t) S));
    UFOIR_TRY(udev_memset(d, P, 0, n * pitch * (size_t) S * sizeof(float)));
    UFOIR_TRY(udev_memset(d, TP, 0, n * pitch * (size_t) S * sizeof(float)));
    UFOIR_TRY(udev_memset(d, sino, 0, na * n * (size_t) S * sizeof(float)));

    /* the fixed rules' shape for the real slice count */
    {
        const void *tiles = NULL;
        int n_tiles = 0;
        float spread = 0.0f;
        UFOIR_TRY(ufoir__projector_tiles(p, A0, &tiles, &n_tiles, &spread));
        UFOIR_TRY(udev_fp_default_cfg(d, &g, n_tiles, n_slices, spread, &def));
    }
    float t_def = 0.0f;
    UFOIR_TRY(time_shape(p, &def, P, TP, sino, S, &t_def));
    best = def;
    float t_best = t_def;
    info.candidates = 1;

    static const int As[3] = {8, 4, 2};
    static const int Js[4] = {1, 2, 4, 8};
    static const int Ks[3] = {32, 16, 8};
    const int sm = udev_sm_count(d);
    for (int ia = 0; ia < 3; ia++) {
        const int A = As[ia];
        int n_tiles = 0;
        float spread = 0.0f;
        UFOIR_TRY(ufoir__projector_tiles(p, A, NULL, &n_tiles, &spread));
        const int underfilled = (long long) n_tiles * S < 2LL * sm;
        for (int ij = 0; ij < 4; ij++)
            for (int win = 0; win <= 1; win++)
                for (int ik = 0; ik < 3; ik++)
                    for (int ds = 1; ds <= 8; ds *= 2) {
                        if ((ds > 1 || win) && !underfilled)
                            continue;
                        udev_fp_cfg c;
                        memset(&c, 0, sizeof(c));
                        c.J = Js[ij];
                        c.A = A;
                        c.win = win;
                        c.K = Ks[ik];
                        c.dsplit = ds;
                        if (udev_fp_cfg_finish(d, &g, spread, &c) != UFOIR_OK || same_shape(&c, &def))
                            continue;
                        /* split parts of fewer than 64 detectors only add overhead */
                        if (ds > 1 && c.dper < 64)
                            continue;
                        float t = 0.0f;
                        UFOIR_TRY(time_shape(p, &c, P, TP, sino, S, &t));
                        info.candidates++;
                        if (t < t_best) {
                            t_best = t;
                            best = c;
                        }
                    }
    }
    if (!(t_best < 0.98f * t_def)) {
        best = def;
        t_best = t_def;
    }
    info_of(&best, &info);
    info.tuned = 1;
    info.ms_default = t_def;
    info.ms_tuned = t_best;

    if (ctx->n_tune == ctx->cap_tune) {
        const int cap = ctx->cap_tune ? 2 * ctx->cap_tune : 16;
        struct ufoir__tune_entry *a = (struct ufoir__tune_entry *) realloc(ctx->tune, sizeof(*a) * (size_t) cap);
        if (!a) {
            rc = ufoir__fail(ctx, UFOIR_ERR_NOMEM, "out of host memory");
            goto done;
        }
        ctx->tune = a;
        ctx->cap_tune = cap;
    }
    {
        struct ufoir__tune_entry *e = &ctx->tune[ctx->n_tune++];
        e->n = p->n_dets;
        e->na = p->n_angles;
        e->step = p->lut_step;
        e->axis = ufoir__axis(p);
        e->arithmetic = p->prm.arithmetic;
        e->slices = n_slices;
        e->cfg = best;
        e->info = info;
    }
    p->fp_cfg = best;
    p->fp_cfg_slices = n_slices;
    p->fp_cfg_valid = 1;
    if (out)
        *out = info;
    rc = ufoir__projector_tiles(p, best.A, NULL, NULL, NULL);
done:
    ufoir__free(ctx, P);
    ufoir__free(ctx, TP);
    ufoir__free(ctx, sino);
    udev_sync(d);
    return rc;
}

int ufoir__fp_tune_wanted(ufoir_projector *p, int n_slices)
{
    const int mode = p->ctx->autotune;
    if (mode == UFOIR_AUTOTUNE_ON)
        return 1;
    if (mode != UFOIR_AUTOTUNE_AUTO || !p->have_geometry || n_slices < 1)
        return 0;
    /* the fixed rules' shape for this call (a shape already tuned for it is set aside) */
    const int valid = p->fp_cfg_valid;
    p->fp_cfg_valid = 0;
    udev_fp_cfg c;
    const void *tiles = NULL;
    int n_tiles = 0;
    const int rc = ufoir__fp_shape(p, n_slices, &c, &tiles, &n_tiles);
    p->fp_cfg_valid = valid;
    return rc == UFOIR_OK && c.dsplit > 1;
}

int ufoir_projector_autotune(ufoir_projector *proj, size_t n_slices, ufoir_fp_tuning *out)
{
    if (!proj || n_slices == 0 || n_slices > 65535)
        return UFOIR_ERR_INVALID;
    return ufoir__fp_tune(proj, (int) n_slices, out);
}
