/*
 * batch.c - mixed SIRT batches: one-slice SIRT jobs of different sizes and
 * angle counts advanced together by a fixed small set of launches per
 * iteration, captured once in a CUDA graph.
 *
 * A member's iteration is the SIRT update of src/tasks/ufo-ir-sirt-task.c:
 * 202-213, r = (b - A x) * R and x = x + C * (lambda A^T r), exactly as
 * ufoir__sirt_body runs it: the padded copies of x, the tiled forward
 * projection into r, the tiled backprojection with the update fused. The
 * batch runs these three steps for all members at once:
 *   1. pad_batch_kernel     one launch, 32 x 32 tiles of every member;
 *   2. fp_tiles_batch_kernel one launch per distinct forward launch shape
 *                           (members grouped by shape), one CTA per
 *                           (member, angle tile, detector part);
 *   3. bp_tiles_batch_kernel one launch, one CTA per (member, pixel tile).
 * Each launch walks a device work list: per member a record of its
 * arguments and an item range (exclusive prefix sums), biggest members
 * first so that the longest CTAs start first. An active flag per member
 * lets members be frozen without re-capturing.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "host.h"

#define MAX_FP_GROUPS 16

typedef struct {
    ufoir_projector *p;
    const float *b;
    float *x;
    float *R, *C;            /* weights, shared by the members of one geometry */
    float *resid, *P, *TP;
    float lambda;
    double cost;             /* interpolated samples per iteration */
    udev_fp_cfg cfg;
} member;

typedef struct {
    udev_fp_cfg cfg;
    int n_jobs, items;
    void *d_recs;
    int *d_start, *d_jidx;
} fp_group;

struct ufoir_batch {
    ufoir_ctx *ctx;
    int n;
    int owns;                /* 1: projectors, weights and member scratch are the batch's */
    member *m;
    ufoir_projector **projs;
    float **weights;         /* R and C per projector (2 per entry) */
    int n_projs;
    fp_group fp[MAX_FP_GROUPS];
    int n_fp;
    void *d_pad_recs;
    int *d_pad_start, *d_ident;
    int pad_items;
    struct {
        int n_jobs, items;
        void *d_recs;
        int *d_start, *d_jidx;
    } bp[2];                 /* backprojection lists: exact, fast arithmetic */
    int *d_active, *h_active;
    int active_dirty;
    void *exec;
    uint64_t exec_kernels;
};

static int cost_desc(const void *a, const void *b, void *ctx)
{
    const member *m = (const member *) ctx;
    const int i = *(const int *) a, j = *(const int *) b;
    if (m[i].cost != m[j].cost)
        return m[i].cost > m[j].cost ? -1 : 1;
    return i - j;
}

/* insertion sort of idx[0..k) by member cost, descending (stable) */
static void order_by_cost(const member *m, int *idx, int k)
{
    for (int a = 1; a < k; a++) {
        const int v = idx[a];
        int b = a;
        while (b > 0 && cost_desc(&idx[b - 1], &v, (void *) m) > 0) {
            idx[b] = idx[b - 1];
            b--;
        }
        idx[b] = v;
    }
}

static int same_launch(const udev_fp_cfg *a, const udev_fp_cfg *b)
{
    return a->J == b->J && a->A == b->A && a->win == b->win && a->threads == b->threads && a->smem == b->smem &&
           a->fm == b->fm;
}

/* Releases the work lists, device tables and captured iteration of
 * build_lists (so that they can be built again). */
static void free_lists(ufoir_batch *b)
{
    ufoir_ctx *ctx = b->ctx;
    udev_sync(ctx->dev);
    udev_graph_destroy(b->exec);
    b->exec = NULL;
    b->exec_kernels = 0;
    for (int k = 0; k < b->n_fp; k++) {
        ufoir__free(ctx, b->fp[k].d_recs);
        ufoir__free(ctx, b->fp[k].d_start);
        ufoir__free(ctx, b->fp[k].d_jidx);
    }
    memset(b->fp, 0, sizeof(b->fp));
    b->n_fp = 0;
    ufoir__free(ctx, b->d_pad_recs);
    ufoir__free(ctx, b->d_pad_start);
    ufoir__free(ctx, b->d_ident);
    b->d_pad_recs = NULL;
    b->d_pad_start = b->d_ident = NULL;
    for (int k = 0; k < 2; k++) {
        ufoir__free(ctx, b->bp[k].d_recs);
        ufoir__free(ctx, b->bp[k].d_start);
        ufoir__free(ctx, b->bp[k].d_jidx);
        b->bp[k].d_recs = NULL;
        b->bp[k].d_start = b->bp[k].d_jidx = NULL;
        b->bp[k].n_jobs = b->bp[k].items = 0;
    }
    ufoir__free(ctx, b->d_active);
    b->d_active = NULL;
}

void ufoir_batch_destroy(ufoir_batch *b)
{
    if (!b)
        return;
    ufoir_ctx *ctx = b->ctx;
    udev *d = ctx->dev;
    free_lists(b);
    for (int i = 0; i < b->n && b->owns; i++) {
        ufoir__free(ctx, b->m[i].resid);
        ufoir__free(ctx, b->m[i].P);
        ufoir__free(ctx, b->m[i].TP);
    }
    for (int i = 0; i < b->n_projs; i++) {
        ufoir__free(ctx, b->weights[2 * i]);
        ufoir__free(ctx, b->weights[2 * i + 1]);
        ufoir_projector_destroy(b->projs[i]);
    }
    /* weights/projs exist only for batches made by ufoir_batch_create */
    udev_sync(d);
    free(b->weights);
    free(b->projs);
    free(b->m);
    free(b->h_active);
    free(b);
}

/* device copy of a host table (complete on return: the host buffer is reused) */
static int upload(ufoir_ctx *ctx, void **dst, const void *src, size_t bytes)
{
    int rc = udev_malloc(ctx->dev, dst, bytes ? bytes : 16);
    if (!rc && bytes)
        rc = udev_memcpy(ctx->dev, *dst, src, bytes);
    return rc;
}

static int check_job(ufoir_ctx *ctx, const ufoir_batch_job *j, size_t i)
{
    if (j->n_dets == 0 || j->n_dets > 65535 || j->n_angles < 16 || !j->sino || !j->vol)
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "batch member %zu: %u x %u (at least 16 angles) or no buffers", i,
                           j->n_dets, j->n_angles);
    if (!(j->relaxation_factor >= 0.0f && j->relaxation_factor <= 1.0f) || !(j->step >= 0.0f) ||
        !(j->axis_position >= -1.0f) || (j->arithmetic != UFOIR_ARITH_EXACT && j->arithmetic != UFOIR_ARITH_FAST))
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "batch member %zu: relaxation_factor, step or axis out of range",
                           i);
    if (!udev_is_device_ptr(ctx->dev, j->sino) || !udev_is_device_ptr(ctx->dev, j->vol))
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "batch member %zu: sinogram and volume must be device memory", i);
    /* the tiled backprojector needs ordered clamp edges (axis at least half
     * a pixel inside the image) */
    const float n = (float) j->n_dets;
    const float axis = j->axis_position < 0.0f ? n / 2.0f : j->axis_position;
    const float half = n - axis * 2.0f < 0.0f ? n - axis : axis;
    if (!(axis - half + 0.5f <= axis + half - 0.5f))
        return ufoir__fail(ctx, UFOIR_ERR_UNSUPPORTED, "batch member %zu: axis %g at the image edge", i,
                           (double) axis);
    return UFOIR_OK;
}

/* Work lists, device tables and the captured iteration of b->m[0..n). */
static int build_lists(ufoir_batch *b)
{
    ufoir_ctx *ctx = b->ctx;
    udev *d = ctx->dev;
    const int n = b->n;
    int rc = UFOIR_OK;
    const size_t fp_rec = udev_fp_record_bytes(), bp_rec = udev_bp_record_bytes(), pad_rec = udev_pad_record_bytes();
    size_t rec_max = fp_rec > bp_rec ? fp_rec : bp_rec;
    rec_max = rec_max > pad_rec ? rec_max : pad_rec;
    unsigned char *recs = (unsigned char *) malloc(rec_max * (size_t) n);
    int *starts = (int *) malloc(sizeof(int) * (size_t) n);
    int *jidx = (int *) malloc(sizeof(int) * (size_t) n);
    int *idx = (int *) malloc(sizeof(int) * (size_t) n);
    int *grouped = (int *) calloc((size_t) n, sizeof(int));
    if (!recs || !starts || !jidx || !idx || !grouped) {
        rc = ufoir__fail(ctx, UFOIR_ERR_NOMEM, "out of host memory");
        goto done;
    }
    for (int i = 0; i < n; i++) {
        idx[i] = i;
        b->h_active[i] = 1;
    }
    order_by_cost(b->m, idx, n);

    /* 1. padding: all members, biggest first */
    {
        int items = 0;
        for (int k = 0; k < n; k++) {
            const member *m = &b->m[idx[k]];
            int it = 0;
            udev_pad_record((int) m->p->n_dets, m->x, m->P, m->TP, recs + pad_rec * (size_t) k, &it);
            starts[k] = items;
            jidx[k] = idx[k];
            items += it;
        }
        b->pad_items = items;
        UFOIR_TRY(upload(ctx, &b->d_pad_recs, recs, pad_rec * (size_t) n));
        UFOIR_TRY(upload(ctx, (void **) &b->d_pad_start, starts, sizeof(int) * (size_t) n));
        UFOIR_TRY(upload(ctx, (void **) &b->d_ident, jidx, sizeof(int) * (size_t) n));
    }
    /* 2. forward projection: one group per launch shape */
    for (int k0 = 0; k0 < n; k0++) {
        const int lead = idx[k0];
        if (grouped[lead])
            continue;
        if (b->n_fp == MAX_FP_GROUPS) {
            rc = ufoir__fail(ctx, UFOIR_ERR_UNSUPPORTED, "batch: more than %d forward launch shapes", MAX_FP_GROUPS);
            goto done;
        }
        fp_group *gr = &b->fp[b->n_fp];
        gr->cfg = b->m[lead].cfg;
        int cnt = 0, items = 0;
        for (int k = k0; k < n; k++) {
            const int i = idx[k];
            member *m = &b->m[i];
            if (grouped[i] || !same_launch(&m->cfg, &gr->cfg))
                continue;
            udev_geom g;
            ufoir__projector_geom(m->p, &g);
            const void *tiles = NULL;
            int n_tiles = 0, it = 0;
            UFOIR_TRY(ufoir__projector_tiles(m->p, m->cfg.A, &tiles, &n_tiles, NULL));
            UFOIR_TRY(udev_fp_record(d, &g, &m->cfg, tiles, n_tiles, m->P, m->TP, m->b, m->R, m->resid, -1.0f,
                                     recs + fp_rec * (size_t) cnt, &it));
            starts[cnt] = items;
            jidx[cnt] = i;
            items += it;
            cnt++;
            grouped[i] = 1;
        }
        gr->n_jobs = cnt;
        gr->items = items;
        UFOIR_TRY(upload(ctx, &gr->d_recs, recs, fp_rec * (size_t) cnt));
        UFOIR_TRY(upload(ctx, (void **) &gr->d_start, starts, sizeof(int) * (size_t) cnt));
        UFOIR_TRY(upload(ctx, (void **) &gr->d_jidx, jidx, sizeof(int) * (size_t) cnt));
        b->n_fp++;
    }
    /* 3. backprojection with the SIRT update: all members of one arithmetic,
     * biggest first */
    for (int fm = 0; fm <= 1; fm++) {
        int items = 0, cnt = 0;
        for (int k = 0; k < n; k++) {
            const member *m = &b->m[idx[k]];
            if ((m->p->prm.arithmetic == UFOIR_ARITH_FAST) != fm)
                continue;
            udev_geom g;
            ufoir__projector_geom(m->p, &g);
            int it = 0;
            UFOIR_TRY(udev_bp_record(d, &g, m->p->subsets, (int) m->p->n_subsets, m->resid, NULL, m->C, m->x, m->x,
                                     m->lambda, recs + bp_rec * (size_t) cnt, &it));
            starts[cnt] = items;
            jidx[cnt] = idx[k];
            items += it;
            cnt++;
        }
        b->bp[fm].n_jobs = cnt;
        b->bp[fm].items = items;
        if (cnt == 0)
            continue;
        UFOIR_TRY(upload(ctx, &b->bp[fm].d_recs, recs, bp_rec * (size_t) cnt));
        UFOIR_TRY(upload(ctx, (void **) &b->bp[fm].d_start, starts, sizeof(int) * (size_t) cnt));
        UFOIR_TRY(upload(ctx, (void **) &b->bp[fm].d_jidx, jidx, sizeof(int) * (size_t) cnt));
    }
    UFOIR_TRY(upload(ctx, (void **) &b->d_active, b->h_active, sizeof(int) * (size_t) n));

    /* one iteration, captured */
    UFOIR_TRY(udev_capture_begin(d));
    rc = udev_pad_batch(d, b->d_pad_recs, b->d_pad_start, n, b->d_ident, b->d_active, b->pad_items);
    for (int k = 0; k < b->n_fp && !rc; k++)
        rc = udev_fp_batch(d, &b->fp[k].cfg, b->fp[k].d_recs, b->fp[k].d_start, b->fp[k].n_jobs, b->fp[k].d_jidx,
                           b->d_active, b->fp[k].items);
    for (int fm = 0; fm <= 1 && !rc; fm++)
        if (b->bp[fm].n_jobs > 0)
            rc = udev_bp_batch(d, fm, b->bp[fm].d_recs, b->bp[fm].d_start, b->bp[fm].n_jobs, b->bp[fm].d_jidx,
                               b->d_active, b->bp[fm].items);
    {
        const int rc2 = udev_capture_end(d, &b->exec, &b->exec_kernels);
        if (!rc)
            rc = rc2;
    }
done:
    free(recs);
    free(starts);
    free(jidx);
    free(idx);
    free(grouped);
    return rc;
}

/* The member's launch shape for `slices` slices, with chunks small enough
 * that the batch kernel's record fits beside its stages. */
static int member_shape(ufoir_ctx *ctx, member *m, int slices)
{
    udev *d = ctx->dev;
    const void *tiles = NULL;
    int n_tiles = 0;
    int rc = ufoir__fp_shape(m->p, slices, &m->cfg, &tiles, &n_tiles);
    if (rc == UFOIR_ERR_UNSUPPORTED)
        return ufoir__fail(ctx, rc, "batch: the tiled forward projector cannot serve n_dets %u", m->p->n_dets);
    while (!rc && !udev_fp_batch_fits(d, &m->cfg) && m->cfg.K > 4) {
        udev_geom g;
        float spread = 0.0f;
        ufoir__projector_geom(m->p, &g);
        rc = ufoir__projector_tiles(m->p, m->cfg.A, NULL, NULL, &spread);
        m->cfg.K /= 2;
        if (!rc)
            rc = udev_fp_cfg_finish(d, &g, spread, &m->cfg);
    }
    return rc;
}

static ufoir_batch *batch_alloc(ufoir_ctx *ctx, int n)
{
    ufoir_batch *b = (ufoir_batch *) calloc(1, sizeof(*b));
    if (!b)
        return NULL;
    b->ctx = ctx;
    b->n = n;
    b->m = (member *) calloc((size_t) n, sizeof(member));
    b->h_active = (int *) malloc(sizeof(int) * (size_t) n);
    if (!b->m || !b->h_active) {
        free(b->m);
        free(b->h_active);
        free(b);
        return NULL;
    }
    return b;
}

int ufoir__batch_build(ufoir_ctx *ctx, const ufoir__bmember *mem, int n, ufoir_batch **out)
{
    *out = NULL;
    if (n <= 0)
        return UFOIR_ERR_INVALID;
    ufoir_batch *b = batch_alloc(ctx, n);
    if (!b)
        return ufoir__fail(ctx, UFOIR_ERR_NOMEM, "out of host memory");
    int rc = UFOIR_OK;
    /* as in ufoir_batch_create: shapes for a full GPU when the members'
     * tiles fill it twice over */
    const int sm = udev_sm_count(ctx->dev);
    long long total = 0;
    for (int i = 0; i < n && !rc; i++) {
        const int A = udev_fp_tile_angles(ctx->dev, (int) mem[i].p->n_dets);
        int nt = 0;
        if (A > 0)
            rc = ufoir__projector_tiles(mem[i].p, A, NULL, &nt, NULL);
        total += nt;
        b->m[i].cost = (double) nt;       /* tiles, until the cost below */
    }
    for (int i = 0; i < n && !rc; i++) {
        member *m = &b->m[i];
        const int nt = (int) m->cost;
        int slices = mem[i].shape_slices;
        if (total >= 2LL * sm && nt > 0) {
            const int fill = (2 * sm + nt - 1) / nt;
            slices = slices > fill ? slices : fill;
        }
        m->p = mem[i].p;
        m->b = mem[i].b;
        m->x = mem[i].x;
        m->R = mem[i].R;
        m->C = mem[i].C;
        m->resid = mem[i].resid;
        m->P = mem[i].P;
        m->TP = mem[i].TP;
        m->lambda = mem[i].lambda;
        m->cost = 2.0 * (double) m->p->n_dets * (double) m->p->n_dets * (double) m->p->n_angles;
        rc = member_shape(ctx, m, slices);
    }
    if (!rc)
        rc = build_lists(b);
    if (rc) {
        ufoir_batch_destroy(b);
        return rc;
    }
    *out = b;
    return UFOIR_OK;
}

int ufoir__batch_launch(ufoir_batch *b, unsigned int iterations)
{
    udev *d = b->ctx->dev;
    int rc;
    if (b->active_dirty) {
        if ((rc = udev_memcpy_async(d, b->d_active, b->h_active, sizeof(int) * (size_t) b->n)))
            return rc;
        b->active_dirty = 0;
    }
    for (unsigned int i = 0; i < iterations; i++)
        if ((rc = udev_graph_launch(d, b->exec, b->exec_kernels)))
            return rc;
    return UFOIR_OK;
}

/* The launch-shape slice count of each geometry. When the batch's tiles fill
 * the GPU twice over, a member's shape is chosen as for a GPU full of work
 * (as many slices as fill it with this geometry's tiles): no detector
 * splits, whose extra CTAs only pay when a projection has too few tiles.
 * Otherwise as for the members sharing the geometry alone. */
static int shape_slices(ufoir_ctx *ctx, ufoir_projector **projs, const int *count, int n_projs, int *eff)
{
    udev *d = ctx->dev;
    const int sm = udev_sm_count(d);
    long long total = 0;
    int *tiles = (int *) calloc((size_t) n_projs, sizeof(int));
    if (!tiles)
        return ufoir__fail(ctx, UFOIR_ERR_NOMEM, "out of host memory");
    int rc = UFOIR_OK;
    for (int g = 0; g < n_projs && !rc; g++) {
        const int A = udev_fp_tile_angles(d, (int) projs[g]->n_dets);
        if (A > 0)
            rc = ufoir__projector_tiles(projs[g], A, NULL, &tiles[g], NULL);
        total += (long long) tiles[g] * count[g];
    }
    for (int g = 0; g < n_projs && !rc; g++) {
        eff[g] = count[g];
        if (total >= 2LL * sm && tiles[g] > 0) {
            const int fill = (2 * sm + tiles[g] - 1) / tiles[g];
            eff[g] = eff[g] > fill ? eff[g] : fill;
        }
    }
    free(tiles);
    return rc;
}

/* Milliseconds of `iters` iterations of the batch as built, after one
 * untimed one. The members' volumes are saved first and put back after, so
 * the batch starts from them as if it had not run. */
static int time_batch(ufoir_batch *b, unsigned int iters, float *ms)
{
    ufoir_ctx *ctx = b->ctx;
    udev *d = ctx->dev;
    size_t total = 0;
    for (int i = 0; i < b->n; i++)
        total += (size_t) b->m[i].p->n_dets * b->m[i].p->n_dets;
    float *save = NULL;
    int rc = ufoir__alloc(ctx, &save, total);
    for (size_t i = 0, off = 0; (int) i < b->n && !rc; off += (size_t) b->m[i].p->n_dets * b->m[i].p->n_dets, i++)
        rc = udev_memcpy_async(d, save + off, b->m[i].x, sizeof(float) * b->m[i].p->n_dets * b->m[i].p->n_dets);
    if (!rc)
        rc = ufoir__batch_launch(b, 1);
    if (!rc)
        rc = udev_timer_begin(d);
    if (!rc)
        rc = ufoir__batch_launch(b, iters);
    if (!rc)
        rc = udev_timer_end(d, ms);
    for (size_t i = 0, off = 0; (int) i < b->n && !rc; off += (size_t) b->m[i].p->n_dets * b->m[i].p->n_dets, i++)
        rc = udev_memcpy_async(d, b->m[i].x, save + off, sizeof(float) * b->m[i].p->n_dets * b->m[i].p->n_dets);
    if (!rc)
        rc = udev_sync(d);
    if (!rc)
        rc = udev_take_kernel_error(d);
    ufoir__free(ctx, save);
    return rc;
}

/* Launch shapes from the projectors' current state, then the lists. */
static int shape_and_build(ufoir_batch *b, const int *geo_of, const int *geo_eff)
{
    free_lists(b);
    for (int i = 0; i < b->n; i++) {
        const int rc = member_shape(b->ctx, &b->m[i], geo_eff[geo_of[i]]);
        if (rc)
            return rc;
    }
    return build_lists(b);
}

int ufoir_batch_create(ufoir_ctx *ctx, const ufoir_batch_job *jobs, size_t n_jobs, ufoir_batch **out)
{
    if (!ctx || !jobs || !out || n_jobs == 0 || n_jobs > 65535)
        return UFOIR_ERR_INVALID;
    *out = NULL;
    udev *d = ctx->dev;
    int rc;
    for (size_t i = 0; i < n_jobs; i++)
        if ((rc = check_job(ctx, &jobs[i], i)))
            return rc;
    const int n = (int) n_jobs;
    ufoir_batch *b = batch_alloc(ctx, n);
    int *geo_count = (int *) calloc((size_t) n, sizeof(int));
    int *geo_of = (int *) malloc(sizeof(int) * (size_t) n);
    int *geo_eff = (int *) calloc((size_t) n, sizeof(int));
    if (b) {
        b->owns = 1;
        b->projs = (ufoir_projector **) calloc((size_t) n, sizeof(void *));
        b->weights = (float **) calloc(2 * (size_t) n, sizeof(float *));
    }
    if (!b || !b->projs || !b->weights || !geo_count || !geo_of || !geo_eff) {
        rc = ufoir__fail(ctx, UFOIR_ERR_NOMEM, "out of host memory");
        goto done;
    }
    /* one projector (LUT, subsets, tiles, weights) per distinct geometry */
    for (int i = 0; i < n; i++) {
        const ufoir_batch_job *j = &jobs[i];
        int g = -1;
        for (int k = 0; k < b->n_projs && g < 0; k++) {
            const ufoir_projector *p = b->projs[k];
            if (p->n_dets == j->n_dets && p->n_angles == j->n_angles && p->prm.step == j->step &&
                p->prm.axis_position == j->axis_position && p->prm.arithmetic == j->arithmetic)
                g = k;
        }
        if (g < 0) {
            ufoir_projector_params pp;
            ufoir_projector_params_init(&pp);
            pp.is_forward = 0;
            pp.step = j->step;
            pp.axis_position = j->axis_position;
            pp.angles_num = j->n_angles;
            pp.arithmetic = j->arithmetic;
            g = b->n_projs;
            UFOIR_TRY(ufoir_projector_create(ctx, &pp, &b->projs[g]));
            b->n_projs++;
            ufoir_projector *p = b->projs[g];
            UFOIR_TRY(ufoir__projector_prepare_na(p, j->n_dets, j->n_angles));
            if (p->n_subsets > 16) {
                rc = ufoir__fail(ctx, UFOIR_ERR_UNSUPPORTED, "batch member %d: %u direction runs (at most 16)", i,
                                 p->n_subsets);
                goto done;
            }
            const size_t nn = j->n_dets, nv = nn * nn, ns = nn * j->n_angles;
            float *R = NULL, *C = NULL, *tmp = NULL;
            UFOIR_TRY(ufoir__alloc(ctx, &R, ns));
            b->weights[2 * g] = R;
            UFOIR_TRY(ufoir__alloc(ctx, &C, nv));
            b->weights[2 * g + 1] = C;
            UFOIR_TRY(ufoir__alloc(ctx, &tmp, ns));
            /* weights with relaxation 1 and correction scale 1 (sirt-task.c:176-193);
             * C serves as the all-ones image before it receives its own values */
            p->prm.relaxation = 1.0f;
            p->prm.correction_scale = 1.0f;
            rc = ufoir__ray_weights(p, R, C);
            if (!rc)
                rc = ufoir__pixel_weights(p, C, tmp);
            ufoir__free(ctx, tmp);
            if (rc)
                goto done;
        }
        geo_of[i] = g;
        geo_count[g]++;
    }
    UFOIR_TRY(shape_slices(ctx, b->projs, geo_count, b->n_projs, geo_eff));
    /* With autotune on, each geometry's shape is searched alone. In a batch a
     * tuned shape that differs from the fixed rules' adds a launch unless
     * other members share it, so the batch with the tuned shapes is timed
     * against the batch with the rules' shapes below and the faster kept. */
    int any_tuned = 0;
    if (ctx->autotune == UFOIR_AUTOTUNE_ON)
        for (int g = 0; g < b->n_projs; g++) {
            ufoir_fp_tuning t;
            UFOIR_TRY(ufoir__fp_tune(b->projs[g], geo_eff[g], &t));
            any_tuned |= b->projs[g]->fp_cfg_valid;
        }
    for (int i = 0; i < n; i++) {
        const ufoir_batch_job *j = &jobs[i];
        member *m = &b->m[i];
        ufoir_projector *p = b->projs[geo_of[i]];
        const size_t nn = j->n_dets, ns = nn * j->n_angles, pitch = (size_t) udev_fp_pitch((int) nn);
        m->p = p;
        m->b = j->sino;
        m->x = j->vol;
        m->R = b->weights[2 * geo_of[i]];
        m->C = b->weights[2 * geo_of[i] + 1];
        m->lambda = j->relaxation_factor;
        m->cost = 2.0 * (double) nn * (double) nn * (double) j->n_angles;
        UFOIR_TRY(ufoir__alloc(ctx, &m->resid, ns));
        UFOIR_TRY(ufoir__alloc(ctx, &m->P, nn * pitch));
        UFOIR_TRY(ufoir__alloc(ctx, &m->TP, nn * pitch));
        UFOIR_TRY(udev_memset(d, m->P, 0, nn * pitch * sizeof(float)));
        UFOIR_TRY(udev_memset(d, m->TP, 0, nn * pitch * sizeof(float)));
        if (!j->keep_vol)
            UFOIR_TRY(udev_fill(d, m->x, nn * nn, 0.0f));
    }
    UFOIR_TRY(shape_and_build(b, geo_of, geo_eff));
    if (any_tuned) {
        /* Where a tuned shape differs from the rules' one, the batch with the
         * tuned shapes is timed against the batch with the rules' shapes, two
         * iterations each on the members' own data (restored after), and the
         * faster is kept. Every member's values are the same either way (the
         * projections are invariant to the launch shape). */
        int *valid = (int *) malloc(sizeof(int) * (size_t) b->n_projs);
        udev_fp_cfg *tuned = (udev_fp_cfg *) malloc(sizeof(udev_fp_cfg) * (size_t) n);
        if (!valid || !tuned) {
            free(valid);
            free(tuned);
            rc = ufoir__fail(ctx, UFOIR_ERR_NOMEM, "out of host memory");
            goto done;
        }
        for (int g = 0; g < b->n_projs; g++) {
            valid[g] = b->projs[g]->fp_cfg_valid;
            b->projs[g]->fp_cfg_valid = 0;
        }
        int differs = 0;
        for (int i = 0; i < n && !rc; i++) {
            tuned[i] = b->m[i].cfg;
            rc = member_shape(ctx, &b->m[i], geo_eff[geo_of[i]]);     /* the rules' shape */
            differs |= !same_launch(&tuned[i], &b->m[i].cfg);
        }
        float ms_tuned = 0.0f, ms_rules = 0.0f;
        if (!rc && differs) {
            rc = time_batch(b, 2, &ms_tuned);           /* the lists built so far are the tuned ones */
            if (!rc) {
                free_lists(b);
                rc = build_lists(b);
            }
            if (!rc)
                rc = time_batch(b, 2, &ms_rules);
        }
        for (int g = 0; g < b->n_projs; g++)
            b->projs[g]->fp_cfg_valid = valid[g];
        if (!rc && differs && ms_tuned < ms_rules)
            rc = shape_and_build(b, geo_of, geo_eff);
        else if (!rc && differs)
            for (int g = 0; g < b->n_projs; g++)
                b->projs[g]->fp_cfg_valid = 0;          /* the rules' shapes stay */
        else
            for (int i = 0; i < n; i++)
                b->m[i].cfg = tuned[i];
        free(valid);
        free(tuned);
        if (rc)
            goto done;
    }
    UFOIR_TRY(udev_sync(d));
    *out = b;
    b = NULL;
done:
    free(geo_count);
    free(geo_of);
    free(geo_eff);
    if (b)
        ufoir_batch_destroy(b);
    return rc;
}

int ufoir_batch_run(ufoir_batch *b, unsigned int iterations)
{
    if (!b)
        return UFOIR_ERR_INVALID;
    const int rc = ufoir__batch_launch(b, iterations);
    return rc ? rc : udev_take_kernel_error(b->ctx->dev);
}

int ufoir_batch_set_active(ufoir_batch *b, size_t member_i, int active)
{
    if (!b || member_i >= (size_t) b->n || (active != 0 && active != 1))
        return UFOIR_ERR_INVALID;
    if (b->h_active[member_i] != active) {
        b->h_active[member_i] = active;
        b->active_dirty = 1;
    }
    return UFOIR_OK;
}

int ufoir_batch_launches(const ufoir_batch *b, unsigned int *launches, unsigned int *fp_shapes)
{
    if (!b)
        return UFOIR_ERR_INVALID;
    if (launches)
        *launches = (unsigned int) b->exec_kernels;
    if (fp_shapes)
        *fp_shapes = (unsigned int) b->n_fp;
    return UFOIR_OK;
}
