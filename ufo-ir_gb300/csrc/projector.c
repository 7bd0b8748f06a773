/*
 * projector.c - the "parallel-projector" plugin on the GPU: properties,
 * requisition (sin/cos LUT and direction subsets), process, forward,
 * backward and single-subset FP/BP
 * (src/tasks/ufo-ir-parallel-projector-task.c,
 *  src/core/ufo-ir-projector-task.c, src/core/ufo-ir-state-dependent-task.c).
 */
#include <ctype.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "host.h"

void ufoir_projector_params_init(ufoir_projector_params *p)
{
    if (!p)
        return;
    memset(p, 0, sizeof(*p));
    strcpy(p->model, "joseph");      /* …parallel-projector-task.c:148 */
    p->angles_num = 0;               /* :149 */
    p->is_forward = 1;               /* ufo-ir-state-dependent-task.c:96 */
    p->axis_position = -1.0f;        /* ufo-ir-projector-task.c:107 */
    p->step = 0.0f;                  /* :108 */
    p->relaxation = 1.0f;            /* :109 */
    p->correction_scale = 1.0f;      /* :110 */
    p->arithmetic = UFOIR_ARITH_EXACT;
}

static int check_params(ufoir_ctx *ctx, ufoir_projector_params *p)
{
    char lower[sizeof(p->model)];
    size_t i;
    for (i = 0; i + 1 < sizeof(lower) && p->model[i]; i++)
        lower[i] = (char) tolower((unsigned char) p->model[i]);
    lower[i] = 0;
    /* set_model lower-cases the name (…parallel-projector-task.c:283-287).
     * "joseph" is the reference's model (projector-parallel-joseph.cl);
     * "siddon" adds exact line integrals of the pixel image (udev_siddon.cu),
     * for the projector's own forward / backward / subset calls. */
    if (strcmp(lower, "joseph") != 0 && strcmp(lower, "siddon") != 0)
        return ufoir__fail(ctx, UFOIR_ERR_UNSUPPORTED,
                           "projector model '%s' is not available ('joseph' or 'siddon')", p->model);
    memcpy(p->model, lower, sizeof(lower));
    /* GParamSpec ranges (ufo-ir-projector-task.c:68-93). */
    if (!(p->axis_position >= -1.0f))
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "axis_position %g outside [-1, MAX]", (double) p->axis_position);
    if (!(p->step >= 0.0f))
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "step %g outside [0, MAX]", (double) p->step);
    if (!isfinite(p->relaxation) || !isfinite(p->correction_scale))
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "relaxation/correction_scale must be finite");
    if (p->arithmetic != UFOIR_ARITH_EXACT && p->arithmetic != UFOIR_ARITH_FAST)
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "arithmetic %d is neither exact (0) nor fast (1)", p->arithmetic);
    return UFOIR_OK;
}

int ufoir_projector_create(ufoir_ctx *ctx, const ufoir_projector_params *p, ufoir_projector **out)
{
    if (!ctx || !out)
        return UFOIR_ERR_INVALID;
    *out = NULL;
    ufoir_projector_params q;
    if (p)
        q = *p;
    else
        ufoir_projector_params_init(&q);
    int rc = check_params(ctx, &q);
    if (rc)
        return rc;
    ufoir_projector *proj = (ufoir_projector *) calloc(1, sizeof(*proj));
    if (!proj)
        return ufoir__fail(ctx, UFOIR_ERR_NOMEM, "out of host memory");
    proj->ctx = ctx;
    proj->prm = q;
    *out = proj;
    return UFOIR_OK;
}

static void free_geometry(ufoir_projector *p)
{
    free(p->h_sin);
    free(p->h_cos);
    free(p->h_dir);
    free(p->subsets);
    p->h_sin = p->h_cos = NULL;
    p->h_dir = NULL;
    p->subsets = NULL;
    if (p->d_sin)
        udev_free(p->ctx->dev, p->d_sin);
    if (p->d_cos)
        udev_free(p->ctx->dev, p->d_cos);
    if (p->d_dir)
        udev_free(p->ctx->dev, p->d_dir);
    for (int k = 0; k < 4; k++) {
        if (p->d_tiles[k])
            udev_free(p->ctx->dev, p->d_tiles[k]);
        p->d_tiles[k] = NULL;
        p->tiles_valid[k] = 0;
    }
    p->fp_cfg_valid = 0;
    p->d_sin = p->d_cos = NULL;
    p->d_dir = NULL;
    p->lut_cap = 0;
    p->have_geometry = 0;
}

void ufoir_projector_destroy(ufoir_projector *proj)
{
    if (!proj)
        return;
    free_geometry(proj);
    udev_sync(proj->ctx->dev);
    free(proj);
}

int ufoir_projector_get_params(const ufoir_projector *proj, ufoir_projector_params *p)
{
    if (!proj || !p)
        return UFOIR_ERR_INVALID;
    *p = proj->prm;
    return UFOIR_OK;
}

int ufoir_projector_set_params(ufoir_projector *proj, const ufoir_projector_params *p)
{
    if (!proj || !p)
        return UFOIR_ERR_INVALID;
    ufoir_projector_params q = *p;
    int rc = check_params(proj->ctx, &q);
    if (rc)
        return rc;
    /* a tuned launch shape belongs to the axis and arithmetic it was timed
     * with (the tile lists stay: graphs captured earlier may refer to them) */
    if (q.axis_position != proj->prm.axis_position || q.arithmetic != proj->prm.arithmetic)
        proj->fp_cfg_valid = 0;
    proj->prm = q;
    return UFOIR_OK;
}

float ufoir__axis(const ufoir_projector *p)
{
    /* axis_position < 0 means dims[0] / 2.0 (…parallel-projector-task.c:524-527, :584-587). */
    float axis = p->prm.axis_position;
    if (axis < 0)
        axis = (float) (p->n_dets / 2.0);
    return axis;
}

/* create_lut_buffer (…parallel-projector-task.c:437-460) and
 * generate_full_subsets_list (:462-498). */
static int build_geometry(ufoir_projector *p, unsigned int n_angles)
{
    ufoir_ctx *ctx = p->ctx;
    const unsigned int cap = n_angles ? n_angles : 1;
    if (cap > p->lut_cap) {
        free_geometry(p);
        p->h_sin = (float *) malloc(sizeof(float) * cap);
        p->h_cos = (float *) malloc(sizeof(float) * cap);
        p->h_dir = (unsigned char *) malloc(cap);
        p->subsets = (ufoir_subset *) malloc(sizeof(ufoir_subset) * cap);
        if (!p->h_sin || !p->h_cos || !p->h_dir || !p->subsets) {
            free_geometry(p);
            return ufoir__fail(ctx, UFOIR_ERR_NOMEM, "out of host memory");
        }
        int rc = udev_malloc(ctx->dev, (void **) &p->d_sin, sizeof(float) * cap);
        if (!rc)
            rc = udev_malloc(ctx->dev, (void **) &p->d_cos, sizeof(float) * cap);
        if (!rc)
            rc = udev_malloc(ctx->dev, (void **) &p->d_dir, cap);
        if (rc) {
            free_geometry(p);
            return rc;
        }
        p->lut_cap = cap;
    }
    const float step = p->prm.step;
    for (unsigned int i = 0; i < n_angles; i++) {
        /* guint * gfloat is a float product; sin/cos run in double. */
        const float angle = (float) i * step;
        p->h_sin[i] = (float) sin((double) angle);
        p->h_cos[i] = (float) cos((double) angle);
    }
    unsigned int idx = 0;
    if (n_angles > 0) {
        int direction = fabs((double) p->h_sin[0]) <= fabs((double) p->h_cos[0]);
        p->subsets[0].direction = direction;
        p->subsets[0].offset = 0;
        p->subsets[0].n = 1;
        p->h_dir[0] = (unsigned char) direction;
        for (unsigned int i = 1; i < n_angles; ++i) {
            direction = fabs((double) p->h_sin[i]) <= fabs((double) p->h_cos[i]);
            p->h_dir[i] = (unsigned char) direction;
            if (direction != p->subsets[idx].direction) {
                idx++;
                p->subsets[idx].direction = direction;
                p->subsets[idx].offset = i;
                p->subsets[idx].n = 1;
            } else {
                p->subsets[idx].n++;
            }
        }
        idx++;
    }
    p->n_subsets = idx;
    int rc = udev_memcpy_async(ctx->dev, p->d_sin, p->h_sin, sizeof(float) * n_angles);
    if (!rc)
        rc = udev_memcpy_async(ctx->dev, p->d_cos, p->h_cos, sizeof(float) * n_angles);
    if (!rc)
        rc = udev_memcpy(ctx->dev, p->d_dir, p->h_dir, n_angles);
    if (rc)
        return rc;
    p->n_angles = n_angles;
    p->lut_step = step;
    p->have_geometry = 1;
    for (int k = 0; k < 4; k++)
        p->tiles_valid[k] = 0;
    p->fp_cfg_valid = 0;
    return UFOIR_OK;
}

int ufoir__projector_prepare_na(ufoir_projector *p, unsigned int n_dets, unsigned int n_angles)
{
    if (n_dets == 0)
        return ufoir__fail(p->ctx, UFOIR_ERR_INVALID, "n_dets must be > 0");
    if (n_dets > 65535)
        return ufoir__fail(p->ctx, UFOIR_ERR_INVALID, "n_dets %u exceeds 65535", n_dets);
    /* The reference rebuilds the LUT only when the angle count changes; a
     * changed step is also honoured here (the reference would keep a stale LUT). */
    if (!p->have_geometry || p->n_angles != n_angles || p->lut_step != p->prm.step) {
        int rc = build_geometry(p, n_angles);
        if (rc)
            return rc;
    }
    p->n_dets = n_dets;
    return UFOIR_OK;
}

int ufoir__projector_prepare(ufoir_projector *p, const size_t in_dims[2])
{
    if (!in_dims || in_dims[0] == 0 || in_dims[1] == 0)
        return ufoir__fail(p->ctx, UFOIR_ERR_INVALID, "input dims must be non-zero");
    /* angles_num == 0 takes the input's dims[1] and keeps it (:315-317). */
    if (p->prm.angles_num == 0)
        p->prm.angles_num = (unsigned int) in_dims[1];
    return ufoir__projector_prepare_na(p, (unsigned int) in_dims[0], p->prm.angles_num);
}

void ufoir__projector_geom(const ufoir_projector *p, udev_geom *g)
{
    g->n_dets = (int) p->n_dets;
    g->n_angles = (int) p->n_angles;
    g->axis = ufoir__axis(p);
    g->d_sin = p->d_sin;
    g->d_cos = p->d_cos;
    g->d_dir = p->d_dir;
    g->fast_arith = p->prm.arithmetic == UFOIR_ARITH_FAST;
}

int ufoir_projector_get_requisition(ufoir_projector *proj, const size_t in_dims[2], size_t out_dims[2])
{
    if (!proj || !in_dims || !out_dims)
        return UFOIR_ERR_INVALID;
    int rc = ufoir__projector_prepare(proj, in_dims);
    if (rc)
        return rc;
    out_dims[0] = proj->n_dets;
    out_dims[1] = proj->prm.is_forward ? proj->n_angles : proj->n_dets;
    return UFOIR_OK;
}

const float *ufoir_projector_get_host_sin_vals(const ufoir_projector *proj)
{
    return proj && proj->have_geometry ? proj->h_sin : NULL;
}

const float *ufoir_projector_get_host_cos_vals(const ufoir_projector *proj)
{
    return proj && proj->have_geometry ? proj->h_cos : NULL;
}

int ufoir_projector_get_subsets(const ufoir_projector *proj, const ufoir_subset **subsets,
                                unsigned int *count)
{
    if (!proj || !subsets || !count)
        return UFOIR_ERR_INVALID;
    if (!proj->have_geometry) {
        *subsets = NULL;
        *count = 0;
        return UFOIR_ERR_STATE;
    }
    *subsets = proj->subsets;
    *count = proj->n_subsets;
    return UFOIR_OK;
}

/* How far apart the rays of one detector at one row lie over the angles
 * [first, first + count) of one direction, maximised over the image: the
 * coordinate (…joseph.cl:68-75, 86) is linear in the detector and the row
 * for each angle, so the spread is largest at the corners of the square.
 * Evaluated in double; the kernel adds a margin for the float recurrence. */
static double tile_spread(const ufoir_projector *p, unsigned int first, unsigned int count, int dir, double axis)
{
    const double n = (double) p->n_dets;
    const double ros = (n - 2.0 * axis) / 2.0, os = n / 2.0;
    double spread = 0.0;
    for (int corner = 0; corner < 4; corner++) {
        const double s = (corner & 1) ? n - 1.0 : 0.0, y = (corner & 2) ? n - 1.0 : 0.0;
        double lo = 1e300, hi = -1e300;
        for (unsigned int a = first; a < first + count; a++) {
            const double sn = p->h_sin[a], cs = p->h_cos[a];
            const double det_step = dir == UFOIR_HORIZONTAL ? -1.0 / sn : 1.0 / cs;
            const double step = dir == UFOIR_HORIZONTAL ? cs / sn : sn / cs;
            const double c = (0.5 + ros + s - 0.5 * n) * det_step - os * step + 0.5 * n + y * step;
            lo = c < lo ? c : lo;
            hi = c > hi ? c : hi;
        }
        spread = hi - lo > spread ? hi - lo : spread;
    }
    return spread;
}

static int tile_slot(int A)
{
    return A == 1 ? 0 : A == 2 ? 1 : A == 4 ? 2 : A == 8 ? 3 : -1;
}

/* Angle tiles of the tiled forward projector: runs of at most A angles that
 * never cross a direction boundary (the full subsets, cut into pieces). */
int ufoir__projector_tiles(ufoir_projector *p, int A, const void **d_tiles, int *n_tiles, float *spread_out)
{
    ufoir_ctx *ctx = p->ctx;
    const int k = tile_slot(A);
    if (k < 0)
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "tile width %d", A);
    if (!p->tiles_valid[k]) {
        int count = 0;
        for (unsigned int i = 0; i < p->n_subsets; i++)
            count += (int) ((p->subsets[i].n + (unsigned int) A - 1) / (unsigned int) A);
        int *h = (int *) malloc(sizeof(int) * 4 * (size_t) (count ? count : 1));
        if (!h)
            return ufoir__fail(ctx, UFOIR_ERR_NOMEM, "out of host memory");
        int t = 0;
        udev_geom g;
        ufoir__projector_geom(p, &g);
        double spread = 0.0;
        for (unsigned int i = 0; i < p->n_subsets; i++)
            for (unsigned int a = 0; a < p->subsets[i].n; a += (unsigned int) A, t++) {
                const unsigned int left = p->subsets[i].n - a;
                h[4 * t + 0] = (int) (p->subsets[i].offset + a);
                h[4 * t + 1] = (int) (left < (unsigned int) A ? left : (unsigned int) A);
                h[4 * t + 2] = p->subsets[i].direction;
                h[4 * t + 3] = 0;
                const double sp = tile_spread(p, (unsigned int) h[4 * t + 0], (unsigned int) h[4 * t + 1],
                                              p->subsets[i].direction, (double) g.axis);
                spread = sp > spread ? sp : spread;
            }
        if (p->d_tiles[k])
            udev_free(ctx->dev, p->d_tiles[k]);
        p->d_tiles[k] = NULL;
        int rc = udev_malloc(ctx->dev, &p->d_tiles[k], sizeof(int) * 4 * (size_t) (count ? count : 1));
        if (!rc)
            rc = udev_memcpy(ctx->dev, p->d_tiles[k], h, sizeof(int) * 4 * (size_t) count);
        free(h);
        if (rc)
            return rc;
        p->n_tiles[k] = count;
        p->tiles_spread[k] = (float) spread;
        p->tiles_valid[k] = 1;
    }
    if (d_tiles)
        *d_tiles = p->d_tiles[k];
    if (n_tiles)
        *n_tiles = p->n_tiles[k];
    if (spread_out)
        *spread_out = p->tiles_spread[k];
    return UFOIR_OK;
}

int ufoir__fp_shape(ufoir_projector *p, int n_slices, udev_fp_cfg *c, const void **d_tiles, int *n_tiles)
{
    udev *d = p->ctx->dev;
    udev_geom g;
    ufoir__projector_geom(p, &g);
    /* a tuned shape serves only the slice count and arithmetic it was timed for */
    if (p->fp_cfg_valid && p->fp_cfg_slices == n_slices && p->fp_cfg.fm == (g.fast_arith ? 1 : 0)) {
        *c = p->fp_cfg;
        return ufoir__projector_tiles(p, c->A, d_tiles, n_tiles, NULL);
    }
    const int A = udev_fp_tile_angles(d, (int) p->n_dets);
    if (A <= 0)
        return UFOIR_ERR_UNSUPPORTED;
    float spread = 0.0f;
    int rc = ufoir__projector_tiles(p, A, d_tiles, n_tiles, &spread);
    if (rc)
        return rc;
    return udev_fp_default_cfg(d, &g, *n_tiles, n_slices, spread, c);
}

int ufoir__fp_scratch_alloc(ufoir_projector *p, ufoir_fp_scratch *s, size_t slices)
{
    const size_t n = p->n_dets, pitch = (size_t) udev_fp_pitch((int) n);
    s->P = s->TP = NULL;
    s->slices = slices;
    const size_t count = n * pitch * slices;
    int rc = ufoir__alloc(p->ctx, &s->P, count);
    if (!rc)
        rc = ufoir__alloc(p->ctx, &s->TP, count);
    if (!rc)
        rc = udev_memset(p->ctx->dev, s->P, 0, count * sizeof(float));
    if (!rc)
        rc = udev_memset(p->ctx->dev, s->TP, 0, count * sizeof(float));
    if (rc)
        ufoir__fp_scratch_free(p, s);
    return rc;
}

void ufoir__fp_scratch_free(ufoir_projector *p, ufoir_fp_scratch *s)
{
    ufoir__free(p->ctx, s->P);
    ufoir__free(p->ctx, s->TP);
    s->P = s->TP = NULL;
}

int ufoir__fp_prepare(ufoir_projector *p, ufoir_fp_scratch *s, const float *vol, int n_slices)
{
    if (udev_fp_tile_angles(p->ctx->dev, (int) p->n_dets) > 0)
        return udev_pad_transpose(p->ctx->dev, vol, s->P, s->TP, (int) p->n_dets, n_slices);
    /* the tiled kernel cannot serve this size: plain transpose for the row kernel */
    return udev_transpose(p->ctx->dev, vol, s->TP, (int) p->n_dets, n_slices);
}

int ufoir__fp_project(ufoir_projector *p, ufoir_fp_scratch *s, const float *vol, const float *src, const float *w,
                      int w_shared, float *out, float scale, int n_slices)
{
    udev_geom g;
    ufoir__projector_geom(p, &g);
    udev_fp_cfg c;
    const void *tiles = NULL;
    int n_tiles = 0;
    const int rc = ufoir__fp_shape(p, n_slices, &c, &tiles, &n_tiles);
    if (rc == UFOIR_OK)
        return udev_fp_tiles_cfg(p->ctx->dev, &g, &c, tiles, n_tiles, s->P, s->TP, src, w, w_shared, out, scale,
                                 n_slices);
    if (rc != UFOIR_ERR_UNSUPPORTED)
        return rc;
    return udev_fp(p->ctx->dev, &g, 0, (int) p->n_angles, -1, vol, s->TP, src, w, w_shared, out, scale, n_slices);
}

int ufoir__fp_full(ufoir_projector *p, ufoir_fp_scratch *s, const float *vol, const float *src, const float *w,
                   int w_shared, float *out, float scale, int n_slices)
{
    int rc = ufoir__fp_prepare(p, s, vol, n_slices);
    if (!rc)
        rc = ufoir__fp_project(p, s, vol, src, w, w_shared, out, scale, n_slices);
    return rc;
}

static int is_siddon(const ufoir_projector *p)
{
    return strcmp(p->prm.model, "siddon") == 0;
}

/* Forward projection of all angles of n_slices volumes (accumulating):
 * sino = sino + scale * A vol. */
/* Siddon forward projection of angles [a0, a0 + na): the padded copies
 * first (scratch s), then the ray walk. */
static int siddon_fp(ufoir_projector *p, ufoir_fp_scratch *s, int a0, int na, const float *dvol, float *dsino,
                     int n_slices)
{
    udev_geom g;
    ufoir__projector_geom(p, &g);
    int rc = udev_pad_transpose(p->ctx->dev, dvol, s->P, s->TP, (int) p->n_dets, n_slices);
    if (!rc)
        rc = udev_siddon_fp(p->ctx->dev, &g, a0, na, s->P, s->TP, dsino, NULL, 0, dsino, p->prm.correction_scale,
                            n_slices);
    return rc;
}

static int fp_all(ufoir_projector *p, const float *dvol, float *dsino, size_t n_slices)
{
    ufoir_fp_scratch s;
    int rc = ufoir__fp_scratch_alloc(p, &s, n_slices);
    if (rc)
        return rc;
    if (is_siddon(p))
        rc = siddon_fp(p, &s, 0, (int) p->n_angles, dvol, dsino, (int) n_slices);
    else
        rc = ufoir__fp_full(p, &s, dvol, dsino, NULL, 0, dsino, p->prm.correction_scale, (int) n_slices);
    ufoir__fp_scratch_free(p, &s);
    return rc;
}

static int bp_all(ufoir_projector *p, float *dvol, const float *dsino, size_t n_slices)
{
    udev_geom g;
    ufoir__projector_geom(p, &g);
    if (is_siddon(p))
        return udev_siddon_bp(p->ctx->dev, &g, p->subsets, (int) p->n_subsets, dsino, dvol, dvol,
                              p->prm.relaxation, (int) n_slices);
    return udev_bp(p->ctx->dev, &g, p->subsets, (int) p->n_subsets, dsino, dvol, NULL, 0, NULL, dvol,
                   p->prm.relaxation, (int) n_slices);
}

int ufoir_projector_forward(ufoir_projector *proj, const float *vol, float *sino, size_t n_dets,
                            size_t n_angles, size_t n_slices)
{
    if (!proj || !vol || !sino || n_slices == 0)
        return UFOIR_ERR_INVALID;
    ufoir_ctx *ctx = proj->ctx;
    int rc = ufoir__projector_prepare_na(proj, (unsigned int) n_dets, (unsigned int) n_angles);
    if (rc)
        return rc;
    ufoir_buf bv = {0}, bs = {0};
    const size_t nv = n_dets * n_dets, ns = n_dets * n_angles;
    UFOIR_TRY(ufoir__buf_in(ctx, &bv, vol, nv * n_slices, 1));
    UFOIR_TRY(ufoir__buf_in(ctx, &bs, sino, ns * n_slices, 1));
    UFOIR_TRY(fp_all(proj, bv.dev, bs.dev, n_slices));
    UFOIR_TRY(ufoir__buf_out(ctx, &bs, 1));
    UFOIR_TRY(udev_sync(ctx->dev));
done:
    ufoir__buf_release(ctx, &bv);
    ufoir__buf_release(ctx, &bs);
    return rc;
}

int ufoir_projector_backward(ufoir_projector *proj, float *vol, const float *sino, size_t n_dets,
                             size_t n_angles, size_t n_slices)
{
    if (!proj || !vol || !sino || n_slices == 0)
        return UFOIR_ERR_INVALID;
    ufoir_ctx *ctx = proj->ctx;
    int rc = ufoir__projector_prepare_na(proj, (unsigned int) n_dets, (unsigned int) n_angles);
    if (rc)
        return rc;
    ufoir_buf bv = {0}, bs = {0};
    const size_t nv = n_dets * n_dets, ns = n_dets * n_angles;
    UFOIR_TRY(ufoir__buf_in(ctx, &bv, vol, nv * n_slices, 1));
    UFOIR_TRY(ufoir__buf_in(ctx, &bs, sino, ns * n_slices, 1));
    UFOIR_TRY(bp_all(proj, bv.dev, bs.dev, n_slices));
    UFOIR_TRY(ufoir__buf_out(ctx, &bv, 1));
    UFOIR_TRY(udev_sync(ctx->dev));
done:
    ufoir__buf_release(ctx, &bv);
    ufoir__buf_release(ctx, &bs);
    return rc;
}

int ufoir_projector_process(ufoir_projector *proj, const float *in, const size_t in_dims[2], float *out,
                            size_t n_slices)
{
    if (!proj || !in || !out || !in_dims || n_slices == 0)
        return UFOIR_ERR_INVALID;
    ufoir_ctx *ctx = proj->ctx;
    size_t out_dims[2];
    int rc = ufoir_projector_get_requisition(proj, in_dims, out_dims);
    if (rc)
        return rc;
    const size_t n = proj->n_dets;
    const size_t nv = n * n, ns = n * proj->n_angles;
    ufoir_buf bi = {0}, bo = {0};
    if (proj->prm.is_forward) {
        /* input is a volume n x n (its dims[1] must match) */
        if (in_dims[1] != n)
            return ufoir__fail(ctx, UFOIR_ERR_INVALID, "forward input must be %zu x %zu", n, n);
        UFOIR_TRY(ufoir__buf_in(ctx, &bi, in, nv * n_slices, 1));
        UFOIR_TRY(ufoir__buf_in(ctx, &bo, out, ns * n_slices, 0));
        UFOIR_TRY(udev_fill(ctx->dev, bo.dev, ns * n_slices, 0.0f));
        UFOIR_TRY(fp_all(proj, bi.dev, bo.dev, n_slices));
    } else {
        if (in_dims[1] != proj->n_angles)
            return ufoir__fail(ctx, UFOIR_ERR_INVALID, "angles_num %u does not match the sinogram's %zu rows",
                               proj->n_angles, in_dims[1]);
        UFOIR_TRY(ufoir__buf_in(ctx, &bi, in, ns * n_slices, 1));
        UFOIR_TRY(ufoir__buf_in(ctx, &bo, out, nv * n_slices, 0));
        UFOIR_TRY(udev_fill(ctx->dev, bo.dev, nv * n_slices, 0.0f));
        UFOIR_TRY(bp_all(proj, bo.dev, bi.dev, n_slices));
    }
    UFOIR_TRY(ufoir__buf_out(ctx, &bo, 1));
    UFOIR_TRY(udev_sync(ctx->dev));
done:
    ufoir__buf_release(ctx, &bi);
    ufoir__buf_release(ctx, &bo);
    return rc;
}

int ufoir_projector_subset_fp(ufoir_projector *proj, const float *vol, float *sino, const ufoir_subset *s)
{
    if (!proj || !vol || !sino || !s)
        return UFOIR_ERR_INVALID;
    ufoir_ctx *ctx = proj->ctx;
    if (!proj->have_geometry)
        return ufoir__fail(ctx, UFOIR_ERR_STATE, "subset_fp before the geometry is known (no requisition yet)");
    if (s->offset + (size_t) s->n > proj->n_angles)
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "subset outside the %u angles", proj->n_angles);
    const size_t n = proj->n_dets, nv = n * n, ns = n * proj->n_angles;
    ufoir_buf bv = {0}, bs = {0};
    udev_geom g;
    ufoir__projector_geom(proj, &g);
    int rc;
    UFOIR_TRY(ufoir__buf_in(ctx, &bv, vol, nv, 1));
    UFOIR_TRY(ufoir__buf_in(ctx, &bs, sino, ns, 1));
    /* The subset's own direction picks the kernel (…parallel-projector-task.c:570). */
    if (is_siddon(proj)) {
        ufoir_fp_scratch fs;
        UFOIR_TRY(ufoir__fp_scratch_alloc(proj, &fs, 1));
        rc = siddon_fp(proj, &fs, (int) s->offset, (int) s->n, bv.dev, bs.dev, 1);
        ufoir__fp_scratch_free(proj, &fs);
        if (rc)
            goto done;
    } else
        UFOIR_TRY(udev_fp(ctx->dev, &g, (int) s->offset, (int) s->n, s->direction ? 1 : 0, bv.dev, NULL, bs.dev,
                          NULL, 0, bs.dev, proj->prm.correction_scale, 1));
    UFOIR_TRY(ufoir__buf_out(ctx, &bs, 1));
    UFOIR_TRY(udev_sync(ctx->dev));
done:
    ufoir__buf_release(ctx, &bv);
    ufoir__buf_release(ctx, &bs);
    return rc;
}

int ufoir_projector_subset_bp(ufoir_projector *proj, float *vol, const float *sino, const ufoir_subset *s)
{
    if (!proj || !vol || !sino || !s)
        return UFOIR_ERR_INVALID;
    ufoir_ctx *ctx = proj->ctx;
    if (!proj->have_geometry)
        return ufoir__fail(ctx, UFOIR_ERR_STATE, "subset_bp before the geometry is known (no requisition yet)");
    if (s->offset + (size_t) s->n > proj->n_angles)
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "subset outside the %u angles", proj->n_angles);
    const size_t n = proj->n_dets, nv = n * n, ns = n * proj->n_angles;
    ufoir_buf bv = {0}, bs = {0};
    udev_geom g;
    ufoir__projector_geom(proj, &g);
    int rc;
    UFOIR_TRY(ufoir__buf_in(ctx, &bv, vol, nv, 1));
    UFOIR_TRY(ufoir__buf_in(ctx, &bs, sino, ns, 1));
    if (is_siddon(proj))
        UFOIR_TRY(udev_siddon_bp(ctx->dev, &g, s, 1, bs.dev, bv.dev, bv.dev, proj->prm.relaxation, 1));
    else
        UFOIR_TRY(udev_bp(ctx->dev, &g, s, 1, bs.dev, bv.dev, NULL, 0, NULL, bv.dev, proj->prm.relaxation, 1));
    UFOIR_TRY(ufoir__buf_out(ctx, &bv, 1));
    UFOIR_TRY(udev_sync(ctx->dev));
done:
    ufoir__buf_release(ctx, &bv);
    ufoir__buf_release(ctx, &bs);
    return rc;
}
