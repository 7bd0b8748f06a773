/*
 * methods.c - SART, SIRT, ASD-POCS and split-Bregman TV on the GPU.
 *
 * Each method follows its reference host loop step for step (the same
 * buffers, the same operation order, the same float scalar arithmetic), with
 * runs of element-wise work fused into the projector kernels:
 *   SIRT iteration  = transpose(x) + FP[(b - Ax) * R] + BP[x + C * (lambda A^T r)]
 *   SART angle step = FP_theta[(b - A_theta x) * R_theta] + BP_theta[x + lambda A_theta^T r]
 * The weights R = inv(FP(1)) and C = inv(BP(1)) depend on the geometry only,
 * so they are computed once per call and shared by all slices.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "host.h"

/* Captured iterations per CUDA graph (bounds graph size for long runs). */
#define GRAPH_CHUNK 64

void ufoir_sart_params_init(ufoir_sart_params *p)
{
    if (!p)
        return;
    p->num_iterations = 10;        /* ufo-ir-method-task.c:111 */
    p->relaxation_factor = 0.25f;  /* ufo-ir-sart-task.c:93 */
}

void ufoir_sirt_params_init(ufoir_sirt_params *p)
{
    if (!p)
        return;
    p->num_iterations = 10;
    p->relaxation_factor = 0.25f;  /* ufo-ir-sirt-task.c:88 */
}

void ufoir_asdpocs_params_init(ufoir_asdpocs_params *p)
{
    if (!p)
        return;
    p->num_iterations = 10;
    p->beta = 1.0f;                /* ufo-ir-asdpocs-task.c:171-180 */
    p->beta_red = 0.995f;
    p->ng = 20;
    p->alpha = 0.2f;
    p->alpha_red = 0.95f;
    p->r_max = 0.95f;
    p->positive_constraint = 1;
    ufoir_sart_params_init(&p->df_minimizer);
    p->norm_mode = UFOIR_NORM_FP64;
}

void ufoir_sbtv_params_init(ufoir_sbtv_params *p)
{
    if (!p)
        return;
    p->num_iterations = 10;
    p->lambda = 0.1f;              /* ufo-ir-sbtv-task.c:114-115 */
    p->mu = 0.5f;
    p->norm_mode = UFOIR_NORM_FP64;
}

/* Shared validation + geometry for all methods. */
static int method_setup(ufoir_projector *proj, const size_t dims[2], size_t n_slices, unsigned int iters)
{
    ufoir_ctx *ctx = proj->ctx;
    if (n_slices == 0)
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "n_slices must be >= 1");
    if (iters < 1)
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "num-iterations must be >= 1");
    if (proj->prm.is_forward)
        return ufoir__fail(ctx, UFOIR_ERR_INVALID,
                           "a method's projector must have is_forward = false (the method's output is the "
                           "projector's backward requisition)");
    if (strcmp(proj->prm.model, "joseph") != 0)
        return ufoir__fail(ctx, UFOIR_ERR_UNSUPPORTED,
                           "the methods run the Joseph model only (projector model '%s')", proj->prm.model);
    int rc = ufoir__projector_prepare(proj, dims);
    if (rc)
        return rc;
    if (dims[1] != proj->n_angles)
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "angles_num %u does not match the sinogram's %zu rows",
                           proj->n_angles, dims[1]);
    return UFOIR_OK;
}

static int check_relax(ufoir_ctx *ctx, float r)
{
    if (!(r >= 0.0f && r <= 1.0f))
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "relaxation_factor %g outside [0, 1]", (double) r);
    return UFOIR_OK;
}

/* R = inv(FP(1)) over all angles for one slice (sirt-task.c:180-185,
 * sart-task.c:193-200). `ones` is scratch of n*n floats. */
int ufoir__ray_weights(ufoir_projector *p, float *R, float *ones)
{
    ufoir_ctx *ctx = p->ctx;
    const size_t n = p->n_dets, nv = n * n, ns = n * p->n_angles;
    ufoir_fp_scratch fs;
    int rc = ufoir__fp_scratch_alloc(p, &fs, 1);
    if (rc)
        return rc;
    rc = udev_fill(ctx->dev, ones, nv, 1.0f);
    if (!rc)
        rc = udev_fill(ctx->dev, R, ns, 0.0f);
    if (!rc)
        rc = ufoir__fp_full(p, &fs, ones, R, NULL, 0, R, 1.0f, 1);
    if (!rc)
        rc = udev_unary(ctx->dev, UDEV_INV, R, 0, 0, R, ns);
    ufoir__fp_scratch_free(p, &fs);
    return rc;
}

/* C = inv(BP(1)) for one slice (sirt-task.c:188-193). `ones` holds ns floats. */
int ufoir__pixel_weights(ufoir_projector *p, float *C, float *ones)
{
    ufoir_ctx *ctx = p->ctx;
    udev_geom g;
    ufoir__projector_geom(p, &g);
    const size_t n = p->n_dets, nv = n * n, ns = n * p->n_angles;
    int rc = udev_fill(ctx->dev, ones, ns, 1.0f);
    if (!rc)
        rc = udev_bp(ctx->dev, &g, p->subsets, (int) p->n_subsets, ones, NULL, NULL, 0, NULL, C, 1.0f, 1);
    if (!rc)
        rc = udev_unary(ctx->dev, UDEV_INV, C, 0, 0, C, nv);
    return rc;
}

/* Runs `iters` repetitions of a captured body, GRAPH_CHUNK per graph. */
typedef int (*body_fn)(void *arg);

static int run_graphed(ufoir_ctx *ctx, unsigned int iters, body_fn body, void *arg)
{
    int rc = UFOIR_OK;
    unsigned int remaining = iters;
    void *exec = NULL;
    unsigned int exec_len = 0;
    uint64_t exec_kernels = 0;
    while (remaining > 0) {
        const unsigned int len = remaining >= GRAPH_CHUNK ? GRAPH_CHUNK : remaining;
        if (!exec || exec_len != len) {
            udev_graph_destroy(exec);
            exec = NULL;
            rc = udev_capture_begin(ctx->dev);
            if (rc)
                return rc;
            for (unsigned int i = 0; i < len && rc == UFOIR_OK; i++)
                rc = body(arg);
            void *e = NULL;
            const int rc2 = udev_capture_end(ctx->dev, &e, &exec_kernels);
            if (rc || rc2) {
                udev_graph_destroy(e);
                return rc ? rc : rc2;
            }
            exec = e;
            exec_len = len;
        }
        rc = udev_graph_launch(ctx->dev, exec, exec_kernels);
        if (rc)
            break;
        remaining -= len;
    }
    if (rc == UFOIR_OK)
        rc = udev_sync(ctx->dev);
    udev_graph_destroy(exec);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* SIRT                                                                     */
/* ------------------------------------------------------------------------ */
int ufoir__sirt_body(void *arg)
{
    ufoir__sirt_iter *s = (ufoir__sirt_iter *) arg;
    udev *d = s->p->ctx->dev;
    /* sirt-task.c:202-213: r = (b - A x) * R;  x = x + C * (lambda A^T r) */
    int rc = ufoir__fp_full(s->p, &s->fs, s->x, s->b, s->R, 1, s->resid, -1.0f, s->n_slices);
    if (!rc)
        rc = udev_bp(d, &s->g, s->p->subsets, (int) s->p->n_subsets, s->resid, NULL, s->C, 1, s->x, s->x,
                     s->lambda, s->n_slices);
    return rc;
}

/* Slice chunks of a SIRT call whose data cross the host boundary. */
#define SIRT_HOST_CHUNKS 4

static int sirt_chunks(int S)
{
    return S < SIRT_HOST_CHUNKS ? S : SIRT_HOST_CHUNKS;
}

/* First slice of chunk k of S slices in `chunks` chunks (the same split
 * everywhere: sizes differ by at most one). */
static int sirt_chunk_start(int S, int chunks, int k)
{
    return (int) (((long long) S * k) / chunks);
}

/* One SIRT iteration (the work of ufoir__sirt_body) split by slice chunks
 * where it meets host data: with chunked_in, the forward projection of chunk
 * k waits only for side-stream mark k (the arrival of that chunk's
 * sinograms); with host_vol, the backprojection runs per chunk and each
 * chunk's final volumes are copied to host_vol on the side stream while the
 * next chunks compute. Per slice the kernels do the same work, so the values
 * are those of the unsplit iteration. */
static int sirt_iteration_split(ufoir__sirt_iter *s, int chunked_in, float *host_vol)
{
    udev *d = s->p->ctx->dev;
    const size_t n = s->p->n_dets, nv = n * n, ns = n * s->p->n_angles;
    const int S = s->n_slices, chunks = sirt_chunks(S);
    int rc = UFOIR_OK;
    if (chunked_in) {
        for (int k = 0; k < chunks && rc == UFOIR_OK; k++) {
            const int s0 = sirt_chunk_start(S, chunks, k), c = sirt_chunk_start(S, chunks, k + 1) - s0;
            rc = udev_side_wait(d, k);
            if (!rc)
                rc = ufoir__fp_full(s->p, &s->fs, s->x + (size_t) s0 * nv, s->b + (size_t) s0 * ns, s->R, 1,
                                    s->resid + (size_t) s0 * ns, -1.0f, c);
        }
    } else {
        rc = ufoir__fp_full(s->p, &s->fs, s->x, s->b, s->R, 1, s->resid, -1.0f, S);
    }
    if (rc)
        return rc;
    if (!host_vol)
        return udev_bp(d, &s->g, s->p->subsets, (int) s->p->n_subsets, s->resid, NULL, s->C, 1, s->x, s->x,
                       s->lambda, S);
    for (int k = 0; k < chunks && rc == UFOIR_OK; k++) {
        const int s0 = sirt_chunk_start(S, chunks, k), c = sirt_chunk_start(S, chunks, k + 1) - s0;
        float *xk = s->x + (size_t) s0 * nv;
        rc = udev_bp(d, &s->g, s->p->subsets, (int) s->p->n_subsets, s->resid + (size_t) s0 * ns, NULL, s->C, 1,
                     xk, xk, s->lambda, c);
        if (!rc)
            rc = udev_copy_after(d, host_vol + (size_t) s0 * nv, xk, (size_t) c * nv * sizeof(float));
    }
    return rc;
}

int ufoir_sirt_process(ufoir_projector *proj, const ufoir_sirt_params *prm, const float *sino,
                       const size_t dims[2], float *vol, size_t n_slices)
{
    if (!proj || !prm || !sino || !vol || !dims)
        return UFOIR_ERR_INVALID;
    ufoir_ctx *ctx = proj->ctx;
    int rc = check_relax(ctx, prm->relaxation_factor);
    if (rc)
        return rc;
    rc = method_setup(proj, dims, n_slices, prm->num_iterations);
    if (rc)
        return rc;
    const size_t n = proj->n_dets, nv = n * n, ns = n * proj->n_angles;
    ufoir_buf bb = {0}, bx = {0};
    float *R = NULL, *C = NULL, *resid = NULL;
    ufoir__sirt_iter it;
    memset(&it, 0, sizeof(it));
    UFOIR_TRY(ufoir__buf_in(ctx, &bb, sino, ns * n_slices, 0));
    UFOIR_TRY(ufoir__buf_in(ctx, &bx, vol, nv * n_slices, 0));
    UFOIR_TRY(ufoir__alloc(ctx, &R, ns));
    UFOIR_TRY(ufoir__alloc(ctx, &C, nv));
    UFOIR_TRY(ufoir__alloc(ctx, &resid, ns * n_slices));
    UFOIR_TRY(ufoir__fp_scratch_alloc(proj, &it.fs, n_slices));
    /* host sinograms move in on the side stream, chunk by chunk, while the
     * weights are computed (they do not read b) and the first forward
     * projection starts on the chunks that have arrived */
    const int host_in = bb.owned, host_out = bx.owned;
    if (host_in) {
        const int chunks = sirt_chunks((int) n_slices);
        UFOIR_TRY(udev_side_fence(ctx->dev));
        for (int k = 0; k < chunks; k++) {
            const size_t s0 = (size_t) sirt_chunk_start((int) n_slices, chunks, k);
            const size_t s1 = (size_t) sirt_chunk_start((int) n_slices, chunks, k + 1);
            UFOIR_TRY(udev_side_copy(ctx->dev, bb.dev + s0 * ns, sino + s0 * ns, (s1 - s0) * ns * sizeof(float), k));
        }
    }

    /* weights with relaxation 1 and correction scale 1 (sirt-task.c:176-193);
     * the output volume serves as the all-ones image before it is zeroed */
    proj->prm.relaxation = 1.0f;
    proj->prm.correction_scale = 1.0f;
    UFOIR_TRY(ufoir__ray_weights(proj, R, bx.dev));
    UFOIR_TRY(ufoir__pixel_weights(proj, C, resid));
    proj->prm.relaxation = prm->relaxation_factor;
    proj->prm.correction_scale = -1.0f;
    UFOIR_TRY(udev_fill(ctx->dev, bx.dev, nv * n_slices, 0.0f));
    if (ufoir__fp_tune_wanted(proj, (int) n_slices))
        UFOIR_TRY(ufoir__fp_tune(proj, (int) n_slices, NULL));

    it.p = proj;
    ufoir__projector_geom(proj, &it.g);
    it.b = bb.dev;
    it.x = bx.dev;
    it.resid = resid;
    it.R = R;
    it.C = C;
    it.lambda = prm->relaxation_factor;
    it.n_slices = (int) n_slices;
    if ((host_in || host_out) && prm->num_iterations > 0) {
        /* the first and last iterations run eagerly, split where they meet
         * host data (sirt_iteration_split), the others as graphs; a kernel
         * error found afterwards still fails the call */
        const unsigned int iters = prm->num_iterations;
        UFOIR_TRY(sirt_iteration_split(&it, host_in, iters == 1 && host_out ? vol : NULL));
        if (iters > 1) {
            UFOIR_TRY(run_graphed(ctx, iters - 2, ufoir__sirt_body, &it));
            UFOIR_TRY(sirt_iteration_split(&it, 0, host_out ? vol : NULL));
        }
        UFOIR_TRY(udev_copy_join(ctx->dev));
        UFOIR_TRY(udev_take_kernel_error(ctx->dev));
        UFOIR_TRY(ufoir__buf_out(ctx, &bx, 0));
    } else {
        UFOIR_TRY(run_graphed(ctx, prm->num_iterations, ufoir__sirt_body, &it));
        UFOIR_TRY(udev_take_kernel_error(ctx->dev));
        UFOIR_TRY(ufoir__buf_out(ctx, &bx, 1));
    }
done:
    udev_copy_join(ctx->dev);     /* side copies finish before their buffers are freed */
    ufoir__free(ctx, R);
    ufoir__free(ctx, C);
    ufoir__fp_scratch_free(proj, &it.fs);
    ufoir__free(ctx, resid);
    ufoir__buf_release(ctx, &bb);
    ufoir__buf_release(ctx, &bx);
    if (rc == UFOIR_OK)
        rc = udev_sync(ctx->dev);
    else
        udev_sync(ctx->dev);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Resident batched SIRT                                                    */
/* ------------------------------------------------------------------------ */
struct ufoir_sirt_batch {
    ufoir_projector *proj;
    ufoir__sirt_iter it;
    float *R, *C, *resid;
    size_t nv;
    void *exec;
    uint64_t exec_kernels;
};

void ufoir_sirt_batch_destroy(ufoir_sirt_batch *b)
{
    if (!b)
        return;
    ufoir_ctx *ctx = b->proj->ctx;
    udev_sync(ctx->dev);
    udev_graph_destroy(b->exec);
    ufoir__free(ctx, b->R);
    ufoir__free(ctx, b->C);
    ufoir__free(ctx, b->resid);
    ufoir__fp_scratch_free(b->proj, &b->it.fs);
    udev_sync(ctx->dev);
    free(b);
}

int ufoir_sirt_batch_create(ufoir_projector *proj, const ufoir_sirt_params *prm, const float *d_sino,
                            const size_t dims[2], float *d_vol, size_t n_slices, ufoir_sirt_batch **out)
{
    if (!proj || !prm || !d_sino || !d_vol || !dims || !out)
        return UFOIR_ERR_INVALID;
    *out = NULL;
    ufoir_ctx *ctx = proj->ctx;
    int rc = check_relax(ctx, prm->relaxation_factor);
    if (rc)
        return rc;
    rc = method_setup(proj, dims, n_slices, 1);
    if (rc)
        return rc;
    if (!udev_is_device_ptr(ctx->dev, d_sino) || !udev_is_device_ptr(ctx->dev, d_vol))
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "sirt batch: sinograms and volumes must be device memory");
    const size_t n = proj->n_dets, nv = n * n, ns = n * proj->n_angles;
    ufoir_sirt_batch *b = (ufoir_sirt_batch *) calloc(1, sizeof(*b));
    if (!b)
        return ufoir__fail(ctx, UFOIR_ERR_NOMEM, "out of host memory");
    b->proj = proj;
    b->nv = nv;
    UFOIR_TRY(ufoir__alloc(ctx, &b->R, ns));
    UFOIR_TRY(ufoir__alloc(ctx, &b->C, nv));
    UFOIR_TRY(ufoir__alloc(ctx, &b->resid, ns * n_slices));
    UFOIR_TRY(ufoir__fp_scratch_alloc(proj, &b->it.fs, n_slices));
    proj->prm.relaxation = 1.0f;
    proj->prm.correction_scale = 1.0f;
    UFOIR_TRY(ufoir__ray_weights(proj, b->R, d_vol));
    UFOIR_TRY(ufoir__pixel_weights(proj, b->C, b->resid));
    proj->prm.relaxation = prm->relaxation_factor;
    proj->prm.correction_scale = -1.0f;
    UFOIR_TRY(udev_fill(ctx->dev, d_vol, nv * n_slices, 0.0f));
    if (ufoir__fp_tune_wanted(proj, (int) n_slices))
        UFOIR_TRY(ufoir__fp_tune(proj, (int) n_slices, NULL));
    b->it.p = proj;
    ufoir__projector_geom(proj, &b->it.g);
    b->it.b = d_sino;
    b->it.x = d_vol;
    b->it.resid = b->resid;
    b->it.R = b->R;
    b->it.C = b->C;
    b->it.lambda = prm->relaxation_factor;
    b->it.n_slices = (int) n_slices;
    UFOIR_TRY(udev_capture_begin(ctx->dev));
    rc = ufoir__sirt_body(&b->it);
    {
        const int rc2 = udev_capture_end(ctx->dev, &b->exec, &b->exec_kernels);
        if (!rc)
            rc = rc2;
    }
    if (rc)
        goto done;
    UFOIR_TRY(udev_sync(ctx->dev));
    *out = b;
    return UFOIR_OK;
done:
    ufoir_sirt_batch_destroy(b);
    return rc;
}

int ufoir_sirt_batch_run(ufoir_sirt_batch *b, unsigned int iterations)
{
    if (!b)
        return UFOIR_ERR_INVALID;
    udev *d = b->proj->ctx->dev;
    for (unsigned int i = 0; i < iterations; i++) {
        int rc = udev_graph_launch(d, b->exec, b->exec_kernels);
        if (rc)
            return rc;
    }
    return udev_take_kernel_error(d);
}

int ufoir_sirt_batch_reset(ufoir_sirt_batch *b)
{
    if (!b)
        return UFOIR_ERR_INVALID;
    udev *d = b->proj->ctx->dev;
    int rc = udev_fill(d, b->it.x, b->nv * (size_t) b->it.n_slices, 0.0f);
    return rc ? rc : udev_sync(d);
}

int ufoir_sirt_batch_profile(ufoir_sirt_batch *b, float ms[3])
{
    if (!b || !ms)
        return UFOIR_ERR_INVALID;
    ufoir__sirt_iter *s = &b->it;
    udev *d = s->p->ctx->dev;
    int rc;
    if ((rc = udev_timer_begin(d)) || (rc = ufoir__fp_prepare(s->p, &s->fs, s->x, s->n_slices)) ||
        (rc = udev_timer_end(d, &ms[0])))
        return rc;
    if ((rc = udev_timer_begin(d)) ||
        (rc = ufoir__fp_project(s->p, &s->fs, s->x, s->b, s->R, 1, s->resid, -1.0f, s->n_slices)) ||
        (rc = udev_timer_end(d, &ms[1])))
        return rc;
    if ((rc = udev_timer_begin(d)) ||
        (rc = udev_bp(d, &s->g, s->p->subsets, (int) s->p->n_subsets, s->resid, NULL, s->C, 1, s->x, s->x,
                      s->lambda, s->n_slices)) ||
        (rc = udev_timer_end(d, &ms[2])))
        return rc;
    return udev_take_kernel_error(d);
}

/* ------------------------------------------------------------------------ */
/* SART                                                                     */
/* ------------------------------------------------------------------------ */
int ufoir__sart_body(void *arg)
{
    ufoir__sart_iter *s = (ufoir__sart_iter *) arg;
    udev *d = s->p->ctx->dev;
    const int n = s->g.n_dets, S = s->n_slices;
    int rc = UFOIR_OK;
    /* sart-task.c:209-217: per angle, r_theta = (b_theta - A_theta x) * R_theta;
     * x = x + lambda A_theta^T r_theta. The volume lives in the layout of the
     * current direction run, transposed while the angles are horizontal, so
     * that every ray walks rows.
     * The padded kernels where they serve the geometry, else the general
     * ones; UFOIR_SART_KERNELS=general selects the general kernels always. */
    const char *only = getenv("UFOIR_SART_KERNELS");
    const int general_only = only && strcmp(only, "general") == 0;
    if (!general_only && udev_sart_padded(d, &s->g, S)) {
        /* padded copies V (vertical run) and H (horizontal run) in s->work */
        int place = -1;
        for (unsigned int a = 0; a < s->p->n_angles && rc == UFOIR_OK; a++) {
            const int dir = s->p->h_dir[a];
            const int want = dir == UFOIR_HORIZONTAL;
            if (want != place) {
                rc = udev_sart_move(d, n, s->x, s->work, place, want, S);
                place = want;
            }
            if (!rc)
                rc = udev_sart_fp(d, &s->g, (int) a, dir, s->table, s->work, place, s->b, s->R, 1, s->resid, -1.0f,
                                  S);
            if (!rc)
                rc = udev_sart_bp(d, &s->g, (int) a, s->p->h_sin[a], s->p->h_cos[a], s->resid, s->work, place,
                                  s->lambda, s->relax_dev, S);
        }
        if (!rc && place >= 0)
            rc = udev_sart_move(d, n, s->x, s->work, place, -1, S);
        return rc;
    }
    /* crossed clamp edges (axis within half a pixel of the image edge): the
     * general kernels on the unpadded volume and its transpose in s->work */
    int transposed = 0;
    for (unsigned int a = 0; a < s->p->n_angles && rc == UFOIR_OK; a++) {
        const int dir = s->p->h_dir[a];
        const int want = dir == UFOIR_HORIZONTAL;
        if (want != transposed) {
            rc = udev_transpose(d, transposed ? s->work : s->x, transposed ? s->x : s->work, n, S);
            transposed = want;
        }
        float *vol = transposed ? s->work : s->x;
        if (!rc)
            rc = udev_fp_angle(d, &s->g, (int) a, dir, s->table, vol, s->b, s->R, 1, s->resid, -1.0f, S);
        if (!rc)
            rc = udev_bp_angle(d, &s->g, (int) a, s->p->h_sin[a], s->p->h_cos[a], s->resid, vol, transposed,
                               s->lambda, s->relax_dev, S);
    }
    if (!rc && transposed)
        rc = udev_transpose(d, s->work, s->x, n, S);
    return rc;
}

size_t ufoir__sart_scratch_bytes(size_t n, size_t na, size_t n_slices)
{
    return sizeof(float) * (udev_sart_work_floats((int) n, (int) n_slices) + udev_fp_block_starts_floats((int) n, (int) na));
}

int ufoir__sart_scratch_alloc(ufoir_projector *p, float **work, float **table, int n_slices)
{
    ufoir_ctx *ctx = p->ctx;
    const size_t n = p->n_dets;
    const size_t wf = udev_sart_work_floats((int) n, n_slices);
    udev_geom g;
    ufoir__projector_geom(p, &g);
    int rc = ufoir__alloc(ctx, work, wf);
    if (!rc)
        rc = udev_memset(ctx->dev, *work, 0, sizeof(float) * wf);   /* the pads stay zero */
    if (!rc)
        rc = ufoir__alloc(ctx, table, udev_fp_block_starts_floats((int) n, (int) p->n_angles));
    if (!rc)
        rc = udev_fp_block_starts(ctx->dev, &g, *table);
    return rc;
}

/* One SART call on resident buffers: x = SART(b), R precomputed. */
static int sart_run(ufoir_projector *proj, unsigned int iters, float lambda, const float *b, float *x,
                    float *resid, const float *R, float *work, float *table, int n_slices)
{
    ufoir_ctx *ctx = proj->ctx;
    const size_t n = proj->n_dets, nv = n * n;
    proj->prm.correction_scale = -1.0f;
    proj->prm.relaxation = lambda;
    int rc = udev_fill(ctx->dev, x, nv * (size_t) n_slices, 0.0f);
    if (rc)
        return rc;
    ufoir__sart_iter it;
    it.p = proj;
    ufoir__projector_geom(proj, &it.g);
    it.b = b;
    it.x = x;
    it.resid = resid;
    it.R = R;
    it.lambda = lambda;
    it.n_slices = n_slices;
    it.work = work;
    it.table = table;
    it.relax_dev = NULL;
    /* one angle sweep per graph: a sweep is already 2 * n_angles kernels */
    int rc2 = UFOIR_OK;
    void *exec = NULL;
    uint64_t kernels = 0;
    rc = udev_capture_begin(ctx->dev);
    if (rc)
        return rc;
    rc = ufoir__sart_body(&it);
    rc2 = udev_capture_end(ctx->dev, &exec, &kernels);
    if (rc || rc2) {
        udev_graph_destroy(exec);
        return rc ? rc : rc2;
    }
    for (unsigned int i = 0; i < iters && rc == UFOIR_OK; i++)
        rc = udev_graph_launch(ctx->dev, exec, kernels);
    if (rc == UFOIR_OK)
        rc = udev_take_kernel_error(ctx->dev);   /* waits for the stream */
    udev_graph_destroy(exec);
    return rc;
}

int ufoir_sart_process(ufoir_projector *proj, const ufoir_sart_params *prm, const float *sino,
                       const size_t dims[2], float *vol, size_t n_slices)
{
    if (!proj || !prm || !sino || !vol || !dims)
        return UFOIR_ERR_INVALID;
    ufoir_ctx *ctx = proj->ctx;
    int rc = check_relax(ctx, prm->relaxation_factor);
    if (rc)
        return rc;
    rc = method_setup(proj, dims, n_slices, prm->num_iterations);
    if (rc)
        return rc;
    const size_t n = proj->n_dets, nv = n * n, ns = n * proj->n_angles;
    ufoir_buf bb = {0}, bx = {0};
    float *R = NULL, *resid = NULL, *work = NULL, *table = NULL;
    UFOIR_TRY(ufoir__buf_in(ctx, &bb, sino, ns * n_slices, 1));
    UFOIR_TRY(ufoir__buf_in(ctx, &bx, vol, nv * n_slices, 0));
    UFOIR_TRY(ufoir__alloc(ctx, &R, ns));
    UFOIR_TRY(ufoir__alloc(ctx, &resid, ns * n_slices > nv ? ns * n_slices : nv));
    UFOIR_TRY(ufoir__sart_scratch_alloc(proj, &work, &table, (int) n_slices));
    proj->prm.correction_scale = 1.0f;
    UFOIR_TRY(ufoir__ray_weights(proj, R, resid));
    UFOIR_TRY(sart_run(proj, prm->num_iterations, prm->relaxation_factor, bb.dev, bx.dev, resid, R, work, table,
                       (int) n_slices));
    UFOIR_TRY(ufoir__buf_out(ctx, &bx, 1));
done:
    ufoir__free(ctx, R);
    ufoir__free(ctx, resid);
    ufoir__free(ctx, work);
    ufoir__free(ctx, table);
    ufoir__buf_release(ctx, &bb);
    ufoir__buf_release(ctx, &bx);
    udev_sync(ctx->dev);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* ASD-POCS                                                                 */
/* ------------------------------------------------------------------------ */
static int asdpocs_check(ufoir_ctx *ctx, const ufoir_asdpocs_params *prm)
{
    int rc;
    if (prm->df_minimizer.num_iterations < 1)
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "df_minimizer num-iterations must be >= 1");
    if ((rc = check_relax(ctx, prm->df_minimizer.relaxation_factor)))
        return rc;
    if (!(prm->beta >= 0 && prm->beta_red >= 0 && prm->alpha >= 0 && prm->alpha_red >= 0 && prm->r_max >= 0))
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "beta, beta_red, alpha, alpha_red, r_max must be >= 0");
    if (prm->ng > 1000)
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "ng %u outside [0, 1000]", prm->ng);
    if (prm->norm_mode != UFOIR_NORM_COMPAT && prm->norm_mode != UFOIR_NORM_FP64)
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "unknown norm_mode %d", prm->norm_mode);
    if (prm->num_iterations < 1)
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "num-iterations must be >= 1");
    return UFOIR_OK;
}

void ufoir__asd_release(ufoir__asd_state *s)
{
    ufoir_ctx *ctx = s->p->ctx;
    udev_graph_destroy(s->sart_exec);
    udev_graph_destroy(s->post_exec);
    s->sart_exec = s->post_exec = NULL;
    ufoir__free(ctx, s->x);
    ufoir__free(ctx, s->x_prev);
    ufoir__free(ctx, s->x_res);
    ufoir__free(ctx, s->b_res);
    ufoir__free(ctx, s->grad);
    ufoir__free(ctx, s->R);
    ufoir__free(ctx, s->work);
    ufoir__free(ctx, s->table);
    ufoir__free(ctx, s->scal);
    ufoir__free(ctx, s->partials);
    ufoir__fp_scratch_free(s->p, &s->fs);
    s->x = s->x_prev = s->x_res = s->b_res = s->grad = s->R = s->work = s->table = s->scal = NULL;
    s->partials = NULL;
}

/* Floats of the device scalar block: beta, relax, it (as int bits), then
 * dp, dd, dg, dtgv, l1 per slice. */
static size_t asd_scalar_floats(size_t S)
{
    return 3 + 5 * S;
}

size_t ufoir__asd_bytes(size_t n, size_t na, size_t S)
{
    const size_t nv = n * n, ns = n * na, pitch = (size_t) udev_fp_pitch((int) n);
    const size_t bres = ns * S > nv ? ns * S : nv;
    return sizeof(float) * (4 * nv * S + bres + ns + 2 * n * pitch * S + asd_scalar_floats(S)) +
           sizeof(double) * udev_l1_partials((int) S) + ufoir__sart_scratch_bytes(n, na, S);
}

/* The part of an outer iteration after the SART sweeps (asdpocs-task.c:461-506),
 * for capture: every scalar stays on the device. */
static int asd_post_body(void *arg)
{
    ufoir__asd_state *s = (ufoir__asd_state *) arg;
    ufoir_projector *proj = s->p;
    udev *d = proj->ctx->dev;
    const size_t n = s->n, na = s->na, nv = s->nv;
    const int S = s->S;
    const ufoir_asdpocs_params *prm = &s->prm;
    const udev_asd_scalars *c = &s->dsc;
    int rc;
    if (prm->positive_constraint && (rc = udev_unary(d, UDEV_POSC, s->x, 0, 0, s->x, nv * S)))
        return rc;
    if ((rc = udev_memcpy_async(d, s->out, s->x, nv * S * sizeof(float))))
        return rc;
    /* b_res = b - A x (:470-475) */
    if ((rc = ufoir__fp_full(proj, &s->fs, s->x, s->b, NULL, 0, s->b_res, -1.0f, S)) ||
        (rc = udev_l1_norm_to(d, s->b_res, n, na, S, prm->norm_mode, s->partials, c->dd)) ||
        (rc = udev_binary(d, UDEV_SUB, s->x, s->x_prev, 0, s->x_res, nv * S)) ||
        (rc = udev_l1_norm_to(d, s->x_res, n, n, S, prm->norm_mode, s->partials, c->dp)) ||
        (rc = udev_asd_init(d, c, prm->alpha, S)) ||
        (rc = udev_memcpy_async(d, s->x_prev, s->x, nv * S * sizeof(float))))
        return rc;
    /* ufo_math_tvstd_method_process_real (:550-580): 20 sub-steps */
    for (int step = 0; step < 20; step++) {
        if ((rc = udev_l1_grad(d, s->x, s->grad, (int) n, (int) n, S)) ||
            (rc = udev_l1_norm_to(d, s->grad, n, n, S, prm->norm_mode, s->partials, c->l1)) ||
            (rc = udev_asd_tv_step(d, s->x, s->grad, c, nv, S)))
            return rc;
    }
    if ((rc = udev_binary(d, UDEV_SUB, s->x, s->x_prev, 0, s->x_res, nv * S)) ||
        (rc = udev_l1_norm_to(d, s->x_res, n, n, S, prm->norm_mode, s->partials, c->dg)))
        return rc;
    return udev_asd_end(d, c, prm->beta_red, prm->r_max, prm->alpha_red, S);
}

static int capture(udev *d, int (*body)(void *), void *arg, void **exec, uint64_t *kernels)
{
    int rc = udev_capture_begin(d);
    if (rc)
        return rc;
    rc = body(arg);
    const int rc2 = udev_capture_end(d, exec, kernels);
    if (rc || rc2) {
        udev_graph_destroy(*exec);
        *exec = NULL;
        return rc ? rc : rc2;
    }
    return UFOIR_OK;
}

/* Buffers, weights, device scalars and the two graphs of an outer iteration
 * (asdpocs-task.c:411-455). The geometry must be prepared; b and out are
 * device memory (S slices). */
int ufoir__asd_setup(ufoir__asd_state *s, ufoir_projector *proj, const ufoir_asdpocs_params *prm, const float *b,
                     float *out, int S)
{
    ufoir_ctx *ctx = proj->ctx;
    memset(s, 0, sizeof(*s));
    s->p = proj;
    s->prm = *prm;
    s->S = S;
    s->n = proj->n_dets;
    s->na = proj->n_angles;
    s->nv = s->n * s->n;
    s->ns = s->n * s->na;
    s->b = b;
    s->out = out;
    ufoir__projector_geom(proj, &s->g);
    const size_t nv = s->nv, ns = s->ns;
    float *h = NULL;
    int rc;
    if (S > 1024)
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "ASD-POCS: %d slices in one call (at most 1024)", S);
    UFOIR_TRY(ufoir__alloc(ctx, &s->x, nv * S));
    UFOIR_TRY(ufoir__alloc(ctx, &s->x_prev, nv * S));
    UFOIR_TRY(ufoir__alloc(ctx, &s->x_res, nv * S));
    UFOIR_TRY(ufoir__alloc(ctx, &s->b_res, ns * S > nv ? ns * S : nv));
    UFOIR_TRY(ufoir__alloc(ctx, &s->grad, nv * S));
    UFOIR_TRY(ufoir__alloc(ctx, &s->R, ns));
    UFOIR_TRY(ufoir__alloc(ctx, &s->scal, asd_scalar_floats((size_t) S)));
    UFOIR_TRY(udev_malloc(ctx->dev, (void **) &s->partials, sizeof(double) * (udev_l1_partials(S) + 1)));
    UFOIR_TRY(ufoir__sart_scratch_alloc(proj, &s->work, &s->table, S));
    UFOIR_TRY(ufoir__fp_scratch_alloc(proj, &s->fs, (size_t) S));
    s->dsc.beta = s->scal;
    s->dsc.relax = s->scal + 1;
    s->dsc.it = (int *) (s->scal + 2);
    s->dsc.dp = s->scal + 3;
    s->dsc.dd = s->dsc.dp + S;
    s->dsc.dg = s->dsc.dd + S;
    s->dsc.dtgv = s->dsc.dg + S;
    s->dsc.l1 = s->dsc.dtgv + S;
    /* initial values (:418-455): beta, the minimizer's relaxation, it = 0,
     * and the norms and TV step at 1 */
    h = (float *) malloc(sizeof(float) * asd_scalar_floats((size_t) S));
    if (!h) {
        rc = ufoir__fail(ctx, UFOIR_ERR_NOMEM, "out of host memory");
        goto done;
    }
    h[0] = prm->beta;
    h[1] = prm->df_minimizer.relaxation_factor;
    memset(&h[2], 0, sizeof(float));
    for (size_t i = 3; i < asd_scalar_floats((size_t) S); i++)
        h[i] = 1.0f;
    UFOIR_TRY(udev_memcpy_async(ctx->dev, s->scal, h, sizeof(float) * asd_scalar_floats((size_t) S)));
    UFOIR_TRY(udev_fill(ctx->dev, s->x, nv * S, 0.0f));
    UFOIR_TRY(udev_fill(ctx->dev, s->x_prev, nv * S, 0.0f));
    /* SART's ray weights depend on the geometry only; the reference
     * recomputes the same values on every df_minimizer call. */
    proj->prm.correction_scale = 1.0f;
    UFOIR_TRY(ufoir__ray_weights(proj, s->R, s->b_res));
    UFOIR_TRY(udev_sync(ctx->dev));     /* h is read by the copy above */
    free(h);
    h = NULL;
    /* one SART sweep, relaxation read from the device scalar */
    s->sweep.p = proj;
    s->sweep.g = s->g;
    s->sweep.b = b;
    s->sweep.x = s->x;
    s->sweep.resid = s->b_res;
    s->sweep.R = s->R;
    s->sweep.lambda = 0.0f;
    s->sweep.relax_dev = s->dsc.relax;
    s->sweep.n_slices = S;
    s->sweep.work = s->work;
    s->sweep.table = s->table;
    UFOIR_TRY(capture(ctx->dev, ufoir__sart_body, &s->sweep, &s->sart_exec, &s->sart_kernels));
    UFOIR_TRY(capture(ctx->dev, asd_post_body, s, &s->post_exec, &s->post_kernels));
    s->beta = prm->beta;
    s->sart_relax = prm->df_minimizer.relaxation_factor;
    s->it = 0;
    return UFOIR_OK;
done:
    free(h);
    ufoir__asd_release(s);
    return rc;
}

/* One outer iteration of asdpocs-task.c:457-506, enqueued without any host
 * synchronisation: the relaxation update, SART from x = 0 (sart-task.c:207),
 * the SART sweeps, then the post-SART graph. */
int ufoir__asd_outer(ufoir__asd_state *s)
{
    ufoir_projector *proj = s->p;
    udev *d = proj->ctx->dev;
    int rc;
    /* g_object_set(df_minimizer, "relaxation_factor", beta) (:459); the
     * property's range is [0, 1] and GObject rejects values outside it. The
     * host follows the same float sequence for the projector's properties. */
    if (s->beta >= 0.0f && s->beta <= 1.0f)
        s->sart_relax = s->beta;
    if ((rc = udev_asd_begin(d, &s->dsc)) || (rc = udev_fill(d, s->x, s->nv * (size_t) s->S, 0.0f)))
        return rc;
    for (unsigned int i = 0; i < s->prm.df_minimizer.num_iterations; i++)
        if ((rc = udev_graph_launch(d, s->sart_exec, s->sart_kernels)))
            return rc;
    if ((rc = udev_graph_launch(d, s->post_exec, s->post_kernels)))
        return rc;
    proj->prm.relaxation = s->sart_relax;
    proj->prm.correction_scale = -1.0f;
    s->beta *= s->prm.beta_red;
    s->it++;
    return UFOIR_OK;
}

static int asdpocs_run(ufoir_projector *proj, const ufoir_asdpocs_params *prm, const float *sino,
                       const size_t dims[2], float *vol, size_t n_slices, float *x_tv,
                       ufoir_asdpocs_scalars *scalars);

int ufoir_asdpocs_process(ufoir_projector *proj, const ufoir_asdpocs_params *prm, const float *sino,
                          const size_t dims[2], float *vol, size_t n_slices)
{
    return asdpocs_run(proj, prm, sino, dims, vol, n_slices, NULL, NULL);
}

int ufoir_asdpocs_process_ex(ufoir_projector *proj, const ufoir_asdpocs_params *prm, const float *sino,
                             const size_t dims[2], float *vol, size_t n_slices, float *x_tv,
                             ufoir_asdpocs_scalars *scalars)
{
    return asdpocs_run(proj, prm, sino, dims, vol, n_slices, x_tv, scalars);
}

static int asdpocs_run(ufoir_projector *proj, const ufoir_asdpocs_params *prm, const float *sino,
                       const size_t dims[2], float *vol, size_t n_slices, float *x_tv,
                       ufoir_asdpocs_scalars *scalars)
{
    if (!proj || !prm || !sino || !vol || !dims)
        return UFOIR_ERR_INVALID;
    ufoir_ctx *ctx = proj->ctx;
    int rc = asdpocs_check(ctx, prm);
    if (rc)
        return rc;
    rc = method_setup(proj, dims, n_slices, prm->num_iterations);
    if (rc)
        return rc;
    const size_t n = proj->n_dets, nv = n * n, ns = n * proj->n_angles;
    ufoir_buf bb = {0}, bo = {0}, bx = {0};
    float *hs = NULL;
    ufoir__asd_state st;
    memset(&st, 0, sizeof(st));
    st.p = proj;
    UFOIR_TRY(ufoir__buf_in(ctx, &bb, sino, ns * n_slices, 1));
    UFOIR_TRY(ufoir__buf_in(ctx, &bo, vol, nv * n_slices, 0));
    UFOIR_TRY(ufoir__asd_setup(&st, proj, prm, bb.dev, bo.dev, (int) n_slices));
    for (unsigned int it = 0; it < prm->num_iterations; it++)
        UFOIR_TRY(ufoir__asd_outer(&st));
    UFOIR_TRY(udev_take_kernel_error(ctx->dev));
    UFOIR_TRY(ufoir__buf_out(ctx, &bo, 1));
    if (x_tv) {
        /* the iterate after the last outer iteration's TV sub-steps */
        UFOIR_TRY(ufoir__buf_in(ctx, &bx, x_tv, nv * n_slices, 0));
        UFOIR_TRY(udev_memcpy_async(ctx->dev, bx.dev, st.x, nv * n_slices * sizeof(float)));
        UFOIR_TRY(ufoir__buf_out(ctx, &bx, 1));
    }
    if (scalars) {
        const size_t S = n_slices;
        hs = (float *) malloc(sizeof(float) * 4 * S);
        if (!hs) {
            rc = ufoir__fail(ctx, UFOIR_ERR_NOMEM, "out of host memory");
            goto done;
        }
        /* dp, dd, dg and dtgv are consecutive runs of S floats */
        UFOIR_TRY(udev_memcpy_async(ctx->dev, hs, st.dsc.dp, sizeof(float) * 4 * S));
        UFOIR_TRY(udev_sync(ctx->dev));
        for (size_t i = 0; i < S; i++) {
            scalars[i].dp = hs[i];
            scalars[i].dd = hs[S + i];
            scalars[i].dg = hs[2 * S + i];
            scalars[i].dtgv = hs[3 * S + i];
        }
    }
done:
    free(hs);
    ufoir__asd_release(&st);
    ufoir__buf_release(ctx, &bb);
    ufoir__buf_release(ctx, &bo);
    ufoir__buf_release(ctx, &bx);
    udev_sync(ctx->dev);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Split-Bregman TV                                                         */
/* ------------------------------------------------------------------------ */
/*
 * SBTV runs S slices in lockstep: processA, the difference operators and the
 * inner products work on all S slices in one launch each, while every
 * slice keeps its own CGS scalars, branches and exits (sbtv-task.c:404-585)
 * on the host, exactly as the per-slice algorithm. A slice that leaves the
 * CGS loop is no longer updated; processA still computes it (its result is
 * discarded), so each slice sees the same operations in the same order as
 * when it runs alone.
 */
#define SBTV_MAX_BATCH 16

typedef struct {
    ufoir_projector *p;
    udev *d;
    udev_geom g;
    size_t n, nv, ns;
    int S;
    float lambda, mu;
    int mode;
    float *tmpA, *tmpAt, *tmpD, *tmpDxt;
    ufoir_fp_scratch fs;
} sbtv_ctx;

/* processA (sbtv-task.c:587-635): out = mu A^T A in + lambda (Dxt Dx in + Dyt Dy in), S slices. */
static int sbtv_processA(sbtv_ctx *c, const float *in, float *out)
{
    udev *d = c->d;
    const int n = (int) c->n, S = c->S;
    const size_t nvS = c->nv * (size_t) S;
    int rc = udev_fill(d, c->tmpA, c->ns * (size_t) S, 0.0f);
    if (!rc)
        rc = ufoir__fp_full(c->p, &c->fs, in, c->tmpA, NULL, 0, c->tmpA, c->p->prm.correction_scale, S);
    if (!rc)
        rc = udev_bp(d, &c->g, c->p->subsets, (int) c->p->n_subsets, c->tmpA, NULL, NULL, 0, NULL, c->tmpAt,
                     c->p->prm.relaxation, S);
    if (!rc)
        rc = udev_unary(d, UDEV_SCALE, c->tmpAt, c->mu, 0, c->tmpAt, nvS);
    if (!rc)
        rc = udev_diff(d, UDEV_DY, in, c->tmpD, n, n, S);
    if (!rc)
        rc = udev_diff(d, UDEV_DYT, c->tmpD, out, n, n, S);
    if (!rc)
        rc = udev_diff(d, UDEV_DX, in, c->tmpD, n, n, S);
    if (!rc)
        rc = udev_diff(d, UDEV_DXT, c->tmpD, c->tmpDxt, n, n, S);
    if (!rc)
        rc = udev_binary(d, UDEV_ADD, out, c->tmpDxt, 0, out, nvS);
    if (!rc)
        rc = udev_unary(d, UDEV_SCALE, out, c->lambda, 0, out, nvS);
    if (!rc)
        rc = udev_binary(d, UDEV_ADD, out, c->tmpAt, 0, out, nvS);
    return rc;
}

/* the reference's inner product of every slice (one launch, one read-back) */
static int sbtv_dots(sbtv_ctx *c, const float *a, const float *b, float *out)
{
    return udev_dot(c->d, a, b, c->n, c->n, c->S, c->mode, out);
}

/* l2_norm (basic-ops-processor.c:239-247): sqrt in double of the float dot. */
static int sbtv_l2s(sbtv_ctx *c, const float *a, float *out)
{
    int rc = sbtv_dots(c, a, a, out);
    for (int s = 0; s < c->S && !rc; s++)
        out[s] = (float) sqrt((double) out[s]);
    return rc;
}

#define SL(ptr, s) ((ptr) + (size_t) (s) * c->nv)

static int copy_s(sbtv_ctx *c, float *dst, const float *src, int s)
{
    return udev_memcpy_async(c->d, SL(dst, s), SL(src, s), c->nv * sizeof(float));
}

static int op_s(sbtv_ctx *c, int op, const float *a, const float *b, float m, float *out, int s)
{
    return udev_binary(c->d, op, SL(a, s), SL(b, s), m, SL(out, s), c->nv);
}

/* per-slice CGS state */
typedef struct {
    float n2b, tolb, normr, normr_act, normmin, rho, alpha;
    unsigned int flag, stag, moresteps;
    int active;      /* still iterating */
    int finished;    /* left before the loop ("initial guess is good enough") */
} cgs_slice;

/* cgs (sbtv-task.c:404-585) on S slices. */
static int sbtv_cgs(sbtv_ctx *c, const float *b, float *x, const float *x0, unsigned int max_iter, float **w)
{
    udev *d = c->d;
    const int S = c->S;
    const size_t nvS = c->nv * (size_t) S;
    float *xmin = w[0], *r = w[1], *rt = w[2], *u = w[3], *tmpa = w[4], *pp = w[5], *ph = w[6], *q = w[7];
    float *vh = w[8], *tempSum = w[9], *uh = w[10], *qh = w[11];
    int rc;
    const float tol = 1E-06f;
    const unsigned int maxmsteps = 5, maxstagsteps = 3;
    cgs_slice st[SBTV_MAX_BATCH];
    float v[SBTV_MAX_BATCH], v2[SBTV_MAX_BATCH];
    memset(st, 0, sizeof(st));
    if ((rc = sbtv_l2s(c, b, v)))
        return rc;
    if ((rc = udev_memcpy_async(d, x, x0, nvS * sizeof(float))) ||
        (rc = udev_memcpy_async(d, xmin, x, nvS * sizeof(float))))
        return rc;
    for (int s = 0; s < S; s++) {
        st[s].n2b = v[s];
        st[s].flag = 1;
        st[s].tolb = tol * st[s].n2b;
    }
    if ((rc = sbtv_processA(c, x, r)) || (rc = udev_binary(d, UDEV_SUB, b, r, 0, r, nvS)) ||
        (rc = sbtv_l2s(c, r, v)))
        return rc;
    int n_active = 0;
    for (int s = 0; s < S; s++) {
        st[s].normr = st[s].normr_act = v[s];
        if (st[s].normr <= st[s].tolb) {
            st[s].finished = 1;   /* "Initial guess is good enough" (:434-440) */
            continue;
        }
        st[s].active = 1;
        st[s].normmin = st[s].normr;
        st[s].rho = 1.0f;
        n_active++;
        if ((rc = copy_s(c, rt, r, s)))
            return rc;
    }
    if ((rc = udev_fill(d, u, nvS, 0.0f)) || (rc = udev_fill(d, tmpa, nvS, 0.0f)) ||
        (rc = udev_fill(d, pp, nvS, 0.0f)) || (rc = udev_fill(d, q, nvS, 0.0f)) ||
        (rc = udev_fill(d, tempSum, nvS, 0.0f)))
        return rc;

    for (unsigned int iter = 0; iter < max_iter && n_active > 0; ++iter) {
        float rho1[SBTV_MAX_BATCH];
        if ((rc = sbtv_dots(c, rt, r, v)))
            return rc;
        for (int s = 0; s < S; s++) {
            if (!st[s].active)
                continue;
            rho1[s] = st[s].rho;
            st[s].rho = v[s];
            const float rho = st[s].rho;
            if (rho == 0 || isinf(rho) || isnan(rho)) {
                st[s].flag = 4;
                st[s].active = 0;
                continue;
            }
            if (iter == 0) {
                if ((rc = copy_s(c, u, r, s)) || (rc = copy_s(c, pp, u, s)))
                    return rc;
            } else {
                const float beta = rho / rho1[s];
                if (beta == 0 || isinf(beta) || isnan(beta)) {
                    st[s].flag = 4;
                    st[s].active = 0;
                    continue;
                }
                if ((rc = op_s(c, UDEV_ADD_SCALED, r, q, beta, u, s)) ||
                    (rc = op_s(c, UDEV_ADD_SCALED, q, pp, beta, tempSum, s)) ||
                    (rc = op_s(c, UDEV_ADD_SCALED, u, tempSum, beta, pp, s)))
                    return rc;
            }
            if ((rc = copy_s(c, ph, pp, s)))
                return rc;
        }
        if ((rc = sbtv_processA(c, ph, vh)) || (rc = sbtv_dots(c, rt, vh, v)))
            return rc;
        for (int s = 0; s < S; s++) {
            if (!st[s].active)
                continue;
            if (v[s] == 0) {
                st[s].flag = 4;
                st[s].active = 0;
                continue;
            }
            st[s].alpha = st[s].rho / v[s];
            if (isinf(st[s].alpha) || isnan(st[s].alpha)) {
                st[s].flag = 4;
                st[s].active = 0;
                continue;
            }
            if ((rc = op_s(c, UDEV_ADD_SCALED, u, vh, -st[s].alpha, q, s)) || (rc = op_s(c, UDEV_ADD, u, q, 0, uh, s)))
                return rc;
        }
        if ((rc = sbtv_l2s(c, uh, v)) || (rc = sbtv_l2s(c, x, v2)))
            return rc;
        for (int s = 0; s < S; s++) {
            if (!st[s].active)
                continue;
            /* fabs() promotes to double; EPS is the double literal 2.2204E-16 (:35, :498) */
            if (fabs((double) st[s].alpha) * (double) v[s] < 2.2204E-16 * (double) v2[s])
                st[s].stag += 1;
            else
                st[s].stag = 0;
            if ((rc = op_s(c, UDEV_ADD_SCALED, x, uh, st[s].alpha, x, s)))
                return rc;
        }
        if ((rc = sbtv_processA(c, uh, qh)))
            return rc;
        for (int s = 0; s < S; s++)
            if (st[s].active && (rc = op_s(c, UDEV_ADD_SCALED, r, qh, -st[s].alpha, r, s)))
                return rc;
        if ((rc = sbtv_l2s(c, r, v)))
            return rc;
        int check = 0;
        for (int s = 0; s < S; s++) {
            if (!st[s].active)
                continue;
            st[s].normr = st[s].normr_act = v[s];
            if (st[s].normr <= st[s].tolb || st[s].stag >= maxstagsteps || st[s].moresteps)
                check = 1;
        }
        if (check) {
            /* the reference applies A to r here (:535) */
            if ((rc = sbtv_processA(c, r, tmpa)))
                return rc;
            int any = 0;
            for (int s = 0; s < S; s++) {
                if (!st[s].active ||
                    !(st[s].normr <= st[s].tolb || st[s].stag >= maxstagsteps || st[s].moresteps))
                    continue;
                if ((rc = op_s(c, UDEV_SUB, b, tmpa, 0, r, s)))
                    return rc;
                any = 1;
            }
            if (any && (rc = sbtv_l2s(c, r, v)))
                return rc;
            for (int s = 0; s < S; s++) {
                if (!st[s].active ||
                    !(st[s].normr <= st[s].tolb || st[s].stag >= maxstagsteps || st[s].moresteps))
                    continue;
                st[s].normr_act = v[s];
                if (st[s].normr_act <= st[s].tolb) {
                    st[s].flag = 0;
                    st[s].active = 0;
                } else {
                    if (st[s].stag >= maxstagsteps && st[s].moresteps == 0)
                        st[s].stag = 0;
                    st[s].moresteps += 1;
                    if (st[s].moresteps >= maxmsteps) {
                        st[s].flag = 3;
                        st[s].active = 0;
                    }
                }
            }
        }
        n_active = 0;
        for (int s = 0; s < S; s++) {
            if (!st[s].active)
                continue;
            if (st[s].normr_act < st[s].normmin) {
                st[s].normmin = st[s].normr_act;
                if ((rc = copy_s(c, xmin, x, s)))
                    return rc;
            }
            if (st[s].stag >= maxstagsteps) {
                st[s].flag = 3;
                st[s].active = 0;
                continue;
            }
            n_active++;
        }
    }
    int any_flag = 0;
    for (int s = 0; s < S; s++)
        any_flag |= !st[s].finished && st[s].flag != 0;
    if (any_flag) {
        if ((rc = sbtv_processA(c, xmin, tmpa)))
            return rc;
        for (int s = 0; s < S; s++)
            if (!st[s].finished && st[s].flag != 0 && (rc = op_s(c, UDEV_SUB, b, tmpa, 0, r, s)))
                return rc;
        if ((rc = sbtv_l2s(c, r, v)))
            return rc;
        for (int s = 0; s < S; s++)
            if (!st[s].finished && st[s].flag != 0 && v[s] <= st[s].normr_act && (rc = copy_s(c, x, xmin, s)))
                return rc;
    }
    return UFOIR_OK;
}

#undef SL

/* normalization (basic-ops-processor.c:342-367), in place on the device. */
static int sbtv_normalize(udev *d, float *v, size_t count)
{
    float lo, hi;
    int rc = udev_minmax(d, v, count, 1, &lo, &hi);
    if (rc)
        return rc;
    const float delta = 1 / (hi - lo);
    return udev_unary(d, UDEV_NORMALIZE, v, delta, lo, v, count);
}

#define SBTV_NBUF 26

int ufoir_sbtv_process(ufoir_projector *proj, const ufoir_sbtv_params *prm, const float *sino,
                       const size_t dims[2], float *vol, size_t n_slices)
{
    if (!proj || !prm || !sino || !vol || !dims)
        return UFOIR_ERR_INVALID;
    ufoir_ctx *ctx = proj->ctx;
    int rc;
    if (!(prm->lambda >= 0.0f) || !(prm->mu >= 0.0f))
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "lambda and mu must be >= 0");
    if (prm->norm_mode != UFOIR_NORM_COMPAT && prm->norm_mode != UFOIR_NORM_FP64)
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "unknown norm_mode %d", prm->norm_mode);
    rc = method_setup(proj, dims, n_slices, prm->num_iterations);
    if (rc)
        return rc;
    const size_t n = proj->n_dets, nv = n * n, ns = n * proj->n_angles;
    const int S_max = n_slices < SBTV_MAX_BATCH ? (int) n_slices : SBTV_MAX_BATCH;
    udev *d = ctx->dev;
    sbtv_ctx c;
    memset(&c, 0, sizeof(c));
    c.p = proj;
    c.d = d;
    ufoir__projector_geom(proj, &c.g);
    c.n = n;
    c.nv = nv;
    c.ns = ns;
    c.lambda = prm->lambda;
    c.mu = prm->mu;
    c.mode = prm->norm_mode;

    ufoir_buf bb = {0}, bo = {0};
    float *buf[SBTV_NBUF] = {0};
    float *f = NULL;
    UFOIR_TRY(ufoir__buf_in(ctx, &bb, sino, ns * n_slices, 1));
    UFOIR_TRY(ufoir__buf_in(ctx, &bo, vol, nv * n_slices, 0));
    UFOIR_TRY(ufoir__alloc(ctx, &f, ns * (size_t) S_max));
    UFOIR_TRY(ufoir__alloc(ctx, &c.tmpA, ns * (size_t) S_max));
    for (int i = 0; i < SBTV_NBUF; i++)
        UFOIR_TRY(ufoir__alloc(ctx, &buf[i], nv * (size_t) S_max));
    c.tmpAt = buf[12];
    c.tmpD = buf[13];
    c.tmpDxt = buf[14];
    UFOIR_TRY(ufoir__fp_scratch_alloc(proj, &c.fs, (size_t) S_max));
    float *fbp = buf[16], *up = buf[17], *bvec = buf[18], *bx = buf[19], *by = buf[20], *dx = buf[21];
    float *dy = buf[22], *tmpx = buf[23], *tmpy = buf[24], *tmp = buf[25];

    for (size_t s0 = 0; s0 < n_slices; s0 += (size_t) S_max) {
        const int S = n_slices - s0 < (size_t) S_max ? (int) (n_slices - s0) : S_max;
        const size_t nvS = nv * (size_t) S;
        c.S = S;
        float *u = bo.dev + s0 * nv;
        /* normalise the input (a copy; the reference does it in place, :239),
         * copy it to f and normalise f again (:246-248), per slice */
        UFOIR_TRY(udev_memcpy_async(d, f, bb.dev + s0 * ns, ns * (size_t) S * sizeof(float)));
        for (int s = 0; s < S; s++) {
            UFOIR_TRY(sbtv_normalize(d, f + (size_t) s * ns, ns));
            UFOIR_TRY(sbtv_normalize(d, f + (size_t) s * ns, ns));
        }
        /* fbp = A^T f (:251-253), u = 0, bx = by = dx = dy = 0, fbp *= mu (:279) */
        UFOIR_TRY(udev_bp(d, &c.g, proj->subsets, (int) proj->n_subsets, f, NULL, NULL, 0, NULL, fbp,
                          proj->prm.relaxation, S));
        UFOIR_TRY(udev_fill(d, u, nvS, 0.0f));
        UFOIR_TRY(udev_fill(d, bx, nvS, 0.0f));
        UFOIR_TRY(udev_fill(d, by, nvS, 0.0f));
        UFOIR_TRY(udev_fill(d, dx, nvS, 0.0f));
        UFOIR_TRY(udev_fill(d, dy, nvS, 0.0f));
        UFOIR_TRY(udev_unary(d, UDEV_SCALE, fbp, c.mu, 0, fbp, nvS));
        const float d_lambda = (float) -1 / c.lambda;

        for (unsigned int it = 0; it < prm->num_iterations; ++it) {
            UFOIR_TRY(udev_memcpy_async(d, up, u, nvS * sizeof(float)));
            /* calculate_b (:304-334) */
            UFOIR_TRY(udev_binary(d, UDEV_SUB, dx, bx, 0, tmp, nvS));
            UFOIR_TRY(udev_diff(d, UDEV_DXT, tmp, tmpx, (int) n, (int) n, S));
            UFOIR_TRY(udev_binary(d, UDEV_SUB, dy, by, 0, tmp, nvS));
            UFOIR_TRY(udev_diff(d, UDEV_DYT, tmp, tmpy, (int) n, (int) n, S));
            UFOIR_TRY(udev_binary(d, UDEV_ADD, tmpx, tmpy, 0, bvec, nvS));
            UFOIR_TRY(udev_unary(d, UDEV_SCALE, bvec, c.lambda, 0, bvec, nvS));
            UFOIR_TRY(udev_binary(d, UDEV_ADD, fbp, bvec, 0, bvec, nvS));

            UFOIR_TRY(sbtv_cgs(&c, bvec, u, up, 30, buf));

            /* update_db (:336-402) */
            float *s_ = buf[0], *top = buf[1], *e12 = buf[2];
            UFOIR_TRY(udev_diff(d, UDEV_DX, u, tmpx, (int) n, (int) n, S));
            UFOIR_TRY(udev_binary(d, UDEV_ADD, tmpx, bx, 0, tmpx, nvS));
            UFOIR_TRY(udev_diff(d, UDEV_DY, u, tmpy, (int) n, (int) n, S));
            UFOIR_TRY(udev_binary(d, UDEV_ADD, tmpy, by, 0, tmpy, nvS));
            UFOIR_TRY(udev_binary(d, UDEV_MUL, tmpx, tmpx, 0, s_, nvS));
            UFOIR_TRY(udev_binary(d, UDEV_MUL, tmpy, tmpy, 0, tmp, nvS));
            UFOIR_TRY(udev_binary(d, UDEV_ADD, s_, tmp, 0, s_, nvS));
            UFOIR_TRY(udev_unary(d, UDEV_SQRT, s_, 0, 0, s_, nvS));
            UFOIR_TRY(udev_unary(d, UDEV_ADDC, s_, d_lambda, 0, top, nvS));
            UFOIR_TRY(udev_unary(d, UDEV_MAXC, top, 0.0f, 0, top, nvS));
            UFOIR_TRY(udev_unary(d, UDEV_MAXC, s_, 1E-12f, 0, e12, nvS));
            UFOIR_TRY(udev_binary(d, UDEV_DIV, top, e12, 0, tmp, nvS));
            UFOIR_TRY(udev_binary(d, UDEV_MUL, tmp, tmpx, 0, dx, nvS));
            UFOIR_TRY(udev_binary(d, UDEV_MUL, tmp, tmpy, 0, dy, nvS));
            UFOIR_TRY(udev_binary(d, UDEV_SUB, tmpx, dx, 0, bx, nvS));
            UFOIR_TRY(udev_binary(d, UDEV_SUB, tmpy, dy, 0, by, nvS));
        }
    }
    UFOIR_TRY(ufoir__buf_out(ctx, &bo, 1));
done:
    for (int i = 0; i < SBTV_NBUF; i++)
        ufoir__free(ctx, buf[i]);
    ufoir__free(ctx, f);
    ufoir__free(ctx, c.tmpA);
    ufoir__fp_scratch_free(proj, &c.fs);
    ufoir__buf_release(ctx, &bb);
    ufoir__buf_release(ctx, &bo);
    udev_sync(ctx->dev);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Exposed reductions                                                       */
/* ------------------------------------------------------------------------ */
int ufoir_l1_norm(ufoir_ctx *ctx, const float *v, size_t w, size_t h, int norm_mode, float *out)
{
    if (!ctx || !v || !out || w == 0 || h == 0)
        return UFOIR_ERR_INVALID;
    ufoir_buf b = {0};
    int rc;
    UFOIR_TRY(ufoir__buf_in(ctx, &b, v, w * h, 1));
    UFOIR_TRY(udev_l1_norm(ctx->dev, b.dev, w, h, 1, norm_mode, out));
done:
    ufoir__buf_release(ctx, &b);
    udev_sync(ctx->dev);
    return rc;
}

int ufoir_dot_product(ufoir_ctx *ctx, const float *a, const float *b, size_t w, size_t h, int norm_mode,
                      float *out)
{
    if (!ctx || !a || !b || !out || w == 0 || h == 0)
        return UFOIR_ERR_INVALID;
    ufoir_buf ba = {0}, bb = {0};
    int rc;
    UFOIR_TRY(ufoir__buf_in(ctx, &ba, a, w * h, 1));
    UFOIR_TRY(ufoir__buf_in(ctx, &bb, b, w * h, 1));
    UFOIR_TRY(udev_dot(ctx->dev, ba.dev, bb.dev, w, h, 1, norm_mode, out));
done:
    ufoir__buf_release(ctx, &ba);
    ufoir__buf_release(ctx, &bb);
    udev_sync(ctx->dev);
    return rc;
}

int ufoir_tv_gradient(ufoir_ctx *ctx, const float *v, size_t w, size_t h, size_t n_slices, float *out)
{
    if (!ctx || !v || !out || w == 0 || h == 0 || n_slices == 0)
        return UFOIR_ERR_INVALID;
    if (w > (size_t) INT32_MAX || h > (size_t) INT32_MAX || n_slices > 65535)
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "tv_gradient: %zu x %zu x %zu is too large", w, h, n_slices);
    ufoir_buf bi = {0}, bo = {0};
    int rc;
    UFOIR_TRY(ufoir__buf_in(ctx, &bi, v, w * h * n_slices, 1));
    UFOIR_TRY(ufoir__buf_in(ctx, &bo, out, w * h * n_slices, 0));
    UFOIR_TRY(udev_l1_grad(ctx->dev, bi.dev, bo.dev, (int) w, (int) h, (int) n_slices));
    UFOIR_TRY(udev_take_kernel_error(ctx->dev));
    UFOIR_TRY(ufoir__buf_out(ctx, &bo, 1));
done:
    ufoir__buf_release(ctx, &bi);
    ufoir__buf_release(ctx, &bo);
    udev_sync(ctx->dev);
    return rc;
}
