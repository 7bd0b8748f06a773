/*
 * serve.c - continuous-batching request loop for reconstruction jobs.
 *
 * One worker thread owns a private context (its own streams) on the caller's
 * GPU. Jobs wait in arrival order; the worker admits queued jobs whenever the
 * active-job limit and the HBM budget allow (which job, per policy:
 * pick_admission), sets each up on its own CUDA stream (sinogram upload,
 * weights, one captured CUDA graph per iteration or sweep), and then gives
 * quanta to the idle active jobs with the least remaining work first, at
 * most max_running with work in flight, issuing a job's next quantum only
 * when its previous one has finished (an event query, never a blocking
 * wait). Different jobs' kernels therefore run side by side on the GPU and a
 * queued job starts as soon as memory frees up. Each job runs exactly the
 * kernels of the plain ufoir_*_process call on one slice (or, with
 * batch_sirt, of a mixed batch, whose members equal their runs alone), so
 * its result is independent of the mix.
 */
#include <errno.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#include "host.h"

#define DEFAULT_MAX_ACTIVE 32
#define DEFAULT_MAX_RUNNING 4
#define DEFAULT_ADMIT_AGE_MS 2000

enum { PH_QUEUED = 0, PH_RUN = 1, PH_FINAL = 2, PH_END = 3 };

typedef struct job {
    uint64_t id;
    ufoir_job_desc d;
    const float *user_sino;
    float *user_vol;
    int state;          /* UFOIR_JOB_* */
    int status;         /* final status */
    double t_submit, t_start, t_end;
    size_t bytes;
    /* runtime (worker thread only) */
    int phase;
    int busy;
    void *stream, *event;
    ufoir_projector *proj;
    float *b, *x, *R, *C, *resid, *work, *table;
    ufoir__sirt_iter sirt;
    ufoir__sart_iter sart;
    ufoir__asd_state asd;
    int asd_live;
    void *graph;
    uint64_t graph_kernels;
    unsigned int done_iters, total_iters;
    unsigned int total_work_iters;  /* iterations the job asks for (known at submission) */
    int pooled;                 /* SIRT job that advances in the server's mixed batch */
    double work_per_iter;       /* interpolated samples of one quantum's iteration */
    struct job *next;
} job;

struct ufoir_server {
    ufoir_ctx *user_ctx;
    ufoir_ctx *ctx;             /* private context of the worker */
    ufoir_serve_config cfg;
    pthread_t worker;
    int worker_started;
    pthread_mutex_t mu;
    pthread_cond_t cv_work, cv_done;
    int stop;
    job **jobs;
    size_t n_jobs, cap_jobs;
    job *pend_head, *pend_tail;
    job **active;
    unsigned int n_active;
    uint64_t reserved, peak_reserved;
    unsigned int peak_active;
    uint64_t submitted, completed, failed, cancelled, rejected;
    double *lat, *qlat;
    size_t n_lat, cap_lat;
    double first_submit, last_done;
    uint64_t starts;            /* job set-ups attempted (failure injection) */
    /* CONTINUOUS: SIRT jobs advance together, one mixed batch (batch.c) of
     * the idle ones per quantum, on the pool's own stream */
    void *pool_stream;
    ufoir_batch *pool;
    uint64_t *pool_ids;         /* job ids of the built batch, in member order */
    unsigned int n_pool, cap_pool;
    int pool_off;               /* set if a batch could not be built: per-job graphs from then on */
    uint64_t pool_quanta;       /* batched iterations issued (statistics) */
};

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double) ts.tv_sec + 1e-9 * (double) ts.tv_nsec;
}

void ufoir_serve_config_init(ufoir_serve_config *c)
{
    if (!c)
        return;
    memset(c, 0, sizeof(*c));
    c->max_active_jobs = DEFAULT_MAX_ACTIVE;
    c->policy = UFOIR_SERVE_CONTINUOUS;
    c->quantum = 1;
    c->max_running = DEFAULT_MAX_RUNNING;
    c->admit_age_ms = DEFAULT_ADMIT_AGE_MS;
    c->batch_sirt = 0;
}

void ufoir_job_desc_init(ufoir_job_desc *j)
{
    if (!j)
        return;
    memset(j, 0, sizeof(*j));
    j->method = UFOIR_METHOD_SIRT;
    j->axis_position = -1.0f;
    ufoir_sart_params_init(&j->sart);
    ufoir_asdpocs_params_init(&j->asdpocs);
}

/* Device bytes a job holds while active (plus the weight scratch). */
static size_t job_bytes(const ufoir_job_desc *d)
{
    const size_t n = d->n_dets, na = d->n_angles, nv = n * n, ns = n * na;
    const size_t fs = 2 * n * (size_t) udev_fp_pitch((int) n);
    switch (d->method) {
    case UFOIR_METHOD_SIRT:
        return sizeof(float) * (ns + nv + ns + ns + nv + 2 * fs);
    case UFOIR_METHOD_SART:
        return sizeof(float) * (ns + nv + (ns > nv ? ns : nv) + ns + fs) + ufoir__sart_scratch_bytes(n, na, 1);
    default:
        return sizeof(float) * (ns + nv + fs) + ufoir__asd_bytes(n, na, 1);
    }
}

/* Interpolated samples of one scheduling quantum's iteration: FP + BP over
 * every angle (2 n^2 n_a); an ASD-POCS outer iteration is its SART sweeps
 * plus one FP. Used to order jobs by remaining work. */
static double job_work_per_iter(const ufoir_job_desc *d)
{
    const double n = d->n_dets, na = d->n_angles, pass = n * n * na;
    if (d->method == UFOIR_METHOD_ASDPOCS)
        return pass * (2.0 * d->asdpocs.df_minimizer.num_iterations + 1.0);
    return 2.0 * pass;
}

static int check_desc(ufoir_ctx *ctx, const ufoir_job_desc *d)
{
    if (d->method != UFOIR_METHOD_SART && d->method != UFOIR_METHOD_SIRT && d->method != UFOIR_METHOD_ASDPOCS)
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "unknown method %d", d->method);
    if (d->n_dets == 0 || d->n_dets > 65535 || d->n_angles == 0)
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "job dims %u x %u invalid", d->n_dets, d->n_angles);
    if (!(d->step >= 0.0f) || !(d->axis_position >= -1.0f))
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "job step/axis_position out of range");
    if (d->method == UFOIR_METHOD_ASDPOCS) {
        const ufoir_asdpocs_params *a = &d->asdpocs;
        if (a->num_iterations < 1 || a->df_minimizer.num_iterations < 1 ||
            !(a->df_minimizer.relaxation_factor >= 0.0f && a->df_minimizer.relaxation_factor <= 1.0f) ||
            !(a->beta >= 0 && a->beta_red >= 0 && a->alpha >= 0 && a->alpha_red >= 0 && a->r_max >= 0) ||
            a->ng > 1000 || (a->norm_mode != UFOIR_NORM_COMPAT && a->norm_mode != UFOIR_NORM_FP64))
            return ufoir__fail(ctx, UFOIR_ERR_INVALID, "ASD-POCS job parameters out of range");
    } else if (d->sart.num_iterations < 1 ||
               !(d->sart.relaxation_factor >= 0.0f && d->sart.relaxation_factor <= 1.0f)) {
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "num-iterations must be >= 1 and relaxation_factor in [0, 1]");
    }
    return UFOIR_OK;
}

/* ---------------------------------------------------------------- worker */

static void job_release(ufoir_server *s, job *j)
{
    ufoir_ctx *ctx = s->ctx;
    if (j->stream)
        udev_use_stream(ctx->dev, j->stream);
    if (j->asd_live) {
        ufoir__asd_release(&j->asd);
        j->asd_live = 0;
    }
    udev_graph_destroy(j->graph);
    j->graph = NULL;
    ufoir__free(ctx, j->b);
    ufoir__free(ctx, j->x);
    ufoir__free(ctx, j->R);
    ufoir__free(ctx, j->C);
    ufoir__free(ctx, j->resid);
    ufoir__free(ctx, j->work);
    ufoir__free(ctx, j->table);
    if (j->sirt.fs.P || j->sirt.fs.TP)
        ufoir__fp_scratch_free(j->proj, &j->sirt.fs);
    j->b = j->x = j->R = j->C = j->resid = j->work = j->table = NULL;
    if (j->stream)
        udev_sync(ctx->dev);
    udev_use_stream(ctx->dev, NULL);
    if (j->proj) {
        ufoir_projector_destroy(j->proj);
        j->proj = NULL;
    }
    udev_event_destroy(j->event);
    j->event = NULL;
    udev_stream_destroy(ctx->dev, j->stream);
    j->stream = NULL;
}

static int capture_body(ufoir_server *s, job *j, int (*body)(void *), void *arg)
{
    int rc = udev_capture_begin(s->ctx->dev);
    if (rc)
        return rc;
    rc = body(arg);
    void *e = NULL;
    const int rc2 = udev_capture_end(s->ctx->dev, &e, &j->graph_kernels);
    if (rc || rc2) {
        udev_graph_destroy(e);
        return rc ? rc : rc2;
    }
    j->graph = e;
    return UFOIR_OK;
}

/* A SIRT job the mixed batch can carry: the tiled projectors serve its
 * geometry (at least 16 angles, at most 16 direction runs, clamp edges in
 * order, a tiled forward launch shape). */
static int pool_eligible(ufoir_server *s, ufoir_projector *p)
{
    if (p->n_angles < 16 || p->n_subsets > 16 || udev_fp_tile_angles(s->ctx->dev, (int) p->n_dets) <= 0)
        return 0;
    const float n = (float) p->n_dets, axis = ufoir__axis(p);
    const float half = n - axis * 2.0f < 0.0f ? n - axis : axis;
    return axis - half + 0.5f <= axis + half - 0.5f;
}

/* Set-up on the job's stream: upload, weights, captured iteration. */
static int job_start(ufoir_server *s, job *j)
{
    ufoir_ctx *ctx = s->ctx;
    udev *d = ctx->dev;
    const ufoir_job_desc *jd = &j->d;
    const size_t n = jd->n_dets, na = jd->n_angles, nv = n * n, ns = n * na;
    int rc;
    s->starts++;
    if (s->cfg.fail_allocation_every && s->starts % s->cfg.fail_allocation_every == 0)
        return ufoir__fail(ctx, UFOIR_ERR_NOMEM, "injected allocation failure (job %llu)",
                           (unsigned long long) j->id);
    if ((rc = udev_stream_create(d, &j->stream)) || (rc = udev_event_create(d, &j->event)))
        return rc;
    udev_use_stream(d, j->stream);
    ufoir_projector_params pp;
    ufoir_projector_params_init(&pp);
    pp.is_forward = 0;
    pp.step = jd->step;
    pp.axis_position = jd->axis_position;
    pp.angles_num = jd->n_angles;
    if ((rc = ufoir_projector_create(ctx, &pp, &j->proj)) ||
        (rc = ufoir__projector_prepare_na(j->proj, (unsigned int) n, (unsigned int) na)))
        return rc;
    if ((rc = ufoir__alloc(ctx, &j->b, ns)) || (rc = ufoir__alloc(ctx, &j->x, nv)) ||
        (rc = udev_memcpy_async(d, j->b, j->user_sino, ns * sizeof(float))))
        return rc;
    ufoir_projector *p = j->proj;
    switch (jd->method) {
    case UFOIR_METHOD_SIRT:
        if ((rc = ufoir__alloc(ctx, &j->R, ns)) || (rc = ufoir__alloc(ctx, &j->C, nv)) ||
            (rc = ufoir__alloc(ctx, &j->resid, ns)) || (rc = ufoir__fp_scratch_alloc(p, &j->sirt.fs, 1)))
            return rc;
        p->prm.relaxation = 1.0f;
        p->prm.correction_scale = 1.0f;
        if ((rc = ufoir__ray_weights(p, j->R, j->x)) || (rc = ufoir__pixel_weights(p, j->C, j->resid)))
            return rc;
        p->prm.relaxation = jd->sart.relaxation_factor;
        p->prm.correction_scale = -1.0f;
        if ((rc = udev_fill(d, j->x, nv, 0.0f)))
            return rc;
        j->sirt.p = p;
        ufoir__projector_geom(p, &j->sirt.g);
        j->sirt.b = j->b;
        j->sirt.x = j->x;
        j->sirt.resid = j->resid;
        j->sirt.R = j->R;
        j->sirt.C = j->C;
        j->sirt.lambda = jd->sart.relaxation_factor;
        j->sirt.n_slices = 1;
        if ((rc = capture_body(s, j, ufoir__sirt_body, &j->sirt)))
            return rc;
        j->total_iters = jd->sart.num_iterations;
        j->pooled = s->cfg.policy == UFOIR_SERVE_CONTINUOUS && s->cfg.batch_sirt && !s->pool_off &&
                    pool_eligible(s, p);
        break;
    case UFOIR_METHOD_SART:
        if ((rc = ufoir__alloc(ctx, &j->R, ns)) || (rc = ufoir__alloc(ctx, &j->resid, ns > nv ? ns : nv)) ||
            (rc = ufoir__sart_scratch_alloc(p, &j->work, &j->table, 1)))
            return rc;
        p->prm.correction_scale = 1.0f;
        if ((rc = ufoir__ray_weights(p, j->R, j->resid)))
            return rc;
        p->prm.correction_scale = -1.0f;
        p->prm.relaxation = jd->sart.relaxation_factor;
        if ((rc = udev_fill(d, j->x, nv, 0.0f)))
            return rc;
        j->sart.p = p;
        ufoir__projector_geom(p, &j->sart.g);
        j->sart.b = j->b;
        j->sart.x = j->x;
        j->sart.resid = j->resid;
        j->sart.R = j->R;
        j->sart.lambda = jd->sart.relaxation_factor;
        j->sart.n_slices = 1;
        j->sart.work = j->work;
        j->sart.table = j->table;
        if ((rc = capture_body(s, j, ufoir__sart_body, &j->sart)))
            return rc;
        j->total_iters = jd->sart.num_iterations;
        break;
    default:
        if ((rc = ufoir__asd_setup(&j->asd, p, &jd->asdpocs, j->b, j->x, 1)))
            return rc;
        j->asd_live = 1;
        j->total_iters = jd->asdpocs.num_iterations;
        break;
    }
    j->done_iters = 0;
    return udev_event_record(d, j->event);
}

/* One scheduling quantum on the job's stream. */
static int job_quantum(ufoir_server *s, job *j)
{
    udev *d = s->ctx->dev;
    udev_use_stream(d, j->stream);
    int rc = UFOIR_OK;
    if (j->d.method == UFOIR_METHOD_ASDPOCS) {
        rc = ufoir__asd_outer(&j->asd);
        j->done_iters++;
    } else {
        const unsigned int q = s->cfg.quantum ? s->cfg.quantum : 1;
        const unsigned int left = j->total_iters - j->done_iters;
        const unsigned int k = left < q ? left : q;
        for (unsigned int i = 0; i < k && rc == UFOIR_OK; i++)
            rc = udev_graph_launch(d, j->graph, j->graph_kernels);
        j->done_iters += k;
    }
    if (rc == UFOIR_OK)
        rc = udev_event_record(d, j->event);
    return rc;
}

static int job_finalize(ufoir_server *s, job *j)
{
    udev *d = s->ctx->dev;
    udev_use_stream(d, j->stream);
    const size_t nv = (size_t) j->d.n_dets * j->d.n_dets;
    int rc = udev_memcpy_async(d, j->user_vol, j->x, nv * sizeof(float));
    if (rc == UFOIR_OK)
        rc = udev_event_record(d, j->event);
    return rc;
}

static void job_finish(ufoir_server *s, job *j, int status)
{
    if (status == UFOIR_OK) {
        udev_use_stream(s->ctx->dev, j->stream);
        status = udev_take_kernel_error(s->ctx->dev);
    }
    job_release(s, j);
    pthread_mutex_lock(&s->mu);
    j->t_end = now_s();
    j->status = status;
    j->state = status == UFOIR_OK ? UFOIR_JOB_DONE : UFOIR_JOB_FAILED;
    s->reserved -= j->bytes;
    if (status == UFOIR_OK) {
        s->completed++;
        if (s->n_lat == s->cap_lat) {
            size_t cap = s->cap_lat ? 2 * s->cap_lat : 256;
            double *a = (double *) realloc(s->lat, cap * sizeof(double));
            double *b = a ? (double *) realloc(s->qlat, cap * sizeof(double)) : NULL;
            if (a)
                s->lat = a;
            if (b) {
                s->qlat = b;
                s->cap_lat = cap;
            }
        }
        if (s->n_lat < s->cap_lat) {
            s->lat[s->n_lat] = 1e3 * (j->t_end - j->t_submit);
            s->qlat[s->n_lat] = 1e3 * (j->t_start - j->t_submit);
            s->n_lat++;
        }
        if (j->t_end > s->last_done)
            s->last_done = j->t_end;
    } else {
        s->failed++;
    }
    for (unsigned int i = 0; i < s->n_active; i++)
        if (s->active[i] == j) {
            memmove(&s->active[i], &s->active[i + 1], (s->n_active - i - 1) * sizeof(job *));
            s->n_active--;
            break;
        }
    pthread_cond_broadcast(&s->cv_done);
    pthread_mutex_unlock(&s->mu);
}

/* One quantum of the mixed batch over the given idle pooled jobs, on the
 * pool's stream: the batch is (re)built when the set of jobs changed since
 * the last build (jobs joined or finished; every job is idle, so no batched
 * work is in flight), then each job's event is recorded after the quantum. */
static int pool_quantum(ufoir_server *s, job **jobs, unsigned int n)
{
    udev *d = s->ctx->dev;
    int rc;
    if (!s->pool_stream && (rc = udev_stream_create(d, &s->pool_stream)))
        return rc;
    udev_use_stream(d, s->pool_stream);
    int same = s->pool && s->n_pool == n;
    for (unsigned int i = 0; i < n && same; i++)
        same = s->pool_ids[i] == jobs[i]->id;
    if (!same) {
        /* members in id order, so that the same set gives the same batch */
        for (unsigned int a = 1; a < n; a++) {
            job *k = jobs[a];
            unsigned int b = a;
            while (b > 0 && jobs[b - 1]->id > k->id) {
                jobs[b] = jobs[b - 1];
                b--;
            }
            jobs[b] = k;
        }
        same = s->pool && s->n_pool == n;
        for (unsigned int i = 0; i < n && same; i++)
            same = s->pool_ids[i] == jobs[i]->id;
    }
    if (!same) {
        ufoir_batch_destroy(s->pool);
        s->pool = NULL;
        s->n_pool = 0;
        if (n > s->cap_pool) {
            uint64_t *ids = (uint64_t *) realloc(s->pool_ids, sizeof(uint64_t) * n);
            if (!ids)
                return ufoir__fail(s->ctx, UFOIR_ERR_NOMEM, "out of host memory");
            s->pool_ids = ids;
            s->cap_pool = n;
        }
        ufoir__bmember *m = (ufoir__bmember *) calloc(n, sizeof(*m));
        if (!m)
            return ufoir__fail(s->ctx, UFOIR_ERR_NOMEM, "out of host memory");
        for (unsigned int i = 0; i < n; i++) {
            job *j = jobs[i];
            m[i].p = j->proj;
            m[i].b = j->b;
            m[i].x = j->x;
            m[i].R = j->R;
            m[i].C = j->C;
            m[i].resid = j->resid;
            m[i].P = j->sirt.fs.P;
            m[i].TP = j->sirt.fs.TP;
            m[i].lambda = j->d.sart.relaxation_factor;
            m[i].shape_slices = 1;
            s->pool_ids[i] = j->id;
        }
        rc = ufoir__batch_build(s->ctx, m, (int) n, &s->pool);
        free(m);
        if (rc)
            return rc;
        s->n_pool = n;
    }
    /* as many iterations as the quantum, but no member past its count */
    unsigned int k = s->cfg.quantum ? s->cfg.quantum : 1;
    for (unsigned int i = 0; i < n; i++) {
        const unsigned int left = jobs[i]->total_iters - jobs[i]->done_iters;
        k = left < k ? left : k;
    }
    if ((rc = ufoir__batch_launch(s->pool, k)))
        return rc;
    s->pool_quanta += k;
    for (unsigned int i = 0; i < n; i++) {
        jobs[i]->done_iters += k;
        if ((rc = udev_event_record(d, jobs[i]->event)))
            return rc;
        jobs[i]->busy = 1;
    }
    return UFOIR_OK;
}

/* Removes j (whose predecessor in the queue is prev, NULL at the head) from
 * the pending queue. Caller holds the lock. */
static void unlink_pending(ufoir_server *s, job *prev, job *j)
{
    if (prev)
        prev->next = j->next;
    else
        s->pend_head = j->next;
    if (s->pend_tail == j)
        s->pend_tail = prev;
    j->next = NULL;
}

/* Picks the next queued job to admit, or NULL. Caller holds the lock.
 *  - ONE_AT_A_TIME: the head of the queue (arrival order), when it fits;
 *  - SJF_ONE_AT_A_TIME: the queued job with the least total work that fits
 *    (ties: arrival order);
 *  - CONTINUOUS: the first job in arrival order that fits the budget. A job
 *    that does not fit may be passed by later jobs that do, until it has
 *    waited admit_age_ms; from then on nothing behind it is admitted, so
 *    the memory that frees up goes to it. */
static job *pick_admission(ufoir_server *s, double now, job **prev_out)
{
    const uint64_t budget = s->cfg.hbm_budget_bytes;
    job *prev = NULL;
    if (s->cfg.policy == UFOIR_SERVE_ONE_AT_A_TIME) {
        job *j = s->pend_head;
        if (j && s->reserved + j->bytes <= budget) {
            *prev_out = NULL;
            return j;
        }
        return NULL;
    }
    if (s->cfg.policy == UFOIR_SERVE_SJF_ONE_AT_A_TIME) {
        job *best = NULL, *best_prev = NULL;
        double best_work = 0.0;
        for (job *j = s->pend_head; j; prev = j, j = j->next) {
            if (s->reserved + j->bytes > budget)
                continue;
            const double w = j->work_per_iter * (double) j->total_work_iters;
            if (!best || w < best_work) {
                best = j;
                best_prev = prev;
                best_work = w;
            }
        }
        *prev_out = best_prev;
        return best;
    }
    const double age_limit = 1e-3 * (double) (s->cfg.admit_age_ms ? s->cfg.admit_age_ms : DEFAULT_ADMIT_AGE_MS);
    for (job *j = s->pend_head; j; prev = j, j = j->next) {
        if (s->reserved + j->bytes <= budget) {
            *prev_out = prev;
            return j;
        }
        if (now - j->t_submit >= age_limit)
            return NULL;      /* an old job waits for memory: admit nothing past it */
    }
    return NULL;
}

static void *worker_main(void *arg)
{
    ufoir_server *s = (ufoir_server *) arg;
    const int serial = s->cfg.policy != UFOIR_SERVE_CONTINUOUS;
    const unsigned int max_active = serial ? 1 : (s->cfg.max_active_jobs ? s->cfg.max_active_jobs : DEFAULT_MAX_ACTIVE);
    const unsigned int max_running = serial ? 1 : (s->cfg.max_running ? s->cfg.max_running : DEFAULT_MAX_RUNNING);
    for (;;) {
        /* admission (order: see pick_admission) */
        job *admit[64];
        unsigned int n_admit = 0;
        pthread_mutex_lock(&s->mu);
        const double now = now_s();
        while (s->pend_head && s->n_active + n_admit < max_active && n_admit < 64) {
            job *prev = NULL;
            job *j = pick_admission(s, now, &prev);
            if (!j)
                break;
            unlink_pending(s, prev, j);
            s->reserved += j->bytes;
            if (s->reserved > s->peak_reserved)
                s->peak_reserved = s->reserved;
            j->state = UFOIR_JOB_RUNNING;
            j->t_start = now_s();
            admit[n_admit++] = j;
        }
        for (unsigned int i = 0; i < n_admit; i++)
            s->active[s->n_active++] = admit[i];
        if (s->n_active > s->peak_active)
            s->peak_active = s->n_active;
        if (s->n_active == 0) {
            if (s->stop && !s->pend_head) {
                pthread_mutex_unlock(&s->mu);
                break;
            }
            if (!s->pend_head)
                pthread_cond_wait(&s->cv_work, &s->mu);
            pthread_mutex_unlock(&s->mu);
            continue;
        }
        job *list[1024];
        unsigned int n_list = s->n_active < 1024 ? s->n_active : 1024;
        memcpy(list, s->active, n_list * sizeof(job *));
        pthread_mutex_unlock(&s->mu);

        for (unsigned int i = 0; i < n_admit; i++) {
            job *j = admit[i];
            const int rc = job_start(s, j);
            if (rc != UFOIR_OK) {
                j->phase = PH_END;
                job_finish(s, j, rc);
            } else {
                j->phase = PH_RUN;
                j->busy = 1;
            }
        }
        int progressed = n_admit > 0;
        /* 1. completions; jobs whose iterations are done are finalized */
        unsigned int running = 0;
        job *idle[1024];
        unsigned int n_idle = 0;
        for (unsigned int i = 0; i < n_list; i++) {
            job *j = list[i];
            if (j->phase == PH_END)
                continue;
            if (j->busy) {
                const int q = udev_event_done(s->ctx->dev, j->event);
                if (q == 0) {
                    running++;
                    continue;
                }
                j->busy = 0;
                progressed = 1;
                if (q < 0) {
                    j->phase = PH_END;
                    job_finish(s, j, q);
                    continue;
                }
            }
            if (j->phase == PH_FINAL) {
                j->phase = PH_END;
                job_finish(s, j, UFOIR_OK);
                progressed = 1;
            } else if (j->phase == PH_RUN && j->done_iters >= j->total_iters) {
                const int rc = job_finalize(s, j);
                j->phase = PH_FINAL;
                if (rc != UFOIR_OK) {
                    j->phase = PH_END;
                    job_finish(s, j, rc);
                } else {
                    j->busy = 1;
                }
                progressed = 1;
            } else if (j->phase == PH_RUN) {
                idle[n_idle++] = j;
            }
        }
        /* 2. quanta: least remaining work first (ties: arrival order), at
         * most max_running jobs with work in flight */
        for (unsigned int a = 1; a < n_idle; a++) {
            job *k = idle[a];
            const double rk = (double) (k->total_iters - k->done_iters) * k->work_per_iter;
            unsigned int b = a;
            while (b > 0) {
                const job *p = idle[b - 1];
                const double rp = (double) (p->total_iters - p->done_iters) * p->work_per_iter;
                if (rp < rk || (rp == rk && p->id < k->id))
                    break;
                idle[b] = idle[b - 1];
                b--;
            }
            idle[b] = k;
        }
        /* the idle pooled SIRT jobs advance together: one quantum of the
         * mixed batch, counted as one job in flight */
        {
            job *pool_now[1024];
            unsigned int n_pool_now = 0, n_rest = 0;
            for (unsigned int i = 0; i < n_idle; i++) {
                if (idle[i]->pooled && !s->pool_off)
                    pool_now[n_pool_now++] = idle[i];
                else
                    idle[n_rest++] = idle[i];
            }
            n_idle = n_rest;
            if (n_pool_now > 0 && running < max_running) {
                const int rc = pool_quantum(s, pool_now, n_pool_now);
                if (rc != UFOIR_OK) {
                    /* no batch: these jobs go on with their own graphs */
                    s->pool_off = 1;
                    for (unsigned int i = 0; i < n_pool_now; i++)
                        idle[n_idle++] = pool_now[i];
                } else {
                    running++;
                }
                progressed = 1;
            } else {
                for (unsigned int i = 0; i < n_pool_now; i++)
                    idle[n_idle++] = pool_now[i];
            }
        }
        for (unsigned int i = 0; i < n_idle && running < max_running; i++) {
            job *j = idle[i];
            if (j->pooled && !s->pool_off)
                continue;      /* waits for the pool's next quantum */
            const int rc = job_quantum(s, j);
            if (rc != UFOIR_OK) {
                j->phase = PH_END;
                job_finish(s, j, rc);
            } else {
                j->busy = 1;
                running++;
            }
            progressed = 1;
        }
        udev_use_stream(s->ctx->dev, NULL);
        if (!progressed)
            usleep(20);
    }
    return NULL;
}

/* ------------------------------------------------------------------ API */

int ufoir_serve_create(ufoir_ctx *ctx, const ufoir_serve_config *cfg, ufoir_server **out)
{
    if (!ctx || !out)
        return UFOIR_ERR_INVALID;
    *out = NULL;
    ufoir_server *s = (ufoir_server *) calloc(1, sizeof(*s));
    if (!s)
        return ufoir__fail(ctx, UFOIR_ERR_NOMEM, "out of host memory");
    if (cfg)
        s->cfg = *cfg;
    else
        ufoir_serve_config_init(&s->cfg);
    if (s->cfg.policy != UFOIR_SERVE_CONTINUOUS && s->cfg.policy != UFOIR_SERVE_ONE_AT_A_TIME &&
        s->cfg.policy != UFOIR_SERVE_SJF_ONE_AT_A_TIME) {
        free(s);
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "unknown serve policy %d", cfg->policy);
    }
    if (s->cfg.hbm_budget_bytes == 0)
        s->cfg.hbm_budget_bytes = ctx->hbm_budget;
    if (s->cfg.max_active_jobs == 0)
        s->cfg.max_active_jobs = DEFAULT_MAX_ACTIVE;
    if (s->cfg.max_active_jobs > 1024)
        s->cfg.max_active_jobs = 1024;
    s->user_ctx = ctx;
    int rc = ufoir_ctx_create(udev_device(ctx->dev), s->cfg.hbm_budget_bytes, &s->ctx);
    /* jobs rarely share a geometry: no launch-shape search inside a job's latency */
    if (rc == UFOIR_OK)
        rc = ufoir_ctx_set_autotune(s->ctx, UFOIR_AUTOTUNE_OFF);
    if (rc) {
        free(s);
        return ufoir__fail(ctx, rc, "serve: private context: %s", ufoir_last_error(NULL));
    }
    s->active = (job **) calloc(s->cfg.max_active_jobs, sizeof(job *));
    if (!s->active) {
        ufoir_ctx_destroy(s->ctx);
        free(s);
        return ufoir__fail(ctx, UFOIR_ERR_NOMEM, "out of host memory");
    }
    pthread_mutex_init(&s->mu, NULL);
    pthread_cond_init(&s->cv_work, NULL);
    pthread_cond_init(&s->cv_done, NULL);
    if (pthread_create(&s->worker, NULL, worker_main, s) != 0) {
        ufoir_ctx_destroy(s->ctx);
        free(s->active);
        free(s);
        return ufoir__fail(ctx, UFOIR_ERR_STATE, "serve: cannot start the worker thread");
    }
    s->worker_started = 1;
    *out = s;
    return UFOIR_OK;
}

static job *find_job(ufoir_server *s, uint64_t id)
{
    if (id == 0 || id > s->n_jobs)
        return NULL;
    return s->jobs[id - 1];
}

int ufoir_serve_submit(ufoir_server *s, const ufoir_job_desc *jd, const float *sino, float *vol, uint64_t *job_id)
{
    if (!s || !jd || !sino || !vol)
        return UFOIR_ERR_INVALID;
    int rc = check_desc(s->user_ctx, jd);
    if (rc)
        return rc;
    job *j = (job *) calloc(1, sizeof(*j));
    if (!j)
        return ufoir__fail(s->user_ctx, UFOIR_ERR_NOMEM, "out of host memory");
    j->d = *jd;
    j->user_sino = sino;
    j->user_vol = vol;
    j->bytes = job_bytes(jd);
    j->work_per_iter = job_work_per_iter(jd);
    j->total_work_iters = jd->method == UFOIR_METHOD_ASDPOCS ? jd->asdpocs.num_iterations : jd->sart.num_iterations;
    pthread_mutex_lock(&s->mu);
    if (s->stop) {
        pthread_mutex_unlock(&s->mu);
        free(j);
        return ufoir__fail(s->user_ctx, UFOIR_ERR_STATE, "serve: server is shutting down");
    }
    if (s->n_jobs == s->cap_jobs) {
        const size_t cap = s->cap_jobs ? 2 * s->cap_jobs : 256;
        job **a = (job **) realloc(s->jobs, cap * sizeof(job *));
        if (!a) {
            pthread_mutex_unlock(&s->mu);
            free(j);
            return ufoir__fail(s->user_ctx, UFOIR_ERR_NOMEM, "out of host memory");
        }
        s->jobs = a;
        s->cap_jobs = cap;
    }
    j->id = (uint64_t) s->n_jobs + 1;
    s->jobs[s->n_jobs++] = j;
    j->t_submit = now_s();
    if (s->submitted == 0)
        s->first_submit = j->t_submit;
    s->submitted++;
    if (job_id)
        *job_id = j->id;
    if (j->bytes > s->cfg.hbm_budget_bytes) {
        j->state = UFOIR_JOB_FAILED;
        j->status = UFOIR_ERR_BUDGET;
        j->t_end = j->t_submit;
        s->rejected++;
        pthread_cond_broadcast(&s->cv_done);
        pthread_mutex_unlock(&s->mu);
        return ufoir__fail(s->user_ctx, UFOIR_ERR_BUDGET, "job needs %zu bytes, budget is %llu", j->bytes,
                           (unsigned long long) s->cfg.hbm_budget_bytes);
    }
    j->state = UFOIR_JOB_QUEUED;
    if (s->pend_tail)
        s->pend_tail->next = j;
    else
        s->pend_head = j;
    s->pend_tail = j;
    pthread_cond_signal(&s->cv_work);
    pthread_mutex_unlock(&s->mu);
    return UFOIR_OK;
}

int ufoir_serve_poll(ufoir_server *s, uint64_t id, int *state)
{
    if (!s || !state)
        return UFOIR_ERR_INVALID;
    pthread_mutex_lock(&s->mu);
    job *j = find_job(s, id);
    int rc = UFOIR_OK;
    if (!j)
        rc = UFOIR_ERR_NOT_FOUND;
    else
        *state = j->state;
    pthread_mutex_unlock(&s->mu);
    return rc;
}

static int finished(const job *j)
{
    return j->state == UFOIR_JOB_DONE || j->state == UFOIR_JOB_FAILED || j->state == UFOIR_JOB_CANCELLED;
}

static void deadline_in(struct timespec *ts, int timeout_ms)
{
    clock_gettime(CLOCK_REALTIME, ts);
    ts->tv_sec += timeout_ms / 1000;
    ts->tv_nsec += (long) (timeout_ms % 1000) * 1000000L;
    if (ts->tv_nsec >= 1000000000L) {
        ts->tv_sec++;
        ts->tv_nsec -= 1000000000L;
    }
}

int ufoir_serve_wait(ufoir_server *s, uint64_t id, int timeout_ms)
{
    if (!s)
        return UFOIR_ERR_INVALID;
    struct timespec ts;
    if (timeout_ms >= 0)
        deadline_in(&ts, timeout_ms);
    pthread_mutex_lock(&s->mu);
    job *j = find_job(s, id);
    if (!j) {
        pthread_mutex_unlock(&s->mu);
        return UFOIR_ERR_NOT_FOUND;
    }
    while (!finished(j)) {
        const int e = timeout_ms >= 0 ? pthread_cond_timedwait(&s->cv_done, &s->mu, &ts)
                                      : pthread_cond_wait(&s->cv_done, &s->mu);
        if (e == ETIMEDOUT && !finished(j)) {
            pthread_mutex_unlock(&s->mu);
            return UFOIR_ERR_TIMEOUT;
        }
    }
    const int rc = j->state == UFOIR_JOB_CANCELLED ? UFOIR_ERR_CANCELLED : j->status;
    pthread_mutex_unlock(&s->mu);
    return rc;
}

int ufoir_serve_cancel(ufoir_server *s, uint64_t id)
{
    if (!s)
        return UFOIR_ERR_INVALID;
    pthread_mutex_lock(&s->mu);
    job *j = find_job(s, id);
    int rc = UFOIR_OK;
    if (!j) {
        rc = UFOIR_ERR_NOT_FOUND;
    } else if (j->state != UFOIR_JOB_QUEUED) {
        rc = UFOIR_ERR_STATE;
    } else {
        job **pp = &s->pend_head;
        job *prev = NULL;
        while (*pp && *pp != j) {
            prev = *pp;
            pp = &(*pp)->next;
        }
        if (*pp) {
            *pp = j->next;
            if (s->pend_tail == j)
                s->pend_tail = prev;
        }
        j->next = NULL;
        j->state = UFOIR_JOB_CANCELLED;
        j->status = UFOIR_ERR_CANCELLED;
        j->t_end = now_s();
        s->cancelled++;
        pthread_cond_broadcast(&s->cv_done);
    }
    pthread_mutex_unlock(&s->mu);
    return rc;
}

int ufoir_serve_drain(ufoir_server *s, int timeout_ms)
{
    if (!s)
        return UFOIR_ERR_INVALID;
    struct timespec ts;
    if (timeout_ms >= 0)
        deadline_in(&ts, timeout_ms);
    pthread_mutex_lock(&s->mu);
    for (;;) {
        int open = s->pend_head != NULL || s->n_active > 0;
        if (!open)
            break;
        const int e = timeout_ms >= 0 ? pthread_cond_timedwait(&s->cv_done, &s->mu, &ts)
                                      : pthread_cond_wait(&s->cv_done, &s->mu);
        if (e == ETIMEDOUT && (s->pend_head || s->n_active > 0)) {
            pthread_mutex_unlock(&s->mu);
            return UFOIR_ERR_TIMEOUT;
        }
    }
    pthread_mutex_unlock(&s->mu);
    return UFOIR_OK;
}

static int cmp_double(const void *a, const void *b)
{
    const double x = *(const double *) a, y = *(const double *) b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

static double percentile(double *sorted, size_t n, double q)
{
    if (n == 0)
        return 0.0;
    double pos = q * (double) (n - 1);
    size_t i = (size_t) pos;
    double f = pos - (double) i;
    if (i + 1 >= n)
        return sorted[n - 1];
    return sorted[i] * (1.0 - f) + sorted[i + 1] * f;
}

int ufoir_serve_get_stats(ufoir_server *s, ufoir_serve_stats *o)
{
    if (!s || !o)
        return UFOIR_ERR_INVALID;
    memset(o, 0, sizeof(*o));
    pthread_mutex_lock(&s->mu);
    o->submitted = s->submitted;
    o->completed = s->completed;
    o->failed = s->failed;
    o->cancelled = s->cancelled;
    o->rejected = s->rejected;
    o->peak_hbm_bytes = s->peak_reserved;
    o->peak_active_jobs = s->peak_active;
    o->batched_iterations = s->pool_quanta;
    const size_t n = s->n_lat;
    double *l = n ? (double *) malloc(n * sizeof(double)) : NULL;
    double *q = n ? (double *) malloc(n * sizeof(double)) : NULL;
    if (n && l && q) {
        memcpy(l, s->lat, n * sizeof(double));
        memcpy(q, s->qlat, n * sizeof(double));
    }
    const double span = s->last_done > s->first_submit ? s->last_done - s->first_submit : 0.0;
    pthread_mutex_unlock(&s->mu);
    if (n && l && q) {
        qsort(l, n, sizeof(double), cmp_double);
        qsort(q, n, sizeof(double), cmp_double);
        double sum = 0;
        for (size_t i = 0; i < n; i++)
            sum += l[i];
        o->p50_latency_ms = percentile(l, n, 0.50);
        o->p99_latency_ms = percentile(l, n, 0.99);
        o->mean_latency_ms = sum / (double) n;
        o->max_latency_ms = l[n - 1];
        o->p50_queue_ms = percentile(q, n, 0.50);
        o->p99_queue_ms = percentile(q, n, 0.99);
    }
    free(l);
    free(q);
    o->busy_seconds = span;
    o->throughput_jobs_per_s = span > 0 ? (double) o->completed / span : 0.0;
    return UFOIR_OK;
}

void ufoir_serve_destroy(ufoir_server *s)
{
    if (!s)
        return;
    pthread_mutex_lock(&s->mu);
    s->stop = 1;
    for (job *j = s->pend_head; j; j = j->next) {
        j->state = UFOIR_JOB_CANCELLED;
        j->status = UFOIR_ERR_CANCELLED;
        s->cancelled++;
    }
    s->pend_head = s->pend_tail = NULL;
    pthread_cond_broadcast(&s->cv_work);
    pthread_cond_broadcast(&s->cv_done);
    pthread_mutex_unlock(&s->mu);
    if (s->worker_started)
        pthread_join(s->worker, NULL);
    if (s->pool_stream) {
        udev_use_stream(s->ctx->dev, s->pool_stream);
        ufoir_batch_destroy(s->pool);
        udev_use_stream(s->ctx->dev, NULL);
        udev_stream_destroy(s->ctx->dev, s->pool_stream);
    }
    free(s->pool_ids);
    for (size_t i = 0; i < s->n_jobs; i++)
        free(s->jobs[i]);
    free(s->jobs);
    free(s->active);
    free(s->lat);
    free(s->qlat);
    ufoir_ctx_destroy(s->ctx);
    pthread_mutex_destroy(&s->mu);
    pthread_cond_destroy(&s->cv_work);
    pthread_cond_destroy(&s->cv_done);
    free(s);
}
