/*
 * host.h - private declarations of the C host library.
 */
#ifndef UFOIR_HOST_H
#define UFOIR_HOST_H

#include <stddef.h>
#include <stdint.h>

#include "udev.h"
#include "ufoir.h"

struct ufoir__tune_entry;

struct ufoir_ctx {
    udev *dev;
    uint64_t hbm_budget;
    char create_err[256];
    int autotune;                       /* UFOIR_AUTOTUNE_*: forward-projector launch-shape search */
    struct ufoir__tune_entry *tune;     /* cache of searched shapes (autotune.c) */
    int n_tune, cap_tune;
};

struct ufoir_projector {
    ufoir_ctx *ctx;
    ufoir_projector_params prm;
    /* geometry built by the requisition (…parallel-projector-task.c:306-347) */
    int have_geometry;
    unsigned int n_dets;
    unsigned int n_angles;
    float lut_step;
    float *h_sin, *h_cos;
    unsigned char *h_dir;
    ufoir_subset *subsets;
    unsigned int n_subsets;
    float *d_sin, *d_cos;
    unsigned char *d_dir;
    unsigned int lut_cap;
    /* angle tiles of the tiled forward projector, one list per tile width
     * A = 1, 2, 4, 8 (slot 0..3; int4 each, device) */
    void *d_tiles[4];
    int n_tiles[4];
    int tiles_valid[4];
    float tiles_spread[4];      /* max over tiles of the angles' coordinate spread (columns) */
    /* launch shape chosen by the autotuner for fp_cfg_slices slices */
    int fp_cfg_valid;
    int fp_cfg_slices;
    udev_fp_cfg fp_cfg;
};

/* Scratch of the tiled forward projector: the padded copy and the padded
 * transpose of n_slices volumes (pad columns zero). */
typedef struct {
    float *P, *TP;
    size_t slices;
} ufoir_fp_scratch;

int ufoir__fp_scratch_alloc(ufoir_projector *p, ufoir_fp_scratch *s, size_t slices);
void ufoir__fp_scratch_free(ufoir_projector *p, ufoir_fp_scratch *s);
/* Forward projection of all angles: out = (src + scale * A vol) [* w]. */
int ufoir__fp_full(ufoir_projector *p, ufoir_fp_scratch *s, const float *vol, const float *src, const float *w,
                   int w_shared, float *out, float scale, int n_slices);
/* Ray weights R = inv(FP(1)) (ones: n*n floats of scratch) and pixel weights
 * C = inv(BP(1)) (ones: n_angles*n floats of scratch) for one slice. */
int ufoir__ray_weights(ufoir_projector *p, float *R, float *ones);
int ufoir__pixel_weights(ufoir_projector *p, float *C, float *ones);

/* One SIRT iteration over n_slices slices (captured into graphs by callers). */
typedef struct {
    ufoir_projector *p;
    udev_geom g;
    const float *b;
    float *x, *resid;
    ufoir_fp_scratch fs;
    const float *R, *C;
    float lambda;
    int n_slices;
} ufoir__sirt_iter;
int ufoir__sirt_body(void *arg);

/* One SART sweep (every angle in order) over n_slices slices. work holds the
 * padded copies of the volume in the layouts of the two direction runs (or,
 * for crossed clamp edges, its transpose); table holds the block-start
 * coordinates of the per-angle forward projection. */
typedef struct {
    ufoir_projector *p;
    udev_geom g;
    const float *b;
    float *x, *resid;
    const float *R;
    float lambda;
    int n_slices;
    float *work, *table;
    const float *relax_dev;     /* if not NULL, lambda is read from here */
} ufoir__sart_iter;
int ufoir__sart_body(void *arg);
/* The sweep's scratch (work, zero-filled, and table; the geometry must be prepared). */
int ufoir__sart_scratch_alloc(ufoir_projector *p, float **work, float **table, int n_slices);
size_t ufoir__sart_scratch_bytes(size_t n, size_t na, size_t n_slices);

/* ASD-POCS split into setup, one outer iteration and release, so that the
 * plain call and the serve loop run the same code. */
typedef struct {
    ufoir_projector *p;
    udev_geom g;
    ufoir_asdpocs_params prm;
    int S;
    size_t n, na, nv, ns;
    const float *b;
    float *out;
    float *x, *x_prev, *x_res, *b_res, *grad, *R;
    float *work, *table;                /* SART sweep scratch */
    ufoir_fp_scratch fs;
    float *scal;                        /* device scalar block (dsc points into it) */
    double *partials;                   /* FP64 norm partials of this state */
    udev_asd_scalars dsc;
    ufoir__sart_iter sweep;
    void *sart_exec, *post_exec;        /* graphs: one SART sweep; the rest of an outer iteration */
    uint64_t sart_kernels, post_kernels;
    float beta, sart_relax;             /* host copies of the float sequence, for the properties */
    unsigned int it;
} ufoir__asd_state;
int ufoir__asd_setup(ufoir__asd_state *s, ufoir_projector *proj, const ufoir_asdpocs_params *prm, const float *b,
                     float *out, int S);
int ufoir__asd_outer(ufoir__asd_state *s);
void ufoir__asd_release(ufoir__asd_state *s);
size_t ufoir__asd_bytes(size_t n, size_t na, size_t S);

/* The angle tiles of width A (1, 2, 4 or 8) of the prepared geometry,
 * built on first use (not inside a stream capture). */
int ufoir__projector_tiles(ufoir_projector *p, int A, const void **d_tiles, int *n_tiles, float *spread);
/* The launch shape of the tiled forward projector for n_slices slices: the
 * tuned one where the autotuner has searched this geometry and slice count
 * (its tiles are built then), else the fixed rules. UFOIR_ERR_UNSUPPORTED if
 * the tiled kernel cannot serve the size. */
int ufoir__fp_shape(ufoir_projector *p, int n_slices, udev_fp_cfg *c, const void **d_tiles, int *n_tiles);
/* Autotuner (autotune.c): searches the launch shapes for this geometry and
 * n_slices (once per context; cached) and records the fastest on the
 * projector. Must not run inside a stream capture. */
int ufoir__fp_tune(ufoir_projector *p, int n_slices, ufoir_fp_tuning *out);
/* Whether a SIRT call on n_slices slices should search first: always with
 * UFOIR_AUTOTUNE_ON, with UFOIR_AUTOTUNE_AUTO where the fixed rules would
 * split each angle tile's detectors over several CTAs (too few tiles to fill
 * the GPU, where the rules were measured 11-32 % off the best shape). */
int ufoir__fp_tune_wanted(ufoir_projector *p, int n_slices);
void ufoir__tune_free(ufoir_ctx *ctx);

/* A member of a mixed SIRT batch whose buffers its owner keeps (the serve
 * loop): prepared projector (tiles built), sinogram b, iterate x, weights R
 * and C, residual and padded-copy scratch (P, TP: zero pad columns), and the
 * slice count its forward launch shape is chosen for. */
typedef struct {
    ufoir_projector *p;
    const float *b;
    float *x, *R, *C, *resid, *P, *TP;
    float lambda;
    int shape_slices;
} ufoir__bmember;
/* Work lists and the captured iteration for these members (batch.c); the
 * batch owns none of the members' buffers. Not inside a stream capture. */
int ufoir__batch_build(ufoir_ctx *ctx, const ufoir__bmember *members, int n, ufoir_batch **out);
/* Enqueues `iterations` iterations of every active member on the current
 * stream, without waiting. */
int ufoir__batch_launch(ufoir_batch *b, unsigned int iterations);

/* The two launches of ufoir__fp_full, separately (for timing). */
int ufoir__fp_prepare(ufoir_projector *p, ufoir_fp_scratch *s, const float *vol, int n_slices);
int ufoir__fp_project(ufoir_projector *p, ufoir_fp_scratch *s, const float *vol, const float *src, const float *w,
                      int w_shared, float *out, float scale, int n_slices);

/* Error helpers: record a message on the context and return the status. */
int ufoir__fail(ufoir_ctx *ctx, int status, const char *fmt, ...);

#define UFOIR_TRY(expr)          \
    do {                         \
        rc = (expr);             \
        if (rc != UFOIR_OK)      \
            goto done;           \
    } while (0)

/* Resolves the geometry for a sinogram/volume input of dims in_dims, exactly
 * as get_requisition does, and uploads the LUT when it changes. */
int ufoir__projector_prepare(ufoir_projector *p, const size_t in_dims[2]);
/* Same, with explicit detector and angle counts (forward/backward calls). */
int ufoir__projector_prepare_na(ufoir_projector *p, unsigned int n_dets, unsigned int n_angles);
/* Device geometry descriptor for the kernels. */
void ufoir__projector_geom(const ufoir_projector *p, udev_geom *g);
/* Axis position with the -1 default resolved to n_dets / 2.0. */
float ufoir__axis(const ufoir_projector *p);

/* Host-or-device staging of a user buffer. */
typedef struct {
    float *dev;          /* device pointer used by kernels */
    float *user;         /* caller's pointer */
    size_t count;        /* floats */
    int owned;           /* 1 if dev was allocated here (user is host memory) */
} ufoir_buf;

int ufoir__buf_in(ufoir_ctx *ctx, ufoir_buf *b, const float *user, size_t count, int copy_in);
/* Copies back to the user (if host) when copy_out, and releases. */
int ufoir__buf_out(ufoir_ctx *ctx, ufoir_buf *b, int copy_out);
void ufoir__buf_release(ufoir_ctx *ctx, ufoir_buf *b);

int ufoir__alloc(ufoir_ctx *ctx, float **p, size_t count);
void ufoir__free(ufoir_ctx *ctx, void *p);

#endif
