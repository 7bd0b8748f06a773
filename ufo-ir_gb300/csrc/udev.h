/*
 * udev.h - thin C ABI between the C host library and the CUDA layer.
 *
 * The host code (geometry, projector, methods, serve loop; all C) never
 * includes CUDA headers: it allocates, copies, launches and captures graphs
 * through these functions, implemented in the .cu files of this directory.
 * Every function returns 0 or a negative ufoir_status and records a message
 * retrievable with udev_error().
 */
#ifndef UFOIR_UDEV_H
#define UFOIR_UDEV_H

#include <stddef.h>
#include <stdint.h>

#include "ufoir.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct udev udev;

int udev_create(int device, udev **out, char *err, size_t errlen);
void udev_destroy(udev *d);
const char *udev_error(const udev *d);
void udev_set_error(udev *d, const char *fmt, ...);
int udev_device(const udev *d);
int udev_sync(udev *d);
void *udev_stream(udev *d);
uint64_t udev_launches(const udev *d);
int udev_mem_info(udev *d, size_t *free_bytes, size_t *total_bytes);
int udev_sm_count(const udev *d);

int udev_malloc(udev *d, void **p, size_t bytes);           /* stream-ordered */
int udev_free(udev *d, void *p);
int udev_host_malloc(udev *d, void **p, size_t bytes);      /* page-locked */
int udev_host_free(udev *d, void *p);
/* 1 if p is device memory of this context's GPU, 0 if host memory. */
int udev_is_device_ptr(udev *d, const void *p);
int udev_memcpy_async(udev *d, void *dst, const void *src, size_t bytes);
int udev_memcpy(udev *d, void *dst, const void *src, size_t bytes);   /* + stream sync */
/* Copies on the context's side stream, overlapping the current stream's work:
 * udev_copy_after starts a copy once everything enqueued on the current
 * stream so far has run; udev_copy_join makes the current stream wait for
 * every side copy issued so far. Not for use while the current stream is
 * being captured. */
int udev_copy_after(udev *d, void *dst, const void *src, size_t bytes);
int udev_copy_join(udev *d);
/* Finer control of the same side stream: udev_side_fence orders it after
 * everything enqueued on the current stream so far; udev_side_copy issues a
 * copy there with no new ordering and marks its end in event `slot`
 * (0 <= slot < UDEV_SIDE_SLOTS); udev_side_wait makes the current stream wait
 * for that mark. */
#define UDEV_SIDE_SLOTS 8
int udev_side_fence(udev *d);
int udev_side_copy(udev *d, void *dst, const void *src, size_t bytes, int slot);
int udev_side_wait(udev *d, int slot);

/* ---- Device-side projection geometry (built by the host from the LUT). ---- */
typedef struct {
    int n_dets;                    /* detector count = volume side */
    int n_angles;
    float axis;                    /* resolved axis position */
    const float *d_sin;            /* [n_angles] float LUT */
    const float *d_cos;
    const unsigned char *d_dir;    /* [n_angles] direction of each angle (full subsets) */
    int fast_arith;                /* 1: the tiled projectors' fast interpolation (not the reference's rounding) */
} udev_geom;

/* Forward projection of angles [a0, a0 + na) for n_slices slices:
 *   out = (src + scale * S) [* w]        (S = Joseph ray sum, 64-sample blocks)
 * Inactive detectors (axis off-centre) give out = src [* w].
 * dir_override < 0 uses the per-angle direction, else forces it.
 * vol is [n][n] per slice; volT its transpose, read by horizontal rays (if
 * NULL they read vol column-wise instead). src/out/w are full sinograms
 * [n_angles][n] per slice; src may equal out; w may be NULL; w_shared != 0
 * means one w for all slices. */
int udev_fp(udev *d, const udev_geom *g, int a0, int na, int dir_override,
            const float *vol, const float *volT, const float *src, const float *w,
            int w_shared, float *out, float scale, int n_slices);

/* Transpose n x n slices. */
int udev_transpose(udev *d, const float *in, float *out, int n, int n_slices);

/* Interpolated samples/s of the forward projector's per-sample sequence run
 * from shared memory on every SM with no global traffic (udev_ceiling.cu). */
int udev_sample_ceiling(udev *d, double *samples_per_s);
/* The same for the backprojector's per-sample sequence. */
int udev_sample_ceiling_bp(udev *d, double *samples_per_s);

/* ---- Per-angle projections of a SART sweep (udev_sart.cu) ---- */
/* Floats of the block-start table: the coordinate of every ray of every
 * angle at the start of each 64-sample block, [n_angles][ceil(n/64)][n]. */
size_t udev_fp_block_starts_floats(int n, int n_angles);
int udev_fp_block_starts(udev *d, const udev_geom *g, float *table);
/* Forward projection of one angle, rays walking the rows of img (the volume
 * for vertical rays, dir 1; its transpose for horizontal rays, dir 0):
 *   out = (src + scale * S) [* w]  for the angle's row of the sinogram. */
int udev_fp_angle(udev *d, const udev_geom *g, int angle, int dir, const float *table, const float *img,
                  const float *src, const float *w, int w_shared, float *out, float scale, int n_slices);
/* vol = vol + relax * A_angle^T sino (one-angle subset), in place; with
 * transposed != 0, vol holds the transpose of the volume. sn, cs: the
 * angle's entries of the float LUT. relax_dev, if not NULL, replaces relax
 * with the value it points to when the kernel runs. */
int udev_bp_angle(udev *d, const udev_geom *g, int angle, float sn, float cs, const float *sino, float *vol,
                  int transposed, float relax, const float *relax_dev, int n_slices);
/* The padded sweep layout: two zero-padded copies of the volume, V (rows =
 * image rows) and H (the transpose), whole 64-row blocks high. The work
 * area (udev_sart_work_floats floats) must be zero-filled once. */
int udev_sart_pitch(int n);
size_t udev_sart_work_floats(int n, int n_slices);
/* 1 if the padded kernels serve this geometry (clamp edges e0 <= e1) for
 * n_slices slices on this GPU (a cluster of the forward projection fits). */
int udev_sart_padded(udev *d, const udev_geom *g, int n_slices);
/* Copies the volume between the user's slices (place -1), V (0) and H (1). */
int udev_sart_move(udev *d, int n, float *x, float *work, int from, int to, int n_slices);
/* udev_fp_angle and udev_bp_angle on the padded copy `place` (0 V for
 * vertical rays, 1 H for horizontal ones). */
int udev_sart_fp(udev *d, const udev_geom *g, int angle, int dir, const float *table, float *work, int place,
                 const float *src, const float *w, int w_shared, float *out, float scale, int n_slices);
int udev_sart_bp(udev *d, const udev_geom *g, int angle, float sn, float cs, const float *sino, float *work,
                 int place, float relax, const float *relax_dev, int n_slices);

/* ---- Tiled forward projector (all angles, shared-memory row streaming) ---- */
/* Row pitch (floats, multiple of 4) of the padded images: 2 zero columns,
 * n values, at least 2 zero columns. */
int udev_fp_pitch(int n);
/* Angles per CTA tile for n detectors; 0 if the tiled kernel cannot serve n. */
int udev_fp_tile_angles(udev *d, int n);
/* Writes the padded copy and the padded transpose of n_slices n x n images
 * into buffers of n * pitch floats per slice whose pad columns are zero. */
int udev_pad_transpose(udev *d, const float *vol, float *volP, float *volTP, int n, int n_slices);
/* Same contract as udev_fp over all angles, reading the padded images.
 * d_tiles: device array of int4 {first angle, count, direction, 0};
 * tile_spread: an upper bound, in columns, of how far the rays of one
 * detector at one row lie apart over the angles of a tile (computed by the
 * projector with its tiles), used to size the column windows of split tiles. */
int udev_fp_tiles(udev *d, const udev_geom *g, const void *d_tiles, int n_tiles, float tile_spread,
                  const float *volP, const float *volTP, const float *src, const float *w, int w_shared,
                  float *out, float scale, int n_slices);
/* Launch shape of the tiled forward projector. J detector pairs per thread
 * and angle slot, A angles per tile (the tile list must have been built with
 * A), win: detector-split CTAs stage column windows, K rows per chunk
 * (4, 8, 16 or 32), dsplit CTAs per tile; the rest is derived by
 * udev_fp_cfg_finish. Every shape gives the same results bit for bit: each
 * ray's arithmetic does not depend on which CTA or lane carries it. */
typedef struct {
    int J, A, win, K, dsplit;
    int threads, dper, wcols, wstride, margin;
    int fm;                        /* fast arithmetic (from the geometry) */
    size_t smem;
} udev_fp_cfg;
/* The fixed rules (what udev_fp_tiles uses) for n_tiles tiles of the
 * default angle count and n_slices slices. */
int udev_fp_default_cfg(udev *d, const udev_geom *g, int n_tiles, int n_slices, float tile_spread, udev_fp_cfg *c);
/* Fills the derived fields of a shape given J, A, win, K, dsplit;
 * UFOIR_ERR_UNSUPPORTED if no kernel or not enough shared memory serves it. */
int udev_fp_cfg_finish(udev *d, const udev_geom *g, float tile_spread, udev_fp_cfg *c);
/* udev_fp_tiles with an explicit shape. */
int udev_fp_tiles_cfg(udev *d, const udev_geom *g, const udev_fp_cfg *c, const void *d_tiles, int n_tiles,
                      const float *volP, const float *volTP, const float *src, const float *w, int w_shared,
                      float *out, float scale, int n_slices);

/* ---- Mixed batches: one launch per kernel over many one-slice jobs ----
 * Each job contributes an opaque record (built on the host by *_record,
 * copied to device memory by the caller) and `items` CTAs; item_start is
 * the exclusive prefix sum of the items (n_jobs entries, device memory),
 * job_index maps a record to its entry of the active array (device ints;
 * 0 = skip the job). */
size_t udev_fp_record_bytes(void);
/* 1 if a shape's shared memory leaves room for the batch kernel's record. */
int udev_fp_batch_fits(const udev *d, const udev_fp_cfg *c);
int udev_fp_record(udev *d, const udev_geom *g, const udev_fp_cfg *c, const void *d_tiles, int n_tiles,
                   const float *volP, const float *volTP, const float *src, const float *w, float *out,
                   float scale, void *record, int *items);
/* All records must share the launch shape's J, A, win, threads and smem. */
int udev_fp_batch(udev *d, const udev_fp_cfg *c, const void *d_records, const int *d_item_start, int n_jobs,
                  const int *d_job_index, const int *d_active, int n_items);
size_t udev_bp_record_bytes(void);
int udev_bp_record(udev *d, const udev_geom *g, const ufoir_subset *subsets, int n_subsets, const float *sino,
                   const float *base, const float *cw, const float *add, float *dst, float relax, void *record,
                   int *items);
int udev_bp_batch(udev *d, int fast_arith, const void *d_records, const int *d_item_start, int n_jobs,
                  const int *d_job_index, const int *d_active, int n_items);
size_t udev_pad_record_bytes(void);
int udev_pad_record(int n, const float *vol, float *volP, float *volTP, void *record, int *items);
int udev_pad_batch(udev *d, const void *d_records, const int *d_item_start, int n_jobs, const int *d_job_index,
                   const int *d_active, int n_items);

/* Backprojection with shared-memory sinogram windows (udev_bp uses it for
 * 16 or more angles); same contract as udev_bp, at most 16 subsets. */
int udev_bp_tiles(udev *d, const udev_geom *g, const ufoir_subset *subsets, int n_subsets,
                  const float *sino, const float *base, const float *cw, int cw_shared,
                  const float *add, float *dst, float relax, int n_slices);
int udev_memset(udev *d, void *p, int value, size_t bytes);
/* Returns UFOIR_ERR_TIMEOUT (and clears the word) if a kernel recorded a
 * bounded-wait timeout since the last check; waits for the stream. */
int udev_take_kernel_error(udev *d);
/* Testing: in the next tiled forward projection launch, the barrier of row
 * chunk `chunk` never completes in any CTA (-1 = none). */
void udev_inject_copy_skip(udev *d, int chunk);

/* The "siddon" model (udev_siddon.cu): exact line integrals of the pixel
 * image, bin k of angle theta being the line X cos - Y sin + axis = k + 0.5.
 * Forward over angles [a0, a0 + na): out = (src + scale * S) [* w] (src may
 * be NULL or equal out), reading the padded copy and padded transpose of
 * udev_pad_transpose (n <= 32768); backward: for each subset
 * v = v + relax * sum, with v starting from base (may alias dst) or 0; at
 * most 16 subsets. */
int udev_siddon_fp(udev *d, const udev_geom *g, int a0, int na, const float *volP, const float *volTP,
                   const float *src, const float *w, int w_shared, float *out, float scale, int n_slices);
int udev_siddon_bp(udev *d, const udev_geom *g, const ufoir_subset *subsets, int n_subsets,
                   const float *sino, const float *base, float *dst, float relax, int n_slices);

/* Pixel-driven backprojection over a list of subsets:
 *   v = base ? base : 0;  for each subset: v = v + relax * sum_{angles} lerp(sino)
 *   if cw: v = v * cw;  if add: v = v + add;  dst = v
 * base / add may alias dst; cw_shared != 0 means one cw for all slices. */
int udev_bp(udev *d, const udev_geom *g, const ufoir_subset *subsets, int n_subsets,
            const float *sino, const float *base, const float *cw, int cw_shared,
            const float *add, float *dst, float relax, int n_slices);

/* ---- Element-wise ops over n contiguous floats. ---- */
enum {
    UDEV_MUL = 0,        /* a * b */
    UDEV_ADD = 1,        /* a + b */
    UDEV_SUB = 2,        /* a - b */
    UDEV_SUB_SCALED = 3, /* a - m * b */
    UDEV_ADD_SCALED = 4, /* a + m * b */
    UDEV_MAX = 5,        /* fmax(a, b) */
    UDEV_DIV = 6         /* a / b */
};
enum {
    UDEV_INV = 0,        /* a != 0 ? 1 / a : 0 */
    UDEV_POSC = 1,       /* a > 0 ? a : 0 */
    UDEV_SQRT = 2,       /* sqrt(a) correctly rounded */
    UDEV_SCALE = 3,      /* a * m */
    UDEV_ADDC = 4,       /* m + a */
    UDEV_MAXC = 5,       /* fmax(a, m) */
    UDEV_NORMALIZE = 6   /* delta * a - lo * delta; m = delta, m2 = lo */
};
int udev_fill(udev *d, float *p, size_t n, float v);
int udev_binary(udev *d, int op, const float *a, const float *b, float m, float *out, size_t n);
int udev_unary(udev *d, int op, const float *a, float m, float m2, float *out, size_t n);

/* TV subgradient (l1_grad) of n_slices w x h images. */
int udev_l1_grad(udev *d, const float *in, float *out, int w, int h, int n_slices);
/* Periodic differences. */
enum { UDEV_DX = 0, UDEV_DXT = 1, UDEV_DY = 2, UDEV_DYT = 3 };
int udev_diff(udev *d, int which, const float *in, float *out, int w, int h, int n_slices);

/* ---- Reductions; one float per slice written to host memory. ---- */
/* sum |v| over each w*h slice, in the index order of ufo_ir_op_l1_norm. */
int udev_l1_norm(udev *d, const float *v, size_t w, size_t h, int n_slices, int mode,
                 float *host_out);
/* The same L1 norm into device memory (n_slices floats), with caller-owned
 * FP64 partials (udev_l1_partials(n_slices) doubles; unused in COMPAT
 * mode): no host synchronisation, capturable. */
size_t udev_l1_partials(int n_slices);
int udev_l1_norm_to(udev *d, const float *v, size_t w, size_t h, int n_slices, int mode, double *partials,
                    float *d_out);

/* ASD-POCS scalars in device memory (udev_asd.cu): beta, the SART
 * relaxation and the outer-iteration count, and per slice the norms dp, dd,
 * dg, l1 and the TV step dtgv. */
typedef struct {
    float *beta, *relax;
    int *it;
    float *dp, *dd, *dg, *dtgv, *l1;
} udev_asd_scalars;
int udev_asd_begin(udev *d, const udev_asd_scalars *S);
int udev_asd_init(udev *d, const udev_asd_scalars *S, float alpha, int n_slices);
int udev_asd_tv_step(udev *d, float *x, const float *grad, const udev_asd_scalars *S, size_t per_slice,
                     int n_slices);
int udev_asd_end(udev *d, const udev_asd_scalars *S, float beta_red, float r_max, float alpha_red, int n_slices);

/* buggy-index dot product of ufo_ir_basic_ops_processor_dot_product. */
int udev_dot(udev *d, const float *a, const float *b, size_t w, size_t h, int n_slices,
             int mode, float *host_out);
/* min and max of each slice (exact; order independent). */
int udev_minmax(udev *d, const float *v, size_t n, int n_slices, float *host_min, float *host_max);

/* ---- Streams and events for concurrent jobs ---- */
int udev_stream_create(udev *d, void **s);
void udev_stream_destroy(udev *d, void *s);
/* Route all later work of this context to stream s (NULL = the context's own). */
void udev_use_stream(udev *d, void *s);
int udev_event_create(udev *d, void **e);
void udev_event_destroy(void *e);
int udev_event_record(udev *d, void *e);   /* on the current stream */
/* 1 if the event's work has completed, 0 if not yet, < 0 on error. */
int udev_event_done(udev *d, void *e);

/* ---- Timing with CUDA events on the context's stream ---- */
int udev_timer_begin(udev *d);
int udev_timer_end(udev *d, float *ms);   /* waits for the stop event */

/* ---- CUDA graphs ---- */
int udev_capture_begin(udev *d);
/* Ends the capture and instantiates it. *kernels = kernel launches captured. */
int udev_capture_end(udev *d, void **exec, uint64_t *kernels);
int udev_graph_launch(udev *d, void *exec, uint64_t kernels);
void udev_graph_destroy(void *exec);

#ifdef __cplusplus
}
#endif
#endif
