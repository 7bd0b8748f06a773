/*
 * ufoir.h - C ABI of the GB300-native ufo-ir iterative-reconstruction path.
 *
 * The library (libufoir.so) replaces ufo-ir's OpenCL hot path: the
 * parallel-beam Joseph projector plugin and the SART / SIRT / ASD-POCS /
 * split-Bregman-TV method plugins built on it. Kernels are hand-written CUDA
 * for sm_103a; the host side is C. No OpenCL, no CPU fallback: every compute
 * entry point runs on the GPU or fails with a status code.
 *
 * Each entry point names the reference interface it replaces as
 * file:line within the ufo-ir source tree.
 *
 * Conventions
 *   - Every call returns 0 (UFOIR_OK) or a negative ufoir_status; the last
 *     error message of a context is available through ufoir_last_error().
 *     Nothing aborts the process and no device code traps.
 *   - Data are float32, row-major with x fastest, exactly as a UfoBuffer's
 *     host array: a sinogram is [n_angles][n_dets], a volume (the
 *     reconstruction grid) is [n_dets][n_dets] (the reference always
 *     reconstructs an n_dets x n_dets grid,
 *     src/tasks/ufo-ir-parallel-projector-task.c:339-346, :576-578).
 *     n_slices > 1 means that many independent slices stored back to back.
 *   - Data pointers may be host memory (pageable or pinned) or device memory
 *     of the context's GPU; the library detects which and stages host data
 *     through HBM itself. Device pointers keep the data resident.
 *   - Calls on one context are serialised on that context's CUDA stream and
 *     return after the result is complete (ufo-core's process() is synchronous).
 */
#ifndef UFOIR_H
#define UFOIR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define UFOIR_API __attribute__((visibility("default")))
#else
#define UFOIR_API
#endif

/* ------------------------------------------------------------------------ */
/* Status codes. The reference logs OpenCL errors and continues, and aborts */
/* on shape errors through g_error (src/core/ufo-ir-basic-ops.c:48, :222);  */
/* this ABI returns a status instead.                                        */
/* ------------------------------------------------------------------------ */
typedef enum {
    UFOIR_OK = 0,
    UFOIR_ERR_INVALID = -1,      /* bad argument, shape or parameter range */
    UFOIR_ERR_CUDA = -2,         /* CUDA runtime error (message has details) */
    UFOIR_ERR_NOMEM = -3,        /* device or host allocation failed */
    UFOIR_ERR_UNSUPPORTED = -4,  /* e.g. a projector model other than "joseph" */
    UFOIR_ERR_BUDGET = -5,       /* request larger than the HBM budget */
    UFOIR_ERR_TIMEOUT = -6,      /* a bounded wait ran out */
    UFOIR_ERR_CANCELLED = -7,    /* job cancelled */
    UFOIR_ERR_STATE = -8,        /* object used in the wrong state */
    UFOIR_ERR_NOT_FOUND = -9,    /* unknown job id */
    UFOIR_ERR_IO = -10           /* a file could not be read, parsed or written */
} ufoir_status;

/* ------------------------------------------------------------------------ */
/* Context: one GPU, one stream, a device memory pool. Replaces ufo-core's  */
/* UfoResources + UfoGpuNode command queue that the plugins borrow          */
/* (src/core/ufo-ir-method-task.c:235-238 declares UFO_TASK_MODE_GPU;      */
/* src/tasks/ufo-ir-sart-task.c:162 hands the node to the projector).       */
/* ------------------------------------------------------------------------ */
typedef struct ufoir_ctx ufoir_ctx;

/* Create a context on CUDA device `device`. hbm_budget_bytes caps what the
 * serve loop admits (0 = 90% of free memory at creation). */
UFOIR_API int ufoir_ctx_create(int device, uint64_t hbm_budget_bytes, ufoir_ctx **out);
UFOIR_API void ufoir_ctx_destroy(ufoir_ctx *ctx);
/* Message of the last failed call on this context ("" if none). */
UFOIR_API const char *ufoir_last_error(const ufoir_ctx *ctx);
UFOIR_API int ufoir_ctx_synchronize(ufoir_ctx *ctx);
/* The stream the context's work is queued on (a cudaStream_t, opaque). */
UFOIR_API void *ufoir_ctx_stream(ufoir_ctx *ctx);
/* Queue the context's work on the caller's stream from now on (NULL: back
 * to the context's own stream), so that the library's kernels are ordered
 * with the caller's own work without host synchronisation. The stream must
 * belong to the context's device and must not be capturing a graph while a
 * method runs (SIRT and SART capture their iterations themselves). Calls
 * that return host results still wait for this stream. Stands in for the
 * per-call stream argument of a stream-based interface; the reference has
 * one in-order OpenCL queue per node (src/tasks/ufo-ir-sart-task.c:162). */
UFOIR_API int ufoir_ctx_set_stream(ufoir_ctx *ctx, void *stream);
/* Device memory helpers (stream-ordered on the context's stream). */
UFOIR_API int ufoir_device_alloc(ufoir_ctx *ctx, size_t bytes, void **ptr);
UFOIR_API int ufoir_device_free(ufoir_ctx *ctx, void *ptr);
/* Page-locked host memory (for fast staging of host inputs/outputs). */
UFOIR_API int ufoir_host_alloc(ufoir_ctx *ctx, size_t bytes, void **ptr);
UFOIR_API int ufoir_host_free(ufoir_ctx *ctx, void *ptr);
/* Copy between any combination of host and device memory; synchronous. */
UFOIR_API int ufoir_memcpy(ufoir_ctx *ctx, void *dst, const void *src, size_t bytes);
/* Streaming multiprocessors of the context's GPU. */
UFOIR_API int ufoir_ctx_sm_count(const ufoir_ctx *ctx);
/* Number of kernels this library launched on the context so far. */
UFOIR_API uint64_t ufoir_ctx_kernel_launches(const ufoir_ctx *ctx);
/* CUDA-event timer on the context's stream: begin records a start event,
 * end records a stop event, waits for it and returns the elapsed device time. */
UFOIR_API int ufoir_ctx_timer_begin(ufoir_ctx *ctx);
/* Testing the device-side bounded waits (no reference counterpart; the
 * reference logs OpenCL errors and continues, src/core/ufo-ir-basic-ops.c:60-64):
 * in the next tiled forward projection launched on this context, the
 * shared-memory barrier of row chunk `chunk` expects 16 bytes more than the
 * chunk's bulk copy brings, in every CTA (-1 cancels), so it never completes.
 * Its waits then run out after their 250 ms limit, the kernel drains its
 * copies (all of which land), writes nothing and records the timeout, and the
 * call returns UFOIR_ERR_TIMEOUT; the context stays usable. One-shot. */
UFOIR_API int ufoir_ctx_inject_copy_timeout(ufoir_ctx *ctx, int chunk);
UFOIR_API int ufoir_ctx_timer_end(ufoir_ctx *ctx, float *ms);

/* ------------------------------------------------------------------------ */
/* Projector: the "parallel-projector" plugin (package "ir").                */
/* ------------------------------------------------------------------------ */

/* Direction of a run of angles; same values as UfoIrProjectionDirection
 * (src/tasks/ufo-ir-parallel-projector-task.h:37-40). */
enum { UFOIR_HORIZONTAL = 0, UFOIR_VERTICAL = 1 };

/* UfoIrProjectionsSubset (…parallel-projector-task.h:49-53). */
typedef struct {
    unsigned int offset;   /* first angle */
    unsigned int n;        /* number of angles */
    int direction;         /* UFOIR_HORIZONTAL (|sin| > |cos|) or UFOIR_VERTICAL */
} ufoir_subset;

/* Properties of the projector node, with the reference's names, ranges and
 * defaults (JSON keys in brackets):
 *   model            ["model"]            "joseph"      (…parallel-projector-task.c:123-128);
 *                                         also "siddon": exact line integrals of the
 *                                         pixel image and their adjoint (projector
 *                                         calls only; the methods need "joseph")
 *   angles_num       ["angles_num"]       0 = from input dims[1] (:132-137, :315-317)
 *   is_forward       ["is_forward"]       1             (src/core/ufo-ir-state-dependent-task.c:75-80)
 *   axis_position    ["axis_position"]    -1 = n_dets/2 (src/core/ufo-ir-projector-task.c:68-73)
 *   step             ["step"]             0 rad         (:75-80)
 *   relaxation       ["relaxation"]       1             (:82-87)
 *   correction_scale ["correction_scale"] 1             (:88-93) */
typedef struct {
    char model[32];
    unsigned int angles_num;
    int is_forward;
    float axis_position;
    float step;
    float relaxation;
    float correction_scale;
    int arithmetic;        /* extension, no reference counterpart: UFOIR_ARITH_EXACT (default) or
                              UFOIR_ARITH_FAST, see below ["arithmetic": "exact" | "fast"] */
} ufoir_projector_params;

/* Interpolation arithmetic of the tiled Joseph projectors (forward over many
 * angles, backprojection over 16 or more angles).
 * EXACT: every operation rounds as the reference's kernels do
 *        ((1 - t) T0 + t T1, products unfused), so results equal the
 *        reference's bit for bit.
 * FAST:  T0 + t (T1 - T0) with the product fused into the accumulation, and
 *        the backprojector's detector shift folded into its row terms: about
 *        a third fewer floating-point operations per sample. Results differ
 *        from the reference's in the last bits: relative L2 below 1e-5 after
 *        one projection and below 1e-4 after 100 SIRT iterations (the
 *        tolerance of this path), tested. The per-angle SART kernels and the
 *        few-angle kernels always compute exactly. */
enum { UFOIR_ARITH_EXACT = 0, UFOIR_ARITH_FAST = 1 };

typedef struct ufoir_projector ufoir_projector;

UFOIR_API void ufoir_projector_params_init(ufoir_projector_params *p);
/* ufo_ir_parallel_projector_task_new (…parallel-projector-task.c:79-82) + setup (:360-388).
 * Fails with UFOIR_ERR_UNSUPPORTED unless model is "joseph" or "siddon"
 * (case-insensitive, the reference lower-cases it, :283-287). The methods
 * (SART, SIRT, ASD-POCS, SBTV) fail with UFOIR_ERR_UNSUPPORTED on a
 * "siddon" projector. */
UFOIR_API int ufoir_projector_create(ufoir_ctx *ctx, const ufoir_projector_params *p,
                                     ufoir_projector **out);
UFOIR_API void ufoir_projector_destroy(ufoir_projector *proj);
/* GObject get/set of the properties above (…projector-task.c:212-259,
 * src/core/ufo-ir-projector-task.c:113-164). */
UFOIR_API int ufoir_projector_get_params(const ufoir_projector *proj, ufoir_projector_params *p);
UFOIR_API int ufoir_projector_set_params(ufoir_projector *proj, const ufoir_projector_params *p);

/* get_requisition (…parallel-projector-task.c:306-347): in_dims = {dims[0],
 * dims[1]} of the input buffer; (re)builds the sin/cos LUT and the direction
 * subsets when the angle count changes; out_dims = {n_dets, n_angles} when
 * is_forward, {n_dets, n_dets} otherwise. */
UFOIR_API int ufoir_projector_get_requisition(ufoir_projector *proj, const size_t in_dims[2],
                                              size_t out_dims[2]);
/* UfoTask process of the standalone node (src/core/ufo-ir-state-dependent-task.c:195-212):
 * zero the output, then forward (is_forward) or backward projection. */
UFOIR_API int ufoir_projector_process(ufoir_projector *proj, const float *in,
                                      const size_t in_dims[2], float *out, size_t n_slices);
/* Vtable forward/backward over the full direction subsets, accumulating
 * into the output (…parallel-projector-task.c:391-429):
 *   sino += correction_scale * A vol ;   vol += relaxation * A^T sino. */
UFOIR_API int ufoir_projector_forward(ufoir_projector *proj, const float *vol, float *sino,
                                      size_t n_dets, size_t n_angles, size_t n_slices);
UFOIR_API int ufoir_projector_backward(ufoir_projector *proj, float *vol, const float *sino,
                                       size_t n_dets, size_t n_angles, size_t n_slices);
/* ufo_ir_parallel_projector_subset_fp / _subset_bp (…parallel-projector-task.h:93-94,
 * .c:167-195): one subset, accumulating; the geometry must have been set by
 * a requisition or a forward/backward call. */
UFOIR_API int ufoir_projector_subset_fp(ufoir_projector *proj, const float *vol, float *sino,
                                        const ufoir_subset *subset);
UFOIR_API int ufoir_projector_subset_bp(ufoir_projector *proj, float *vol, const float *sino,
                                        const ufoir_subset *subset);
/* get_host_sin_vals / get_host_cos_vals (…parallel-projector-task.h:96-97);
 * NULL before the first requisition. */
UFOIR_API const float *ufoir_projector_get_host_sin_vals(const ufoir_projector *proj);
UFOIR_API const float *ufoir_projector_get_host_cos_vals(const ufoir_projector *proj);
/* The full direction-subset list (…parallel-projector-task.c:462-498). */
UFOIR_API int ufoir_projector_get_subsets(const ufoir_projector *proj, const ufoir_subset **subsets,
                                          unsigned int *count);

/* ------------------------------------------------------------------------ */
/* Methods (plugins "sart", "sirt", "asdpocs", "sbtv").                      */
/* Each *_process call is the method's UfoTask process: the sinogram(s) in, */
/* the n_dets x n_dets reconstruction(s) out, starting from x = 0 as the    */
/* reference does. The projector's geometry comes from the sinogram dims    */
/* (n_dets = dims[0], n_angles = angles_num or dims[1]) as in               */
/* src/core/ufo-ir-method-task.c:241-252. Methods leave the projector's     */
/* relaxation / correction_scale properties where the reference leaves them.*/
/* ------------------------------------------------------------------------ */

/* Norm arithmetic for the host-side reductions of ASD-POCS and SBTV.
 * COMPAT: float, sequential, in the reference's order (bit-identical to the
 *         reference's host loops; slow - one thread per sum).
 * FP64:   the same terms accumulated in double by a deterministic parallel
 *         reduction, rounded to float (default). */
enum { UFOIR_NORM_COMPAT = 0, UFOIR_NORM_FP64 = 1 };

/* "num-iterations" [1, MAX] default 10 (src/core/ufo-ir-method-task.c:75-80);
 * "relaxation_factor" [0, 1] default 0.25 (src/tasks/ufo-ir-sart-task.c:76-81,
 * src/tasks/ufo-ir-sirt-task.c:73-77). */
typedef struct {
    unsigned int num_iterations;
    float relaxation_factor;
} ufoir_sart_params;
typedef ufoir_sart_params ufoir_sirt_params;

/* src/tasks/ufo-ir-asdpocs-task.c:104-181. ng is accepted and ignored, as in
 * the reference (20 TV sub-steps are hard-coded at :573). df_minimizer holds
 * the nested SART node's properties. */
typedef struct {
    unsigned int num_iterations;   /* outer iterations, default 10 */
    float beta;                    /* [0, MAX] 1.0 */
    float beta_red;                /* [0, MAX] 0.995 */
    float alpha;                   /* [0, MAX] 0.2 */
    float alpha_red;               /* [0, MAX] 0.95 */
    float r_max;                   /* [0, MAX] 0.95 */
    unsigned int ng;               /* [0, 1000] 20 (unused) */
    int positive_constraint;       /* TRUE */
    ufoir_sart_params df_minimizer;
    int norm_mode;                 /* UFOIR_NORM_FP64 */
} ufoir_asdpocs_params;

/* src/tasks/ufo-ir-sbtv-task.c:90-116: lambda [0, MAX] 0.1, mu [0, MAX] 0.5. */
typedef struct {
    unsigned int num_iterations;
    float lambda;
    float mu;
    int norm_mode;                 /* UFOIR_NORM_FP64 */
} ufoir_sbtv_params;

UFOIR_API void ufoir_sart_params_init(ufoir_sart_params *p);
UFOIR_API void ufoir_sirt_params_init(ufoir_sirt_params *p);
UFOIR_API void ufoir_asdpocs_params_init(ufoir_asdpocs_params *p);
UFOIR_API void ufoir_sbtv_params_init(ufoir_sbtv_params *p);

/* SART: src/tasks/ufo-ir-sart-task.c:173-228. */
UFOIR_API int ufoir_sart_process(ufoir_projector *proj, const ufoir_sart_params *p,
                                 const float *sino, const size_t sino_dims[2], float *vol,
                                 size_t n_slices);
/* SIRT: src/tasks/ufo-ir-sirt-task.c:164-222. n_slices > 1 runs the batched
 * form: one FP and one BP launch per iteration for all slices, the whole
 * iteration loop captured in one CUDA graph. */
UFOIR_API int ufoir_sirt_process(ufoir_projector *proj, const ufoir_sirt_params *p,
                                 const float *sino, const size_t sino_dims[2], float *vol,
                                 size_t n_slices);
/* ASD-POCS: src/tasks/ufo-ir-asdpocs-task.c:411-580. */
UFOIR_API int ufoir_asdpocs_process(ufoir_projector *proj, const ufoir_asdpocs_params *p,
                                    const float *sino, const size_t sino_dims[2], float *vol,
                                    size_t n_slices);
/* ASD-POCS with its internal state returned, for inspection and tests. The
 * reference's output is copied before the TV stage of each outer iteration
 * (src/tasks/ufo-ir-asdpocs-task.c:468), so the TV steepest descent
 * (ufo_math_tvstd_method_process_real, :550-580, kernel l1_grad of
 * src/kernels/ufo-math-tvstd-method.cl:5-57) shows only in these locals of
 * process() (:411-509):
 *   x_tv     (may be NULL) n_slices volumes, host or device: x after the 20 TV
 *            sub-steps of the last outer iteration;
 *   scalars  (may be NULL) n_slices records: dp, dd, dg and dtgv as they
 *            stand when process() returns (dtgv after the :501-503 update).
 * vol and every other argument are as in ufoir_asdpocs_process. */
typedef struct {
    float dp, dd, dg, dtgv;
} ufoir_asdpocs_scalars;
UFOIR_API int ufoir_asdpocs_process_ex(ufoir_projector *proj, const ufoir_asdpocs_params *p,
                                       const float *sino, const size_t sino_dims[2], float *vol,
                                       size_t n_slices, float *x_tv, ufoir_asdpocs_scalars *scalars);
/* Split-Bregman TV: src/tasks/ufo-ir-sbtv-task.c:230-635. The reference
 * min-max-normalises its input sinogram in place (:239); this call leaves
 * the caller's sinogram untouched and works on a normalised copy. */
UFOIR_API int ufoir_sbtv_process(ufoir_projector *proj, const ufoir_sbtv_params *p,
                                 const float *sino, const size_t sino_dims[2], float *vol,
                                 size_t n_slices);

/* ------------------------------------------------------------------------ */
/* Resident batched SIRT: ufoir_sirt_process split into setup and replayed */
/* iterations, for many slices whose data stay in HBM. Creation computes   */
/* the weights (once, shared by all slices), zeroes the volumes and        */
/* captures one iteration                                                   */
/* (transpose + FP + BP launches over all slices) as a CUDA graph; run()    */
/* replays it. Results equal ufoir_sirt_process with the same iteration     */
/* count, bit for bit. No reference counterpart beyond sirt-task.c:164-222: */
/* it splits that process() into setup and iterations.                      */
/* ------------------------------------------------------------------------ */
typedef struct ufoir_sirt_batch ufoir_sirt_batch;

/* d_sino: n_slices sinograms in device memory; d_vol: n_slices output
 * volumes in device memory (zeroed here). Both must stay valid until destroy. */
UFOIR_API int ufoir_sirt_batch_create(ufoir_projector *proj, const ufoir_sirt_params *p,
                                      const float *d_sino, const size_t sino_dims[2], float *d_vol,
                                      size_t n_slices, ufoir_sirt_batch **out);
/* Advance every slice by `iterations` SIRT iterations (synchronous). */
UFOIR_API int ufoir_sirt_batch_run(ufoir_sirt_batch *b, unsigned int iterations);
/* Restart from x = 0. */
UFOIR_API int ufoir_sirt_batch_reset(ufoir_sirt_batch *b);
/* Run one iteration eagerly with CUDA events around each launch on the
 * context's stream; ms[0..2] = transpose, forward projection, backprojection
 * durations in milliseconds. The iteration counts toward the result. */
UFOIR_API int ufoir_sirt_batch_profile(ufoir_sirt_batch *b, float ms[3]);
UFOIR_API void ufoir_sirt_batch_destroy(ufoir_sirt_batch *b);

/* ------------------------------------------------------------------------ */
/* Autotuner of the tiled forward projector (no reference counterpart; the  */
/* reference's OpenCL launches use fixed work sizes,                        */
/* src/tasks/ufo-ir-parallel-projector-task.c:501-625). With autotune on, a */
/* context searches the forward projector's launch shapes (angles per tile, */
/* detector pairs per thread, rows per staged chunk, CTAs per tile, column  */
/* windows) the first time a method or batch meets a geometry (n_dets,      */
/* n_angles, step, axis) and slice count, timing each candidate with CUDA   */
/* events on scratch data, and keeps the fastest (the fixed rules unless a  */
/* shape is at least 2 % faster). Every shape computes each ray with the    */
/* same arithmetic, so results do not depend on the choice, bit for bit.    */
/* ------------------------------------------------------------------------ */
typedef struct {
    int J, A, win, K, dsplit, threads;   /* the chosen shape */
    int tuned;                           /* 1 if the search ran (or was cached), 0 = fixed rules */
    unsigned int candidates;             /* shapes timed */
    float ms_default, ms_tuned;          /* one forward projection, fixed rules vs chosen shape */
} ufoir_fp_tuning;

#define UFOIR_AUTOTUNE_OFF 0    /* the fixed rules everywhere */
#define UFOIR_AUTOTUNE_ON 1     /* search for every SIRT call and mixed batch */
#define UFOIR_AUTOTUNE_AUTO 2   /* (default) search for SIRT calls whose tiles cannot fill the GPU */
/* Sets the context's mode (UFOIR_AUTOTUNE_*). AUTO searches only where the
 * fixed rules would split each angle tile's detectors over several CTAs
 * (one slice, or few angles): there the rules were measured 11-32 % slower
 * than the best shape (one 1448^2 x 1200 slice 0.96 -> 0.85 ms per forward
 * projection, 2900^2 x 360 1.91 -> 1.37 ms). The search runs once per
 * geometry and slice count and context, in the call's set-up. Mixed batches
 * search only with ON; the serve loop never searches. */
UFOIR_API int ufoir_ctx_set_autotune(ufoir_ctx *ctx, int on);
/* Searches now for the projector's geometry (set by a requisition or a
 * forward/backward call) and n_slices slices, even with autotune off, and
 * reports the result; later calls on this projector with n_slices slices use
 * the chosen shape. */
UFOIR_API int ufoir_projector_autotune(ufoir_projector *proj, size_t n_slices, ufoir_fp_tuning *out);

/* ------------------------------------------------------------------------ */
/* Mixed SIRT batches: many one-slice SIRT jobs of different sizes and       */
/* angle counts advanced together. One iteration of every member is a fixed */
/* small set of launches captured in one CUDA graph: one padding launch for */
/* all members, one forward-projection launch per distinct launch shape (the */
/* autotuner's per geometry when the context's autotune is on), and one     */
/* backprojection launch for all members; each launch walks a work list of  */
/* (member, tile) items, biggest members first. Each member computes        */
/* exactly what ufoir_sirt_process computes for it alone, bit for bit. The  */
/* reference advances one slice per process() call                         */
/* (src/core/ufo-ir-method-task.c:221-252, src/tasks/ufo-ir-sirt-task.c:164-222). */
/* ------------------------------------------------------------------------ */
typedef struct {
    unsigned int n_dets, n_angles;    /* sinogram dims; the volume is n_dets x n_dets */
    float step;                       /* projector "step" (radians) */
    float axis_position;              /* projector "axis_position" (-1 = n_dets / 2) */
    float relaxation_factor;          /* SIRT "relaxation_factor" [0, 1] */
    const float *sino;                /* device memory, n_angles x n_dets */
    float *vol;                       /* device memory, n_dets x n_dets */
    int keep_vol;                     /* 0: start from x = 0 (as process() does); 1: from vol's content */
    int arithmetic;                   /* UFOIR_ARITH_EXACT (0) or UFOIR_ARITH_FAST */
} ufoir_batch_job;

typedef struct ufoir_batch ufoir_batch;

/* Members need n_angles >= 16 and an axis at least half a pixel inside the
 * image (the tiled projectors; others give UFOIR_ERR_UNSUPPORTED). sino and
 * vol must stay valid until destroy. With the context's autotune on, where a
 * tuned shape differs from the fixed rules' one, creation times the batch
 * both ways (one untimed and two timed iterations each, the members' volumes
 * saved before and restored after) and keeps the faster. */
UFOIR_API int ufoir_batch_create(ufoir_ctx *ctx, const ufoir_batch_job *jobs, size_t n_jobs, ufoir_batch **out);
/* Advances every active member by `iterations` SIRT iterations (synchronous). */
UFOIR_API int ufoir_batch_run(ufoir_batch *b, unsigned int iterations);
/* Freezes (0) or resumes (1) a member; frozen members are skipped by every
 * launch. All members start active. */
UFOIR_API int ufoir_batch_set_active(ufoir_batch *b, size_t member, int active);
/* Kernel launches of one batched iteration, and distinct forward shapes. */
UFOIR_API int ufoir_batch_launches(const ufoir_batch *b, unsigned int *launches, unsigned int *fp_shapes);
UFOIR_API void ufoir_batch_destroy(ufoir_batch *b);

/* ------------------------------------------------------------------------ */
/* Serving: a request loop over reconstruction jobs of mixed size, method   */
/* and iteration count. The reference processes one slice per process()    */
/* call on a ufo-core GPU node thread (src/core/ufo-ir-method-task.c:221-252) */
/* and has no serving mode; this is the continuous-batching counterpart of  */
/* calling ufoir_*_process once per job.                                    */
/*                                                                          */
/* A worker thread admits queued jobs while the HBM budget and the         */
/* active-job limit allow, keeps each admitted job's sinogram and iterate   */
/* resident on the device, and advances every active job a quantum at a    */
/* time on the job's own CUDA stream, so the work of different jobs         */
/* overlaps on the GPU and a job is admitted as soon as memory frees up.    */
/* Each job runs exactly the kernels of the plain call, so its result does  */
/* not depend on what else is in flight. Admission (CONTINUOUS) is in       */
/* arrival order, except that a job that does not fit the budget may be    */
/* passed by later jobs that do until it has waited admit_age_ms; quanta   */
/* go to the admitted jobs with the least remaining work. For comparison,  */
/* ONE_AT_A_TIME runs one job at a time in arrival order (the plain per-job */
/* path) and SJF_ONE_AT_A_TIME one job at a time, the queued job with the   */
/* least work first (the ordering of CONTINUOUS without its overlap).       */
/* ------------------------------------------------------------------------ */
/* Methods of a job or graph; the serve loop runs SART, SIRT and ASD-POCS. */
enum { UFOIR_METHOD_SART = 0, UFOIR_METHOD_SIRT = 1, UFOIR_METHOD_ASDPOCS = 2, UFOIR_METHOD_SBTV = 3 };
enum {
    UFOIR_JOB_QUEUED = 0,
    UFOIR_JOB_RUNNING = 1,
    UFOIR_JOB_DONE = 2,
    UFOIR_JOB_FAILED = 3,
    UFOIR_JOB_CANCELLED = 4
};
enum { UFOIR_SERVE_CONTINUOUS = 0, UFOIR_SERVE_ONE_AT_A_TIME = 1, UFOIR_SERVE_SJF_ONE_AT_A_TIME = 2 };

typedef struct {
    int method;                       /* UFOIR_METHOD_* */
    unsigned int n_dets;              /* sinogram dims[0]; volume n_dets x n_dets */
    unsigned int n_angles;            /* sinogram dims[1] */
    float step;                       /* projector "step" */
    float axis_position;              /* projector "axis_position" (-1 = centre) */
    ufoir_sart_params sart;           /* SART and SIRT: num-iterations, relaxation_factor */
    ufoir_asdpocs_params asdpocs;     /* ASD-POCS */
} ufoir_job_desc;

typedef struct {
    uint64_t hbm_budget_bytes;        /* 0 = the context's budget */
    unsigned int max_active_jobs;     /* jobs admitted (resident) at once; 0 = 32 */
    int policy;                       /* UFOIR_SERVE_* */
    unsigned int quantum;             /* SIRT iterations / SART sweeps per scheduling turn; 0 = 1 */
    unsigned int fail_allocation_every; /* testing: make every k-th job allocation fail (0 = off) */
    unsigned int max_running;         /* CONTINUOUS: jobs with work in flight at once, the ones
                                         with the least remaining work first; 0 = 4 */
    unsigned int admit_age_ms;        /* CONTINUOUS: how long a queued job that does not fit the
                                         budget may be passed by later jobs; 0 = 2000 */
    unsigned int batch_sirt;          /* CONTINUOUS: 1 = the SIRT jobs the tiled projectors serve
                                         advance together, one mixed batch (ufoir_batch) of the idle
                                         ones per quantum: more throughput for many small jobs, but a
                                         small job then waits for the biggest member's iteration every
                                         quantum; 0 (default) = each on its own graph */
} ufoir_serve_config;

typedef struct {
    uint64_t submitted, completed, failed, cancelled, rejected;
    double p50_latency_ms, p99_latency_ms, mean_latency_ms, max_latency_ms;
    double p50_queue_ms, p99_queue_ms;
    double throughput_jobs_per_s;     /* completed / (last completion - first submission) */
    double busy_seconds;              /* first submission to last completion */
    uint64_t peak_hbm_bytes;          /* largest sum of reserved job memory */
    unsigned int peak_active_jobs;
    uint64_t batched_iterations;      /* mixed-batch iterations issued (batch_sirt) */
} ufoir_serve_stats;

typedef struct ufoir_server ufoir_server;

UFOIR_API void ufoir_serve_config_init(ufoir_serve_config *c);
UFOIR_API void ufoir_job_desc_init(ufoir_job_desc *j);
/* The server works on its own stream(s) on ctx's device and owns a worker
 * thread; ctx must outlive it. */
UFOIR_API int ufoir_serve_create(ufoir_ctx *ctx, const ufoir_serve_config *cfg, ufoir_server **out);
/* Queue a job. sino (host memory, n_angles x n_dets floats) must stay valid
 * until the job is admitted; vol (host memory, n_dets x n_dets floats)
 * until it completes. Invalid parameters fail here (UFOIR_ERR_INVALID); a job
 * larger than the whole budget is refused (UFOIR_ERR_BUDGET). */
UFOIR_API int ufoir_serve_submit(ufoir_server *s, const ufoir_job_desc *job, const float *sino, float *vol,
                                 uint64_t *job_id);
UFOIR_API int ufoir_serve_poll(ufoir_server *s, uint64_t job_id, int *state);
/* Wait up to timeout_ms (< 0 = forever) for the job to finish. Returns the
 * job's own status (UFOIR_OK when done), UFOIR_ERR_CANCELLED, or
 * UFOIR_ERR_TIMEOUT if it is still queued or running. */
UFOIR_API int ufoir_serve_wait(ufoir_server *s, uint64_t job_id, int timeout_ms);
/* Cancel a job that is still queued (running jobs finish). */
UFOIR_API int ufoir_serve_cancel(ufoir_server *s, uint64_t job_id);
/* Wait until every submitted job has finished (or timeout_ms passes). */
UFOIR_API int ufoir_serve_drain(ufoir_server *s, int timeout_ms);
UFOIR_API int ufoir_serve_get_stats(ufoir_server *s, ufoir_serve_stats *out);
/* Cancels queued jobs, waits for running ones, stops the worker. */
UFOIR_API void ufoir_serve_destroy(ufoir_server *s);

/* ------------------------------------------------------------------------ */
/* Reductions used by the methods, exposed for callers and tests.           */
/* ufo_ir_op_l1_norm (src/core/ufo-ir-basic-ops.c:259-277) and              */
/* ufo_ir_basic_ops_processor_dot_product (src/core/ufo-ir-basic-ops-processor.c:148-196, */
/* including its index expression partNum * i at :189). w = dims[0],        */
/* h = dims[1]. Results are written to *out (host).                          */
/* ------------------------------------------------------------------------ */
UFOIR_API int ufoir_l1_norm(ufoir_ctx *ctx, const float *v, size_t w, size_t h, int norm_mode,
                            float *out);
UFOIR_API int ufoir_dot_product(ufoir_ctx *ctx, const float *a, const float *b, size_t w,
                                size_t h, int norm_mode, float *out);
/* The TV subgradient of ASD-POCS's steepest-descent stage: kernel l1_grad
 * (src/kernels/ufo-math-tvstd-method.cl:5-57, launched over (w, h) by
 * src/tasks/ufo-ir-asdpocs-task.c:563-571) on n_slices images of w x h
 * floats stored back to back: the 7-point stencil with EPS 1e-3 and a zero
 * border. v and out: host or device memory. */
UFOIR_API int ufoir_tv_gradient(ufoir_ctx *ctx, const float *v, size_t w, size_t h, size_t n_slices,
                                float *out);

/* Measurement (no counterpart in the reference): the interpolated-sample  */
/* rate ceiling of the device, i.e. the forward projector's exact per-      */
/* sample instruction sequence run from shared memory by every SM with no   */
/* global traffic. Projector sample rates are reported against it.          */
UFOIR_API int ufoir_sample_ceiling(ufoir_ctx *ctx, double *samples_per_s);
/* The same for the backprojector's per-sample sequence (per angle: the     */
/* angle record and row products from shared memory; per pixel pair: the   */
/* coordinate, floor, two window taps per pixel, filter and sum).          */
UFOIR_API int ufoir_sample_ceiling_bp(ufoir_ctx *ctx, double *samples_per_s);

/* ------------------------------------------------------------------------ */
/* Allocation-free L1 norm. No counterpart in the reference.                */
/*                                                                          */
/* For callers that must not allocate device memory where they need the    */
/* norm: code whose GPU memory belongs to another allocator (a host         */
/* framework's pooling allocator) or sits under a hard per-process limit    */
/* (an MPS client with a set memory limit), where a library must not grow   */
/* its own footprint, and loops that must not take the allocator's locks or */
/* the implicit synchronisation cudaMalloc/cudaFree can cause. It computes  */
/* what ufoir_l1_norm computes with UFOIR_NORM_FP64 (same result bit for    */
/* bit), for n_slices slices of `count` floats stored back to back, but     */
/* keeps its partial sums in a fixed device array inside the library       */
/* instead of allocating:                                                   */
/*   - the array holds UFOIR_NOALLOC_MAX_SLICES x 512 doubles (256 KiB) and  */
/*     every GPU that loads the library keeps it until the process exits;   */
/*   - n_slices > UFOIR_NOALLOC_MAX_SLICES is rejected with                 */
/*     UFOIR_ERR_INVALID and nothing is launched;                           */
/*   - the first call in a CUDA context (normally: the first call on a      */
/*     device) looks up the array's device address there with               */
/*     cudaGetSymbolAddress, with that context current, and caches it per   */
/*     context; make that first call before any stream capture. A device    */
/*     reset gives a new context, whose first call looks the address up     */
/*     again;                                                               */
/*   - all calls share the array, so calls whose work overlaps on the GPU   */
/*     (different streams without ordering between them) race and give      */
/*     wrong results; each call overwrites every partial it reads, so       */
/*     nothing needs clearing between calls.                                */
/* d_v (input) and d_out (n_slices floats, output) are device memory of the */
/* current device; the work is queued on `stream` (a cudaStream_t, NULL =   */
/* the default stream) and d_out is valid once the stream reaches it. No   */
/* cudaMalloc, cudaFree or allocating library call is made. The status is   */
/* this call's own: an error the caller left pending is not reported.       */
/* ------------------------------------------------------------------------ */
#define UFOIR_NOALLOC_MAX_SLICES 64
UFOIR_API int ufoir_l1_norm_fp64_noalloc(const float *d_v, size_t count, unsigned int n_slices,
                                         float *d_out, void *stream);

/* ------------------------------------------------------------------------ */
/* Graphs in ufo-core's JSON format (json-sample.json): a "read" node, one  */
/* ufo-ir method node of package "ir" (sart, sirt, asdpocs, sbtv) with its  */
/* "projector" object (and ASD-POCS's "df_minimizer" SART object), and a    */
/* "write" node, joined by edges read -> method -> write. Property names    */
/* follow GObject: '-' and '_' are the same character. Values are checked   */
/* against the property ranges above; an unknown property, plugin or        */
/* package is an error (UFOIR_ERR_INVALID / UFOIR_ERR_UNSUPPORTED), with a   */
/* message in err. Replaces ufo_plugin_manager + ufo_task_graph_read_from_  */
/* file for these nodes (ufo-core; the reference's graphs use it through    */
/* ufo-launch / ufo-runjson).                                              */
/* Extension (no counterpart in the reference): a method node may set      */
/* "norm-mode": "compat" | "fp64" for ASD-POCS and SBTV.                    */
/* ------------------------------------------------------------------------ */
#define UFOIR_PATH_MAX 1024
typedef struct {
    int method;                          /* UFOIR_METHOD_* */
    ufoir_projector_params projector;    /* the method's "projector" node */
    ufoir_sart_params sart;              /* SART / SIRT node */
    ufoir_asdpocs_params asdpocs;        /* ASD-POCS node (df_minimizer inside) */
    ufoir_sbtv_params sbtv;              /* SBTV node */
    char read_path[UFOIR_PATH_MAX];      /* "read": "path" (a file or a glob pattern); "" = none */
    unsigned int read_raw_width;         /* "read": "raw-width", "raw-height", "raw-offset" for  */
    unsigned int read_raw_height;        /*   raw float32 files (0 = the file is a TIFF)        */
    uint64_t read_raw_offset;
    char write_filename[UFOIR_PATH_MAX]; /* "write": "filename" (printf counter, e.g. out%03i.tif); "" = none */
} ufoir_graph;

UFOIR_API int ufoir_graph_parse(const char *json, size_t len, ufoir_graph *out, char *err, size_t errlen);
UFOIR_API int ufoir_graph_load(const char *path, ufoir_graph *out, char *err, size_t errlen);
/* The job description of a graph's method node for a sinogram of n_dets x
 * n_angles (SART, SIRT, ASD-POCS; SBTV gives UFOIR_ERR_UNSUPPORTED). */
UFOIR_API int ufoir_graph_job_desc(const ufoir_graph *g, unsigned int n_dets, unsigned int n_angles,
                                   ufoir_job_desc *out);
/* Runs a graph: reads every sinogram slice of read_path (TIFF pages, or raw
 * float32 slices of raw-width x raw-height), reconstructs them with the
 * method node, and writes the volumes to write_filename: one file per slice
 * when it holds a printf counter (counter from 0), else one multi-page TIFF.
 * *n_slices (may be NULL) receives the number of slices written. */
UFOIR_API int ufoir_graph_run(ufoir_ctx *ctx, const ufoir_graph *g, unsigned int *n_slices);

/* ------------------------------------------------------------------------ */
/* Slice files at the graph's edges (the reference's graphs use ufo-filters' */
/* read/write plugins): classic TIFF with 32-bit float, 16-bit or 8-bit      */
/* unsigned samples, one sample per pixel, uncompressed strips, either byte  */
/* order (read; written little-endian float32), one slice per page; raw      */
/* float32 in host byte order. Errors return UFOIR_ERR_IO (or _INVALID) with */
/* a message in ufoir_io_last_error() (per thread).                          */
/* ------------------------------------------------------------------------ */
UFOIR_API const char *ufoir_io_last_error(void);
UFOIR_API int ufoir_io_tiff_info(const char *path, unsigned int *width, unsigned int *height, unsigned int *pages);
UFOIR_API int ufoir_io_read_tiff(const char *path, unsigned int page, float *out, size_t count);
UFOIR_API int ufoir_io_write_tiff(const char *path, const float *data, unsigned int width, unsigned int height,
                                  unsigned int pages);
UFOIR_API int ufoir_io_read_raw(const char *path, uint64_t offset, float *out, size_t count);
UFOIR_API int ufoir_io_write_raw(const char *path, const float *data, size_t count);

#ifdef __cplusplus
}
#endif
#endif
