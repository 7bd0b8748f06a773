/*
 * CPU oracle for the ufo-ir iterative-reconstruction path.
 *
 * TEST INFRASTRUCTURE ONLY. Nothing in the product library links or calls this
 * code; it is loaded by the tests, by __graft_entry__.smoke() and by the CPU
 * baseline leg of bench.py, always as the result compared with, never as the
 * thing measured.
 *
 * Contents:
 *   - a plain-C restatement of the reference's OpenCL kernels
 *     (src/kernels/projector-parallel-joseph.cl, ufo-ir-basic-ops.cl,
 *      ufo-math-tvstd-method.cl, ufo-ir-gradient-processor.cl) and of the
 *     OpenCL 1.2 image sampler they rely on (linear / nearest filtering,
 *     CLK_ADDRESS_CLAMP zero border, CLK_ADDRESS_CLAMP_TO_EDGE);
 *   - a plain-C restatement of the host logic: sin/cos LUT and direction
 *     subsets (src/tasks/ufo-ir-parallel-projector-task.c:437-498), the
 *     state-dependent forward/backward loops, SART, SIRT, ASD-POCS and
 *     split-Bregman TV (src/tasks/ufo-ir-{sart,sirt,asdpocs,sbtv}-task.c) and
 *     the host-side norms/element-wise ops (src/core/ufo-ir-basic-ops.c,
 *     src/core/ufo-ir-basic-ops-processor.c);
 *   - an FP64 twin of all of the above (suffix _d) that uses the same float
 *     sin/cos LUT, used to state the arithmetic error of every result.
 *
 * Every float routine follows the reference's operation order with IEEE
 * single precision and no contraction (built with -ffp-contract=off), so
 * results are deterministic on x86-64 and aarch64.
 *
 * Kernels are reached through a table (oracle_kernels) so the same host-loop
 * restatement can drive either this port or the reference's own kernel
 * sources compiled through the OpenCL-C shim (oracle/_ref, ref_kernels.cpp).
 */
#ifndef UFOIR_ORACLE_H
#define UFOIR_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Mirrors UfoIrGeometryDims (src/tasks/ufo-ir-parallel-projector-task.h:55-61). */
typedef struct {
    unsigned long height;
    unsigned long width;
    unsigned long n_dets;
    unsigned long n_angles;
} oracle_dims;

/* Mirrors UfoIrProjectionsSubset (…parallel-projector-task.h:49-53);
 * direction: 0 = Horizontal (|sin| > |cos|), 1 = Vertical. */
typedef struct {
    unsigned int offset;
    unsigned int n;
    int direction;
} oracle_subset;

/* One float image as the OpenCL kernels see it: row-major, x fastest. */
typedef struct {
    float *data;
    long width;
    long height;
} oracle_image;

/* Kernel table: one entry per reference OpenCL kernel on the path. Each call
 * runs the kernel's whole NDRange (global size = the reference host's). */
typedef struct {
    /* FP_hor / FP_vert (projector-parallel-joseph.cl:36-156); NDRange
     * (sino.width, part.n); launched by …parallel-projector-task.c:563-625. */
    void (*fp)(oracle_image vol, oracle_image sino, const float *sin_val,
               const float *cos_val, oracle_dims dims, float axis_pos,
               oracle_subset part, float correction_scale);
    /* BP (projector-parallel-joseph.cl:158-218); NDRange (vol.width,
     * vol.height); launched by …parallel-projector-task.c:501-560. */
    void (*bp)(oracle_image vol, oracle_image sino, float relax,
               const float *sin_val, const float *cos_val, oracle_dims dims,
               float axis_pos, oracle_subset part);
    void (*op_set)(oracle_image a, float value);                       /* ufo-ir-basic-ops.cl:4-16 */
    void (*op_inv)(oracle_image a);                                     /* :18-36 (in place) */
    void (*op_mul)(oracle_image a, oracle_image b, oracle_image out);   /* :38-58 */
    void (*op_add)(oracle_image a, oracle_image b, oracle_image out);   /* :60-80 */
    void (*op_deduction)(oracle_image a, oracle_image b, oracle_image out); /* :82-102 */
    void (*op_deduction2)(oracle_image a, oracle_image b, float m, oracle_image out); /* :104-125 */
    void (*op_add2)(oracle_image a, oracle_image b, float m, oracle_image out); /* :127-148 */
    void (*op_mul_rows)(oracle_image a, oracle_image b, oracle_image out,
                        unsigned int offset, unsigned int n);          /* :150-171 */
    void (*op_posc)(oracle_image a, oracle_image out);                  /* :255-273 */
    void (*l1_grad)(oracle_image in, oracle_image out);                 /* ufo-math-tvstd-method.cl:5-57 */
    void (*dx)(const float *in, float *out, long w, long h);            /* ufo-ir-gradient-processor.cl:1-11 */
    void (*dxt)(const float *in, float *out, long w, long h);           /* :13-24 */
    void (*dy)(const float *in, float *out, long w, long h);            /* :26-37 */
    void (*dyt)(const float *in, float *out, long w, long h);           /* :39-51 */
} oracle_kernels;

/* Kernel table of this C restatement. */
const oracle_kernels *oracle_port_kernels(void);

/* Number of OpenMP threads used by the NDRange loops (0 = OpenMP default). */
void oracle_set_threads(int n);
int oracle_get_threads(void);

/* ---------------------------------------------------------------------- */
/* Geometry (…parallel-projector-task.c:437-498, sart-task.c:230-248).      */
/* ---------------------------------------------------------------------- */

/* sin/cos LUT: angle_i = (float)(i * step), value = (float)sin((double)angle). */
void oracle_make_lut(unsigned int n_angles, float step, float *sin_out, float *cos_out);
/* Maximal runs of equal direction; returns the subset count. */
unsigned int oracle_make_full_subsets(const float *sin_val, const float *cos_val,
                                      unsigned int n_angles, oracle_subset *out);
/* One subset per angle (SART). */
void oracle_make_angle_subsets(const float *sin_val, const float *cos_val,
                               unsigned int n_angles, oracle_subset *out);

/* Projector state shared by the host loops (the projector object's properties). */
typedef struct {
    unsigned int n_dets;
    unsigned int n_angles;
    float step;
    float axis_position;      /* property value; < 0 means n_dets / 2 */
    float relaxation;         /* property, default 1 */
    float correction_scale;   /* property, default 1 */
} oracle_projector;

/* forward/backward over the full subsets (…parallel-projector-task.c:391-429),
 * accumulating into the output as the reference does (no zeroing). */
void oracle_forward(const oracle_kernels *k, const oracle_projector *p,
                    const float *vol, float *sino);
void oracle_backward(const oracle_kernels *k, const oracle_projector *p,
                     float *vol, const float *sino);
/* state-dependent process: zero the output, then forward or backward
 * (src/core/ufo-ir-state-dependent-task.c:195-212). */
void oracle_projector_process(const oracle_kernels *k, const oracle_projector *p,
                              int is_forward, const float *in, float *out);

/* ---------------------------------------------------------------------- */
/* Methods. sino is [n_angles][n_dets], vol is [n_dets][n_dets].           */
/* ---------------------------------------------------------------------- */

enum { ORACLE_NORM_COMPAT = 0, ORACLE_NORM_FP64 = 1 };

/* sart-task.c:173-228. Leaves p->relaxation / p->correction_scale as the
 * reference leaves the projector's properties. */
void oracle_sart(const oracle_kernels *k, oracle_projector *p, unsigned int iters,
                 float relaxation_factor, const float *sino, float *vol);
/* sirt-task.c:164-222. */
void oracle_sirt(const oracle_kernels *k, oracle_projector *p, unsigned int iters,
                 float relaxation_factor, const float *sino, float *vol);

/* SIRT split into its weight computation (sirt-task.c:176-193) and the
 * iteration loop (:201-215) continuing from vol; used to time one iteration. */
void oracle_sirt_weights(const oracle_kernels *k, oracle_projector *p, float *ray_weights,
                         float *pixel_weights);
void oracle_sirt_iterate(const oracle_kernels *k, oracle_projector *p, unsigned int iters,
                         float relaxation_factor, const float *sino, float *ray_weights,
                         float *pixel_weights, float *vol);

typedef struct {
    unsigned int num_iterations;   /* outer iterations, method-task default 10 */
    float beta, beta_red, alpha, alpha_red, r_max;
    unsigned int ng;               /* accepted, ignored (asdpocs-task.c:573 uses 20) */
    int positive_constraint;
    unsigned int sart_iterations;  /* df_minimizer num-iterations */
    float sart_relaxation;         /* df_minimizer relaxation_factor before the first
                                      outer iteration (kept when beta leaves [0, 1]) */
    int norm_mode;                 /* ORACLE_NORM_* */
} oracle_asdpocs_params;

/* asdpocs-task.c:411-580. If x_internal is non-NULL it receives the
 * post-TV iterate of the last outer iteration (the reference's x). */
void oracle_asdpocs(const oracle_kernels *k, oracle_projector *p,
                    const oracle_asdpocs_params *prm, const float *sino,
                    float *vol, float *x_internal);
/* The same, and scalars[0..3] receive the locals dp, dd, dg and dtgv of
 * process() as they stand at its return (asdpocs-task.c:411-509). */
void oracle_asdpocs_state(const oracle_kernels *k, oracle_projector *p,
                          const oracle_asdpocs_params *prm, const float *sino,
                          float *vol, float *x_internal, float scalars[4]);

typedef struct {
    unsigned int num_iterations;
    float lambda, mu;
    int norm_mode;
} oracle_sbtv_params;

/* sbtv-task.c:230-635. sino is normalised in place, as the reference does
 * with its input buffer (sbtv-task.c:239). */
void oracle_sbtv(const oracle_kernels *k, oracle_projector *p,
                 const oracle_sbtv_params *prm, float *sino, float *vol);

/* Host reductions (float sequential, as the reference). */
float oracle_l1_norm(const float *v, unsigned long w, unsigned long h);          /* basic-ops.c:259-277 */
float oracle_dot_product(const float *a, const float *b, unsigned long w, unsigned long h); /* basic-ops-processor.c:148-196 */
float oracle_l1_norm_fp64(const float *v, unsigned long w, unsigned long h);
float oracle_dot_product_fp64(const float *a, const float *b, unsigned long w, unsigned long h);

/* ---------------------------------------------------------------------- */
/* FP64 twin: same algorithms, double arithmetic, same float LUT.           */
/* ---------------------------------------------------------------------- */
void oracle_forward_d(const oracle_projector *p, const double *vol, double *sino);
void oracle_backward_d(const oracle_projector *p, double *vol, const double *sino);
void oracle_sirt_d(oracle_projector *p, unsigned int iters, float relaxation_factor,
                   const double *sino, double *vol);
void oracle_sart_d(oracle_projector *p, unsigned int iters, float relaxation_factor,
                   const double *sino, double *vol);
void oracle_asdpocs_d(oracle_projector *p, const oracle_asdpocs_params *prm,
                      const double *sino, double *vol, double *x_internal);
void oracle_asdpocs_d_state(oracle_projector *p, const oracle_asdpocs_params *prm,
                            const double *sino, double *vol, double *x_internal,
                            double scalars[4]);
void oracle_sbtv_d(oracle_projector *p, const oracle_sbtv_params *prm,
                   double *sino, double *vol);

#ifdef __cplusplus
}
#endif
#endif
