/*
 * CPU oracle for the ufo-ir iterative-reconstruction path (see oracle.h).
 * TEST INFRASTRUCTURE ONLY: the product never links this file.
 *
 * Build: gcc -std=c11 -O2 -ffp-contract=off -fno-fast-math -fopenmp -fPIC -shared
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static void *xmalloc(size_t n)
{
    void *p = malloc(n ? n : 1);
    if (!p) {
        fprintf(stderr, "oracle: out of memory (%zu bytes)\n", n);
        abort();
    }
    return p;
}

static void *xcalloc(size_t n, size_t s)
{
    void *p = calloc(n ? n : 1, s ? s : 1);
    if (!p) {
        fprintf(stderr, "oracle: out of memory\n");
        abort();
    }
    return p;
}

typedef struct {
    double *data;
    long width;
    long height;
} oracle_image_d;

/* Kernel table of the FP64 twin (same slots as oracle_kernels, double data). */
typedef struct {
    void (*fp)(oracle_image_d, oracle_image_d, const float *, const float *, oracle_dims,
               float, oracle_subset, float);
    void (*bp)(oracle_image_d, oracle_image_d, float, const float *, const float *,
               oracle_dims, float, oracle_subset);
    void (*op_set)(oracle_image_d, float);
    void (*op_inv)(oracle_image_d);
    void (*op_mul)(oracle_image_d, oracle_image_d, oracle_image_d);
    void (*op_add)(oracle_image_d, oracle_image_d, oracle_image_d);
    void (*op_deduction)(oracle_image_d, oracle_image_d, oracle_image_d);
    void (*op_deduction2)(oracle_image_d, oracle_image_d, float, oracle_image_d);
    void (*op_add2)(oracle_image_d, oracle_image_d, float, oracle_image_d);
    void (*op_mul_rows)(oracle_image_d, oracle_image_d, oracle_image_d, unsigned int, unsigned int);
    void (*op_posc)(oracle_image_d, oracle_image_d);
    void (*l1_grad)(oracle_image_d, oracle_image_d);
    void (*dx)(const double *, double *, long, long);
    void (*dxt)(const double *, double *, long, long);
    void (*dy)(const double *, double *, long, long);
    void (*dyt)(const double *, double *, long, long);
} oracle_kernels_d;

/* float instantiation: the reference's arithmetic */
#define REAL float
#define IMG oracle_image
#define SFX _f
#define FLOOR floorf
#define FABS fabsf
#define SQRT sqrtf
#define KT oracle_kernels
#include "oracle_impl.inc"
#undef REAL
#undef IMG
#undef SFX
#undef FLOOR
#undef FABS
#undef SQRT
#undef KT

/* double instantiation: FP64 twin */
#define REAL double
#define IMG oracle_image_d
#define SFX _d
#define FLOOR floor
#define FABS fabs
#define SQRT sqrt
#define KT oracle_kernels_d
#include "oracle_impl.inc"
#undef REAL
#undef IMG
#undef SFX
#undef FLOOR
#undef FABS
#undef SQRT
#undef KT

static const oracle_kernels port_f = {
    k_fp_f, k_bp_f, k_set_f, k_inv_f, k_mul_f, k_add_f, k_deduction_f, k_deduction2_f,
    k_add2_f, k_mul_rows_f, k_posc_f, k_l1_grad_f, k_dx_f, k_dxt_f, k_dy_f, k_dyt_f,
};

static const oracle_kernels_d port_d = {
    k_fp_d, k_bp_d, k_set_d, k_inv_d, k_mul_d, k_add_d, k_deduction_d, k_deduction2_d,
    k_add2_d, k_mul_rows_d, k_posc_d, k_l1_grad_d, k_dx_d, k_dxt_d, k_dy_d, k_dyt_d,
};

const oracle_kernels *oracle_port_kernels(void)
{
    return &port_f;
}

void oracle_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0)
        omp_set_num_threads(n);
#else
    (void) n;
#endif
}

int oracle_get_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* create_lut_buffer (…parallel-projector-task.c:437-460): the product
 * i * angles_step is a float product (guint times gfloat). */
void oracle_make_lut(unsigned int n_angles, float step, float *sin_out, float *cos_out)
{
    for (unsigned int i = 0; i < n_angles; i++) {
        const float a = (float) i * step;
        const double rad_angle = a;
        sin_out[i] = (float) sin(rad_angle);
        cos_out[i] = (float) cos(rad_angle);
    }
}

/* generate_full_subsets_list (…parallel-projector-task.c:463-498). */
unsigned int oracle_make_full_subsets(const float *s, const float *c, unsigned int n_angles,
                                      oracle_subset *out)
{
    if (n_angles == 0)
        return 0;
    unsigned int idx = 0;
    int direction = fabs((double) s[0]) <= fabs((double) c[0]);
    out[0].direction = direction;
    out[0].offset = 0;
    out[0].n = 1;
    for (unsigned int i = 1; i < n_angles; ++i) {
        direction = fabs((double) s[i]) <= fabs((double) c[i]);
        if (direction != out[idx].direction) {
            idx++;
            out[idx].direction = direction;
            out[idx].offset = i;
            out[idx].n = 1;
        } else {
            out[idx].n++;
        }
    }
    return idx + 1;
}

/* generate_subsets (sart-task.c:230-248). */
void oracle_make_angle_subsets(const float *s, const float *c, unsigned int n_angles,
                               oracle_subset *out)
{
    for (unsigned int i = 0; i < n_angles; ++i) {
        out[i].direction = fabs((double) s[i]) <= fabs((double) c[i]);
        out[i].offset = i;
        out[i].n = 1;
    }
}

void oracle_forward(const oracle_kernels *k, const oracle_projector *p, const float *vol, float *sino)
{
    geom_f g;
    geom_init_f(&g, p);
    fwd_f(k, p, &g, vol, sino);
    geom_free_f(&g);
}

void oracle_backward(const oracle_kernels *k, const oracle_projector *p, float *vol, const float *sino)
{
    geom_f g;
    geom_init_f(&g, p);
    bwd_f(k, p, &g, vol, sino);
    geom_free_f(&g);
}

void oracle_projector_process(const oracle_kernels *k, const oracle_projector *p, int is_forward,
                              const float *in, float *out)
{
    const long n = (long) p->n_dets;
    if (is_forward) {
        k->op_set(img_f(out, n, (long) p->n_angles), 0.0f);
        oracle_forward(k, p, in, out);
    } else {
        k->op_set(img_f(out, n, n), 0.0f);
        oracle_backward(k, p, out, in);
    }
}

void oracle_sart(const oracle_kernels *k, oracle_projector *p, unsigned int iters,
                 float relaxation_factor, const float *sino, float *vol)
{
    sart_impl_f(k, p, iters, relaxation_factor, sino, vol);
}

void oracle_sirt(const oracle_kernels *k, oracle_projector *p, unsigned int iters,
                 float relaxation_factor, const float *sino, float *vol)
{
    sirt_impl_f(k, p, iters, relaxation_factor, sino, vol);
}

void oracle_sirt_weights(const oracle_kernels *k, oracle_projector *p, float *ray_weights,
                         float *pixel_weights)
{
    geom_f g;
    geom_init_f(&g, p);
    sirt_weights_f(k, p, &g, ray_weights, pixel_weights);
    geom_free_f(&g);
}

void oracle_sirt_iterate(const oracle_kernels *k, oracle_projector *p, unsigned int iters,
                         float relaxation_factor, const float *sino, float *ray_weights,
                         float *pixel_weights, float *vol)
{
    geom_f g;
    geom_init_f(&g, p);
    sirt_iterate_f(k, p, &g, iters, relaxation_factor, sino, ray_weights, pixel_weights, vol);
    geom_free_f(&g);
}

void oracle_asdpocs(const oracle_kernels *k, oracle_projector *p, const oracle_asdpocs_params *prm,
                    const float *sino, float *vol, float *x_internal)
{
    asdpocs_impl_f(k, p, prm, sino, vol, x_internal, NULL);
}

void oracle_asdpocs_state(const oracle_kernels *k, oracle_projector *p, const oracle_asdpocs_params *prm,
                          const float *sino, float *vol, float *x_internal, float scalars[4])
{
    asdpocs_impl_f(k, p, prm, sino, vol, x_internal, scalars);
}

void oracle_sbtv(const oracle_kernels *k, oracle_projector *p, const oracle_sbtv_params *prm,
                 float *sino, float *vol)
{
    sbtv_impl_f(k, p, prm, sino, vol);
}

float oracle_l1_norm(const float *v, unsigned long w, unsigned long h)
{
    return h_l1_norm_f(v, w, h, ORACLE_NORM_COMPAT);
}

float oracle_dot_product(const float *a, const float *b, unsigned long w, unsigned long h)
{
    return h_dot_f(a, b, w, h, ORACLE_NORM_COMPAT);
}

float oracle_l1_norm_fp64(const float *v, unsigned long w, unsigned long h)
{
    return h_l1_norm_f(v, w, h, ORACLE_NORM_FP64);
}

float oracle_dot_product_fp64(const float *a, const float *b, unsigned long w, unsigned long h)
{
    return h_dot_f(a, b, w, h, ORACLE_NORM_FP64);
}

/* ---- FP64 twin entry points ---- */

void oracle_forward_d(const oracle_projector *p, const double *vol, double *sino)
{
    geom_d g;
    geom_init_d(&g, p);
    fwd_d(&port_d, p, &g, vol, sino);
    geom_free_d(&g);
}

void oracle_backward_d(const oracle_projector *p, double *vol, const double *sino)
{
    geom_d g;
    geom_init_d(&g, p);
    bwd_d(&port_d, p, &g, vol, sino);
    geom_free_d(&g);
}

void oracle_sirt_d(oracle_projector *p, unsigned int iters, float relaxation_factor,
                   const double *sino, double *vol)
{
    sirt_impl_d(&port_d, p, iters, relaxation_factor, sino, vol);
}

void oracle_sart_d(oracle_projector *p, unsigned int iters, float relaxation_factor,
                   const double *sino, double *vol)
{
    sart_impl_d(&port_d, p, iters, relaxation_factor, sino, vol);
}

void oracle_asdpocs_d(oracle_projector *p, const oracle_asdpocs_params *prm,
                      const double *sino, double *vol, double *x_internal)
{
    oracle_asdpocs_params q = *prm;
    q.norm_mode = ORACLE_NORM_FP64;
    asdpocs_impl_d(&port_d, p, &q, sino, vol, x_internal, NULL);
}

void oracle_asdpocs_d_state(oracle_projector *p, const oracle_asdpocs_params *prm, const double *sino,
                            double *vol, double *x_internal, double scalars[4])
{
    oracle_asdpocs_params q = *prm;
    q.norm_mode = ORACLE_NORM_FP64;
    asdpocs_impl_d(&port_d, p, &q, sino, vol, x_internal, scalars);
}

void oracle_sbtv_d(oracle_projector *p, const oracle_sbtv_params *prm, double *sino, double *vol)
{
    oracle_sbtv_params q = *prm;
    q.norm_mode = ORACLE_NORM_FP64;
    sbtv_impl_d(&port_d, p, &q, sino, vol);
}
