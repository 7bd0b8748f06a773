/*
 * joseph.cuh - device arithmetic of the parallel-beam Joseph projector,
 * written so that every operation rounds exactly as the reference's OpenCL
 * kernels do on an IEEE device (projector-parallel-joseph.cl), with no
 * contraction into FMA:
 *
 *  - the sampler's linear filter at a texel-centre minor coordinate reduces
 *    to  (1 - t) * T0 + t * T1  with  t = frac(c - 0.5), i0 = floor(c - 0.5)
 *    (OpenCL 1.2 section 8.2; the weights of the other axis are exactly 1 and 0);
 *  - texels outside the image read 0 (CLK_ADDRESS_CLAMP border);
 *  - the forward projector's start coordinate contains the double literal
 *    0.5, so its first product is evaluated in double (…joseph.cl:73, :134);
 *  - the moving coordinate is a float recurrence c += step (…joseph.cl:86, :147).
 */
#ifndef UFOIR_JOSEPH_CUH
#define UFOIR_JOSEPH_CUH

#include <cuda_runtime.h>

namespace joseph {

/* Per-geometry constants shared by FP and BP (…joseph.cl:51-60, :174-187). */
struct AxisConsts {
    float required_width;   /* axis_pos * 2 */
    float diff;             /* width - required_width */
    float ros;              /* diff / 2: rotation-centre shift */
    float os;               /* width / 2: origin shift */
};

__device__ __forceinline__ AxisConsts axis_consts(int width, float axis)
{
    AxisConsts k;
    const float w = (float) width;
    k.required_width = __fmul_rn(axis, 2.0f);
    k.diff = __fsub_rn(w, k.required_width);
    k.ros = __fdiv_rn(k.diff, 2.0f);
    k.os = __fdiv_rn(w, 2.0f);
    return k;
}

/* Inactive-detector switch (…joseph.cl:62-66, :123-127). */
__device__ __forceinline__ bool detector_inactive(const AxisConsts &k, int s)
{
    return (k.diff < 0.0f && (float) s < fabsf(k.diff)) ||
           (k.diff > 0.0f && (float) s > k.required_width);
}

/* Steps of a ray: horizontal (dir 0) walks x with y += cos/sin; vertical
 * (dir 1) walks y with x += sin/cos (…joseph.cl:68-69, :129-130). */
__device__ __forceinline__ void ray_steps(int dir, float sn, float cs, float &det_step,
                                          float &slice_step)
{
    if (dir == 0) {
        det_step = __fdiv_rn(-1.0f, sn);
        slice_step = __fdiv_rn(cs, sn);
    } else {
        det_step = __fdiv_rn(1.0f, cs);
        slice_step = __fdiv_rn(sn, cs);
    }
}

/* Start value of the interpolated coordinate of ray s (…joseph.cl:73-75, :134-136):
 * ((0.5 + ros + s - 0.5f*n) * det_step + (-os)*slice_step + 0.5f*n), the
 * first product in double, the second in float, result rounded to float. */
__device__ __forceinline__ float ray_start(const AxisConsts &k, int s, int n, float det_step,
                                           float slice_step)
{
    const float half_n = __fmul_rn(0.5f, (float) n);
    double t = __dadd_rn(0.5, (double) k.ros);
    t = __dadd_rn(t, (double) s);
    t = __dsub_rn(t, (double) half_n);
    t = __dmul_rn(t, (double) det_step);
    t = __dadd_rn(t, (double) __fmul_rn(-k.os, slice_step));
    t = __dadd_rn(t, (double) half_n);
    return __double2float_rn(t);
}

/* Number of 64-sample blocks: ceil(convert_float(width) / BLOCK_SIZE) (…joseph.cl:81). */
__device__ __forceinline__ int n_blocks(int width)
{
    return (int) ceilf(__fdiv_rn((float) width, 64.0f));
}

/* Linear-filter weights at coordinate c: index i0 and fraction t. */
__device__ __forceinline__ void lerp_coord(float c, int &i0, float &t)
{
    const float cm = __fsub_rn(c, 0.5f);
    const float f = floorf(cm);
    i0 = (int) f;
    t = __fsub_rn(cm, f);
}

__device__ __forceinline__ float lerp(float t, float t0, float t1)
{
    return __fadd_rn(__fmul_rn(__fsub_rn(1.0f, t), t0), __fmul_rn(t, t1));
}

/* Bounds-checked texel of a row with a zero border. */
__device__ __forceinline__ float texel(const float *__restrict__ row, int i, int n)
{
    return (i >= 0 && i < n) ? __ldg(row + i) : 0.0f;
}

/* Edges of the backprojector's simulated clamp-to-edge (…joseph.cl:180-182). */
__device__ __forceinline__ void bp_edges(const AxisConsts &k, int width, float axis, float &e0,
                                         float &e1)
{
    const float half = k.diff < 0.0f ? __fsub_rn((float) width, axis) : axis;
    e0 = __fadd_rn(__fsub_rn(axis, half), 0.5f);
    e1 = __fsub_rn(__fadd_rn(axis, half), 0.5f);
}

}  // namespace joseph

#endif
