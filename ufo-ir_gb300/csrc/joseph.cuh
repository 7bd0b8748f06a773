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

#include <cstdint>

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

/* 32-bit shared-memory load. */
__device__ __forceinline__ float lds(uint32_t addr)
{
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(addr));
    return v;
}

/* floor() by a round-toward-minus-infinity add of 1.5 * 2^23: for
 * |x| < 2^22, y = x + M lands in [2^23, 2^24) where floats are integers, so
 * y - M == floor(x) exactly and the bits of y are floor(x) + kFloorMagicBits. */
constexpr float kFloorMagic = 12582912.0f;
constexpr int kFloorMagicBits = 0x4B400000;

/*
 * Paired forms for two samples at once, on the packed FP32 instructions of
 * sm_100 and later (PTX add/sub/mul/fma .f32x2). Each lane rounds exactly as
 * the scalar instruction. The code generator fuses a packed multiply that
 * feeds a packed add into one fused multiply-add even with explicit rounding
 * modifiers, which changes the rounding, so every product that is added
 * later is written as fma(a, b, z) with z = -0.0 supplied at run time (the
 * compiler cannot fold it): a*b + (-0) rounds exactly as a*b, signed zeros
 * included, and an fma cannot be fused further.
 */
__device__ __forceinline__ unsigned long long pack2(float2 a)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
    return r;
}

__device__ __forceinline__ float2 unpack2(unsigned long long r)
{
    float2 a;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
    return a;
}

__device__ __forceinline__ float2 splat(float a)
{
    return make_float2(a, a);
}

__device__ __forceinline__ float2 add2(float2 a, float2 b)
{
    unsigned long long r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)));
    return unpack2(r);
}

/* round toward minus infinity */
__device__ __forceinline__ float2 add2_rd(float2 a, float2 b)
{
    unsigned long long r;
    asm("add.rm.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)));
    return unpack2(r);
}

__device__ __forceinline__ float2 sub2(float2 a, float2 b)
{
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)));
    return unpack2(r);
}

/* a * b as fma(a, b, z), z = (-0, -0) from a run-time value: a product that
 * can be added to something else without being fused into it. */
__device__ __forceinline__ float2 mul2z(float2 a, float2 b, float2 z)
{
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)), "l"(pack2(z)));
    return unpack2(r);
}

/* (1 - t) * T0 + t * T1 per lane, each operation rounded. */
__device__ __forceinline__ float2 lerp2(float2 t, float2 t0, float2 t1, float2 z)
{
    return add2(mul2z(sub2(splat(1.0f), t), t0, z), mul2z(t, t1, z));
}

/* a * b + c per lane, fused (one rounding). */
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c)
{
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)), "l"(pack2(c)));
    return unpack2(r);
}

/*
 * Fast arithmetic (the projector's "arithmetic" = "fast"): acc + lerp as
 * (acc + T0) + t * (T1 - T0) with the product fused, three packed operations
 * instead of the exact form's five (1 - t, two products, their sum, the
 * accumulation). The value differs from the exact form's by a few units in
 * the last place of the sum; the relative L2 error of a whole projection
 * stays far below 1e-5.
 */
__device__ __forceinline__ float2 lerp_acc_fast2(float2 acc, float2 t, float2 t0, float2 t1)
{
    return fma2(t, sub2(t1, t0), add2(acc, t0));
}

/*
 * floor(c - 0.5) and t = (c - 0.5) - floor(c - 0.5) for coordinates c >= 0.5,
 * in three paired operations: y = rd(c + (2^23 - 0.5)) lands in [2^23, 2^24)
 * with bits kHalfFloorBits + floor(c - 0.5); y - (2^23 - 0.5) and c minus it
 * are exact, and c - 0.5 itself is exact for c >= 0.5, so t is the same
 * fraction the four-step form computes.
 */
constexpr float kHalfFloorMagic = 8388607.5f;
constexpr int kHalfFloorBits = 0x4B000000;

__device__ __forceinline__ float2 floor_half2(float2 c, float2 &t)
{
    const float2 y = add2_rd(c, splat(kHalfFloorMagic));
    t = sub2(c, sub2(y, splat(kHalfFloorMagic)));
    return y;
}

/* The same for any |c - 0.5| < 2^22 (bits kFloorMagicBits + floor(c - 0.5)). */
__device__ __forceinline__ float2 floor_any2(float2 c, float2 &t)
{
    const float2 cm = sub2(c, splat(0.5f));
    const float2 y = add2_rd(cm, splat(kFloorMagic));
    t = sub2(cm, sub2(y, splat(kFloorMagic)));
    return y;
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
