/*
 * udev_ceiling.cu - the interpolated-sample rate ceilings of this GPU: each
 * projector's exact per-sample sequence run from shared memory by every SM,
 * with no global traffic, no barriers and no bank conflicts. The projectors'
 * samples/s are reported against them.
 *  - forward: packed FP32 floor, linear filter and sums, two shared-memory
 *    taps per sample, index clamp (fp_tiles_kernel's inner loop). The rate
 *    does not change with occupancy (24 to 64 warps per SM give the same);
 *    it is bound by the FMA pipe, where a packed FP32 instruction takes two
 *    cycles.
 *  - backward: bp_tiles_kernel's inner loop for an unclamped tile: per angle
 *    the angle record and the row products from shared memory, per pixel pair
 *    the coordinate, the three-step floor, two taps per pixel from the
 *    angle's window, the filter and the per-pixel sum; 16 pixels per thread
 *    and three 256-thread CTAs per SM, as the kernel runs.
 */
#include <cuda_runtime.h>

#include "joseph.cuh"
#include "udev_internal.cuh"

namespace {

constexpr int kRowFloats = 1024;     /* one shared row */
constexpr int kRows = 2048;          /* rows walked per launch */
constexpr int kPairs = 8;            /* 16 rays per thread, as the FP kernel at n = 1448 */
constexpr int kThreads = 768;

__global__ void __launch_bounds__(kThreads, 1) sample_ceiling_kernel(float neg_zero, float *out)
{
    __shared__ float row[2][kRowFloats];
    for (int i = (int) threadIdx.x; i < 2 * kRowFloats; i += kThreads)
        (&row[0][0])[i] = (float) ((i * 37) & 255) * 0.0078125f;
    __syncthreads();
    const float2 z2 = joseph::splat(neg_zero);
    const uint32_t base = (uint32_t) __cvta_generic_to_shared(&row[0][0]);
    const uint32_t col_lim = (uint32_t) kRowFloats - 2u;
    float2 c[kPairs], inner[kPairs], sum[kPairs], stp[kPairs];
#pragma unroll
    for (int k = 0; k < kPairs; ++k) {
        /* adjacent lanes one texel apart: conflict-free shared loads, as the
         * projectors' lane layouts are */
        const float s0 = (float) ((threadIdx.x + k * 97) % 900) + 8.25f;
        c[k] = make_float2(s0, s0 + 1.5f);
        stp[k] = joseph::splat(0.001953125f * (float) (k + 1));
        inner[k] = make_float2(0.0f, 0.0f);
        sum[k] = make_float2(0.0f, 0.0f);
    }
    for (int r = 0; r < kRows; ++r) {
        const uint32_t rs = base + 4u * (uint32_t) ((r & 1) * kRowFloats);
#pragma unroll
        for (int k = 0; k < kPairs; ++k) {
            float2 t;
            const float2 y = joseph::floor_any2(c[k], t);
            const uint32_t p0 = min((uint32_t) (__float_as_int(y.x) - joseph::kFloorMagicBits + 2), col_lim);
            const uint32_t p1 = min((uint32_t) (__float_as_int(y.y) - joseph::kFloorMagicBits + 2), col_lim);
            const uint32_t a0 = rs + 4u * p0, a1 = rs + 4u * p1;
            const float2 t0 = make_float2(joseph::lds(a0), joseph::lds(a1));
            const float2 t1 = make_float2(joseph::lds(a0 + 4u), joseph::lds(a1 + 4u));
            inner[k] = joseph::add2(inner[k], joseph::lerp2(t, t0, t1, z2));
            c[k] = joseph::add2(c[k], stp[k]);
        }
        if (((r + 1) & 63) == 0) {
#pragma unroll
            for (int k = 0; k < kPairs; ++k) {
                sum[k] = joseph::add2(sum[k], inner[k]);
                inner[k] = make_float2(0.0f, 0.0f);
            }
        }
    }
    float acc = 0.0f;
#pragma unroll
    for (int k = 0; k < kPairs; ++k)
        acc += sum[k].x + sum[k].y;
    out[blockIdx.x * kThreads + threadIdx.x] = acc;
}

constexpr int kBpAngles = 4096;      /* angles walked per launch */
constexpr int kBpChunk = 32;         /* distinct angles staged, as one chunk of the kernel */
constexpr int kBpWin = 320;          /* window per angle */

__global__ void __launch_bounds__(256) sample_ceiling_bp_kernel(float neg_zero, float *out)
{
    __shared__ float win[kBpChunk][kBpWin];
    __shared__ float4 ang[kBpChunk];
    __shared__ float4 nys[kBpChunk][8][4];
    const int tid = (int) (threadIdx.y * 32 + threadIdx.x);
    for (int i = tid; i < kBpChunk * kBpWin; i += 256)
        (&win[0][0])[i] = (float) ((i * 37) & 255) * 0.0078125f;
    if (tid < kBpChunk)
        ang[tid] = make_float4(0.96875f - 0.0078125f * (float) tid, 0.5f, __int_as_float(0), 0.0f);
    /* row products of rows ty + 8p, spread so that the coordinates stay in
     * [150, 300] */
    for (int i = tid; i < kBpChunk * 8 * 16; i += 256)
        reinterpret_cast<float *>(&nys[0][0][0])[i] = (float) ((i * 7) % 97) + 30.0f;
    __syncthreads();
    const float2 z2 = joseph::splat(neg_zero);
    const float2 shift2 = joseph::splat(120.25f);
    const float fX = (float) threadIdx.x + 0.5f;
    const uint32_t win0 = (uint32_t) __cvta_generic_to_shared(&win[0][0]);
    float2 sum[8];
#pragma unroll
    for (int q = 0; q < 8; ++q)
        sum[q] = make_float2(0.0f, 0.0f);
#pragma unroll 1
    for (int a = 0; a < kBpAngles; ++a) {
        const int i = a & (kBpChunk - 1);
        const float4 an = ang[i];
        float2 ny[8];
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            const float4 v = nys[i][threadIdx.y][f];
            ny[2 * f] = make_float2(v.x, v.y);
            ny[2 * f + 1] = make_float2(v.z, v.w);
        }
        const uint32_t base = win0 + 4u * (uint32_t) (i * kBpWin) -
                              4u * ((uint32_t) __float_as_int(an.z) + (uint32_t) joseph::kHalfFloorBits);
        const float2 fxc = joseph::splat(__fmul_rn(fX, an.x));
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const float2 sc = joseph::add2(joseph::add2(fxc, ny[q]), shift2);
            float2 t;
            const float2 y = joseph::floor_half2(sc, t);
            const uint32_t a0 = base + 4u * (uint32_t) __float_as_int(y.x);
            const uint32_t a1 = base + 4u * (uint32_t) __float_as_int(y.y);
            const float2 t0 = make_float2(joseph::lds(a0), joseph::lds(a1));
            const float2 t1 = make_float2(joseph::lds(a0 + 4u), joseph::lds(a1 + 4u));
            sum[q] = joseph::add2(sum[q], joseph::lerp2(t, t0, t1, z2));
        }
    }
    float acc = 0.0f;
#pragma unroll
    for (int q = 0; q < 8; ++q)
        acc += sum[q].x + sum[q].y;
    out[blockIdx.x * 256 + tid] = acc;
}

}  // namespace

extern "C" int udev_sample_ceiling_bp(udev *d, double *samples_per_s)
{
    UDEV_BIND(d);
    const int blocks = 3 * d->sm_count;
    float *out = nullptr;
    int rc = udev_malloc(d, (void **) &out, sizeof(float) * (size_t) blocks * 256);
    if (rc)
        return rc;
    sample_ceiling_bp_kernel<<<blocks, dim3(32, 8), 0, d->stream>>>(-0.0f, out);
    rc = udev_after_launch(d, "sample_ceiling_bp_kernel");
    float ms = 0.0f;
    if (!rc)
        rc = udev_timer_begin(d);
    if (!rc) {
        sample_ceiling_bp_kernel<<<blocks, dim3(32, 8), 0, d->stream>>>(-0.0f, out);
        rc = udev_after_launch(d, "sample_ceiling_bp_kernel");
    }
    if (!rc)
        rc = udev_timer_end(d, &ms);
    udev_free(d, out);
    if (rc)
        return rc;
    const double samples = (double) blocks * 256 * 16 * kBpAngles;
    *samples_per_s = ms > 0.0f ? samples / (ms * 1e-3) : 0.0;
    return UFOIR_OK;
}

extern "C" int udev_sample_ceiling(udev *d, double *samples_per_s)
{
    UDEV_BIND(d);
    const int blocks = d->sm_count;
    float *out = nullptr;
    int rc = udev_malloc(d, (void **) &out, sizeof(float) * (size_t) blocks * kThreads);
    if (rc)
        return rc;
    /* warm-up, then a timed launch */
    sample_ceiling_kernel<<<blocks, kThreads, 0, d->stream>>>(-0.0f, out);
    rc = udev_after_launch(d, "sample_ceiling_kernel");
    float ms = 0.0f;
    if (!rc)
        rc = udev_timer_begin(d);
    if (!rc) {
        sample_ceiling_kernel<<<blocks, kThreads, 0, d->stream>>>(-0.0f, out);
        rc = udev_after_launch(d, "sample_ceiling_kernel");
    }
    if (!rc)
        rc = udev_timer_end(d, &ms);
    udev_free(d, out);
    if (rc)
        return rc;
    const double samples = (double) blocks * kThreads * kPairs * 2 * kRows;
    *samples_per_s = ms > 0.0f ? samples / (ms * 1e-3) : 0.0;
    return UFOIR_OK;
}
