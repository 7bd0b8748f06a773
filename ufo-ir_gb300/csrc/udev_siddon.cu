/*
 * udev_siddon.cu - the "siddon" projector model: exact line integrals of the
 * pixel image (piecewise constant), and their exact adjoint.
 *
 * The reference ships only the Joseph model, but its projector exposes a
 * "model" property for others (parallel-projector-task.c:123-128). This
 * model keeps the geometry of the reference's backprojector
 * (projector-parallel-joseph.cl:174-195): pixel (i, j) covers
 * X in [i - n/2, i + 1 - n/2], Y in [j - n/2, j + 1 - n/2], and detector
 * bin k of angle theta is the line X cos - Y sin + axis = k + 0.5 (cos, sin
 * from the float LUT; lengths are measured with the line's normal scaled to
 * unit length, as sin^2 + cos^2 of the LUT is not exactly 1). The ray
 * of a bin meets pixel (i, j) over the chord of a line through a unit
 * square: with a = |cos|, b = |sin| and d the distance of the line from the
 * pixel centre, measured along the detector,
 *   L(d) = 1 / max(a, b)                 for |d| <= |a - b| / 2,
 *   L(d) = ((a + b) / 2 - |d|) / (a b)   up to |d| = (a + b) / 2, 0 beyond.
 *
 * Forward: one thread per ray walks the slabs (rows for |cos| >= |sin|,
 * columns otherwise) of the zero-padded image or its padded transpose, the
 * copies the Joseph forward projector reads; in a slab the ray covers at
 * most two pixels, and its length in the slab (1 / max(a, b)) splits where
 * it crosses the pixel boundary. Backward: one thread per pixel evaluates L for the (at most
 * two) bins whose lines cross the pixel, per angle. Both compute the same
 * chord lengths, so the backprojector is the adjoint of the forward one up
 * to rounding. Arithmetic is FP32; the sums are per ray in slab order and
 * per pixel in angle order, with the reference's contract for accumulation
 * (sino = src + scale * S; per subset v = v + relax * sum).
 */
#include <cuda_runtime.h>

#include "udev_internal.cuh"

namespace {

struct SiddonFpArgs {
    const float *volP;      /* padded image rows (walked by row-mode rays) */
    const float *volTP;     /* padded transposed rows (column-mode rays) */
    const float *src;
    const float *w;
    float *out;
    const float *sinv;
    const float *cosv;
    int n;
    int a0;
    int na;
    int pitch;
    float axis;
    float scale;
    long long volp_stride;
    long long sino_stride;
    long long w_stride;
};

constexpr int kPadL = 2;                       /* zero columns left of a padded row */
constexpr float kFloorMagic = 12582912.0f;     /* 1.5 * 2^23 */
constexpr int kFloorMagicBits = 0x4B400000;

/*
 * Grid (ceil(n / 128), na, slices), 128 threads: thread = detector bin.
 * A ray walks the rows of the padded image (rows for |cos| >= |sin|, else
 * the rows of the padded transpose, i.e. the image's columns) with the
 * coordinate across the slab at its lower edge, x0 + j slope, formed by one
 * fma from the ray start (no drift). In slab j the ray spans [lo, hi]
 * (hi - lo = |slope| <= 1): pixel floor(lo), and where it crosses the next
 * boundary the fraction f = (floor(lo) + 1 - lo) / |slope| of the length
 * stays in that pixel and 1 - f goes to the next. floor() is a
 * round-toward-minus-infinity add of 1.5 * 2^23 (exact for |x| < 2^22);
 * the padded column floor(lo) + 2 is clamped (as unsigned) to n + 2, whose
 * two taps are pad zeros, so rays outside the image read zeros without
 * bounds checks.
 */
template <bool UP>
__device__ __forceinline__ float siddon_walk(const float *__restrict__ img, int n, int pitch, float x0, float slope,
                                             float inv)
{
    const uint32_t lim = (uint32_t) n + 2u;
    float sum = 0.0f, xa = x0, jf = 0.0f;
    uint32_t ro = 0;
#pragma unroll 4
    for (int j = 0; j < n; ++j) {
        jf += 1.0f;
        const float xb = fmaf(jf, slope, x0);
        const float lo = UP ? xa : xb;
        const float y = __fadd_rd(lo, kFloorMagic);
        const float c1 = (y - kFloorMagic) + 1.0f;        /* floor(lo) + 1 */
        const uint32_t p = min((uint32_t) (__float_as_int(y) - (kFloorMagicBits - kPadL)), lim);
        const float *row = img + ro + p;
        const float v0 = __ldg(row), v1 = __ldg(row + 1);
        /* the part of the slab's length left of the boundary c1: all of it
         * when the ray does not reach c1 ((c1 - lo) / |slope| >= 1) */
        const float f = fminf((c1 - lo) * inv, 1.0f);
        sum += f * v0 + (1.0f - f) * v1;
        xa = xb;
        ro += (uint32_t) pitch;
    }
    return sum;
}

__global__ void __launch_bounds__(128) siddon_fp_kernel(SiddonFpArgs P)
{
    const int k = (int) (blockIdx.x * blockDim.x + threadIdx.x);
    const int angle = P.a0 + (int) blockIdx.y;
    const int slice = (int) blockIdx.z;
    const int n = P.n;
    if (k >= n)
        return;
    const float sr = __ldg(P.sinv + angle), cr = __ldg(P.cosv + angle);
    const float r = sqrtf(sr * sr + cr * cr);
    const float sn = sr / r, cs = cr / r;
    const float half = 0.5f * (float) n;
    const float u0 = (((float) k + 0.5f) - P.axis) / r;   /* X cos - Y sin = u0, unit normal */
    const bool rows = fabsf(cs) >= fabsf(sn);
    /* rows: X(Y) = (u0 + Y sin) / cos; columns: Y(X) = (X cos - u0) / sin */
    const float len = rows ? 1.0f / fabsf(cs) : 1.0f / fabsf(sn);
    const float slope = rows ? sn / cs : cs / sn;
    const float x0 = (rows ? u0 / cs : (-u0) / sn) + (-half) * slope + half;
    const float inv = 1.0f / fabsf(slope);         /* inf for slope 0: never crosses */
    const float *img = (rows ? P.volP : P.volTP) + (size_t) slice * P.volp_stride;
    /* the slope's sign is the angle's (uniform per block), so each loop
     * knows which slab end is the lower one */
    const float sum = slope >= 0.0f ? siddon_walk<true>(img, n, P.pitch, x0, slope, inv)
                                    : siddon_walk<false>(img, n, P.pitch, x0, slope, inv);
    const size_t oidx = (size_t) slice * P.sino_stride + (size_t) angle * n + k;
    float result = P.src ? P.src[oidx] : 0.0f;
    result += P.scale * (sum * len);
    if (P.w)
        result *= P.w[(size_t) slice * P.w_stride + (size_t) angle * n + k];
    P.out[oidx] = result;
}

constexpr int kMaxSub = 16;

struct SiddonBpArgs {
    const float *sino;
    const float *base;
    float *dst;
    const float *sinv;
    const float *cosv;
    int n;
    int n_subsets;
    float axis;
    float relax;
    long long vol_stride;
    long long sino_stride;
    unsigned int sub_offset[kMaxSub];
    unsigned int sub_n[kMaxSub];
};

/* Per angle, per block: the constants of L and the bin coordinate of the
 * block's centre, C = Xc cos - Yc sin + axis - 0.5, split as kb + frac
 * (kb an integer, frac a float). */
struct SiddonAngle {
    float4 geo;     /* cos, sin, frac, 1 / r */
    float4 shape;   /* p, w / (a b), h = 1 / max(a, b), 1 / (a b) */
    int kb;
};

constexpr int kBpW = 32, kBpH = 8, kBpThreads = kBpW * kBpH;
constexpr int kBpPx = 2;                       /* pixels per thread, 32 columns apart */
constexpr int kBpTileW = kBpW * kBpPx;         /* tile: 64 x 8 pixels */

/* Grid (ceil(n / 64), ceil(n / 8), slices), block 32 x 8: a thread owns
 * pixels tx and tx + 32 of its tile row.
 * The block's threads stage up to 256 angles' constants in shared memory,
 * then each pixel visits the two bins whose lines can cross it: with
 * t = uc - 0.5 the bin coordinate of its centre, bins floor(t) and
 * floor(t) + 1 at distances frac(t) and 1 - frac(t) (every other bin is at
 * least one bin away, beyond the support (a + b) / 2 <= 0.7072). A pixel's
 * t is the tile centre's fraction plus its offset (|dx| <= 31.5, |dy| <= 3.5)
 * times cos and sin, two fmas: ~2e-6 bins of rounding. */
__global__ void __launch_bounds__(kBpThreads) siddon_bp_kernel(SiddonBpArgs P)
{
    __shared__ SiddonAngle ang[kBpThreads];
    const int tid = (int) (threadIdx.y * kBpW + threadIdx.x);
    const int i0 = (int) (blockIdx.x * kBpTileW + threadIdx.x);
    const int j = (int) (blockIdx.y * kBpH + threadIdx.y);
    const int slice = (int) blockIdx.z;
    const int n = P.n;
    const float half = 0.5f * (float) n;
    /* tile centre and the pixels' offsets from it (all exact: half-integers) */
    const float Xc = (float) (blockIdx.x * kBpTileW + kBpTileW / 2) - half;
    const float Yc = (float) (blockIdx.y * kBpH + kBpH / 2) - half;
    float dx[kBpPx];
    bool inside[kBpPx];
    size_t pix[kBpPx];
    float v[kBpPx];
    bool any = false;
#pragma unroll
    for (int u = 0; u < kBpPx; ++u) {
        dx[u] = ((float) (threadIdx.x + kBpW * u) + 0.5f) - (float) (kBpTileW / 2);
        inside[u] = i0 + kBpW * u < n && j < n;
        any = any || inside[u];
        pix[u] = (size_t) slice * P.vol_stride + (size_t) j * n + (size_t) (i0 + kBpW * u);
        v[u] = (inside[u] && P.base) ? P.base[pix[u]] : 0.0f;
    }
    const float dy = ((float) threadIdx.y + 0.5f) - (float) (kBpH / 2);
    const float *sino = P.sino + (size_t) slice * P.sino_stride;
    for (int s = 0; s < P.n_subsets; ++s) {
        const int count = (int) P.sub_n[s];
        float sum[kBpPx];
#pragma unroll
        for (int u = 0; u < kBpPx; ++u)
            sum[u] = 0.0f;
        for (int q0 = 0; q0 < count; q0 += kBpThreads) {
            const int nq = min(kBpThreads, count - q0);
            if (tid < nq) {
                const int angle = (int) P.sub_offset[s] + q0 + tid;
                const float cr = __ldg(P.cosv + angle), sr = __ldg(P.sinv + angle);
                const float r = sqrtf(cr * cr + sr * sr), ir = 1.0f / r;
                const float a = fabsf(cr) * ir, b = fabsf(sr) * ir;
                const float ab = a * b;
                /* Xc cos - Yc sin + (axis - 0.5) as hi + lo: the products'
                 * rounding errors (exact by FMA) and both sums' (TwoSum), with
                 * explicit rounding so that no contraction merges the steps */
                const float pa = __fmul_rn(Xc, cr), pb = __fmul_rn(Yc, sr);
                const float ea = fmaf(Xc, cr, -pa), eb = fmaf(Yc, sr, -pb);
                const float s1 = __fsub_rn(pa, pb);
                const float b1 = __fsub_rn(s1, pa);
                const float e1 = __fadd_rn(__fsub_rn(pa, __fsub_rn(s1, b1)), __fsub_rn(-pb, b1));
                const float ax = P.axis - 0.5f;
                const float hi = __fadd_rn(s1, ax);
                const float b2 = __fsub_rn(hi, s1);
                const float e2 = __fadd_rn(__fsub_rn(s1, __fsub_rn(hi, b2)), __fsub_rn(ax, b2));
                const float kbf = floorf(hi);
                SiddonAngle A;
                /* hi - kb is exact (the fraction bits of hi) */
                const float frac = __fadd_rn(__fsub_rn(hi, kbf), __fadd_rn(__fadd_rn(e1, __fsub_rn(ea, eb)), e2));
                A.geo = make_float4(cr, sr, frac, ir);
                /* 1 / (a b) stays finite (3e38) for axis-aligned angles, where
                 * every offset beyond p = w gets L = 0 */
                const float iab = ab > 0.0f ? 1.0f / ab : 3.0e38f;
                A.shape = make_float4(0.5f * fabsf(a - b), 0.5f * (a + b) * iab, 1.0f / fmaxf(a, b), iab);
                A.kb = (int) kbf;
                ang[tid] = A;
            }
            __syncthreads();
            if (any) {
                const float *row = sino + (size_t) (P.sub_offset[s] + q0) * n;
#pragma unroll 2
                for (int q = 0; q < nq; ++q, row += n) {
                    const float4 g = ang[q].geo;
                    const float4 h = ang[q].shape;
                    const int kb = ang[q].kb;
                    const float ty = fmaf(-dy, g.y, g.z);
#pragma unroll
                    for (int u = 0; u < kBpPx; ++u) {
                        const float t = fmaf(dx[u], g.x, ty);
                        /* floor(t) by a round-down add of 1.5 * 2^23 (|t| < 2^22) */
                        const float y = __fadd_rd(t, kFloorMagic);
                        const float f = t - (y - kFloorMagic);     /* exact */
                        const int ka = kb + (__float_as_int(y) - kFloorMagicBits);
                        const float da = f * g.w, db = g.w - da;
                        /* L(d) = h up to p, then (w - d) / (a b) down to 0 */
                        const float la = da <= h.x ? h.z : fmaxf(0.0f, fmaf(-da, h.w, h.y));
                        const float lb = db <= h.x ? h.z : fmaxf(0.0f, fmaf(-db, h.w, h.y));
                        const float va = (unsigned int) ka < (unsigned int) n ? __ldg(row + ka) : 0.0f;
                        const float vb = (unsigned int) (ka + 1) < (unsigned int) n ? __ldg(row + ka + 1) : 0.0f;
                        sum[u] = fmaf(la, va, sum[u]);
                        sum[u] = fmaf(lb, vb, sum[u]);
                    }
                }
            }
            __syncthreads();
        }
#pragma unroll
        for (int u = 0; u < kBpPx; ++u)
            v[u] += P.relax * sum[u];
    }
#pragma unroll
    for (int u = 0; u < kBpPx; ++u)
        if (inside[u])
            P.dst[pix[u]] = v[u];
}

}  // namespace

extern "C" int udev_siddon_fp(udev *d, const udev_geom *g, int a0, int na, const float *volP, const float *volTP,
                              const float *src, const float *w, int w_shared, float *out, float scale, int n_slices)
{
    if (n_slices <= 0 || na <= 0)
        return UFOIR_OK;
    const int n = g->n_dets;
    if (a0 < 0 || a0 + na > g->n_angles || n < 1 || n > 32768 || n_slices > 65535 || na > 65535) {
        udev_set_error(d, "siddon_fp: angles [%d, %d) of %d, n = %d, %d slices out of range", a0, a0 + na,
                       g->n_angles, n, n_slices);
        return UFOIR_ERR_INVALID;
    }
    UDEV_BIND(d);
    SiddonFpArgs A;
    A.volP = volP;
    A.volTP = volTP;
    A.src = src;
    A.w = w;
    A.out = out;
    A.sinv = g->d_sin;
    A.cosv = g->d_cos;
    A.n = n;
    A.a0 = a0;
    A.na = na;
    A.pitch = udev_fp_pitch(n);
    A.axis = g->axis;
    A.scale = scale;
    A.volp_stride = (long long) n * A.pitch;
    A.sino_stride = (long long) g->n_angles * n;
    A.w_stride = w_shared ? 0 : A.sino_stride;
    dim3 grid(udev_div_up(n, 128), (unsigned int) na, (unsigned int) n_slices);
    siddon_fp_kernel<<<grid, 128, 0, d->stream>>>(A);
    return udev_after_launch(d, "siddon_fp_kernel");
}

extern "C" int udev_siddon_bp(udev *d, const udev_geom *g, const ufoir_subset *subsets, int n_subsets,
                              const float *sino, const float *base, float *dst, float relax, int n_slices)
{
    if (n_slices <= 0)
        return UFOIR_OK;
    const int n = g->n_dets;
    if (n_subsets < 0 || n_subsets > kMaxSub || n < 1 || n_slices > 65535) {
        udev_set_error(d, "siddon_bp: %d subsets (at most %d), %d slices", n_subsets, kMaxSub, n_slices);
        return UFOIR_ERR_INVALID;
    }
    SiddonBpArgs A;
    for (int s = 0; s < n_subsets; ++s) {
        if (subsets[s].offset + subsets[s].n > (unsigned int) g->n_angles) {
            udev_set_error(d, "siddon_bp: subset %d [%u, %u) beyond %d angles", s, subsets[s].offset,
                           subsets[s].offset + subsets[s].n, g->n_angles);
            return UFOIR_ERR_INVALID;
        }
        A.sub_offset[s] = subsets[s].offset;
        A.sub_n[s] = subsets[s].n;
    }
    UDEV_BIND(d);
    A.sino = sino;
    A.base = base;
    A.dst = dst;
    A.sinv = g->d_sin;
    A.cosv = g->d_cos;
    A.n = n;
    A.n_subsets = n_subsets;
    A.axis = g->axis;
    A.relax = relax;
    A.vol_stride = (long long) n * n;
    A.sino_stride = (long long) g->n_angles * n;
    dim3 grid(udev_div_up(n, kBpTileW), udev_div_up(n, kBpH), (unsigned int) n_slices);
    siddon_bp_kernel<<<grid, dim3(kBpW, kBpH), 0, d->stream>>>(A);
    return udev_after_launch(d, "siddon_bp_kernel");
}
