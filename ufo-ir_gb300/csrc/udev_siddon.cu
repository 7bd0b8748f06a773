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
 * columns otherwise); in a slab the ray covers at most two pixels, and its
 * length in the slab (1 / max(a, b)) splits where it crosses the pixel
 * boundary. Backward: one thread per pixel evaluates L for the (at most
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
    const float *vol;
    const float *src;
    const float *w;
    float *out;
    const float *sinv;
    const float *cosv;
    int n;
    int a0;
    int na;
    float axis;
    float scale;
    long long vol_stride;
    long long sino_stride;
    long long w_stride;
};

/* Grid (ceil(n / 128), na, slices), 128 threads: thread = detector bin. */
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
    const float *img = P.vol + (size_t) slice * P.vol_stride;
    float sum = 0.0f;
    if (fabsf(cs) >= fabsf(sn)) {
        /* rows: X(Y) = (u0 + Y sin) / cos, |dX/dY| <= 1 */
        const float len = 1.0f / fabsf(cs);
        const float slope = sn / cs;
        /* column coordinate at row j's lower edge, x0 + j slope with one
         * rounding (no drift along the ray) */
        const float x0 = u0 / cs + (-half) * slope + half;
        float xa = x0;
        for (int j = 0; j < n; ++j) {
            const float xb = fmaf((float) (j + 1), slope, x0);
            const float lo = fminf(xa, xb), hi = fmaxf(xa, xb);
            const float c0f = floorf(lo);
            const int c0 = (int) c0f;
            float v0 = (c0 >= 0 && c0 < n) ? __ldg(img + (size_t) j * n + c0) : 0.0f;
            if (hi > c0f + 1.0f) {
                /* crosses the boundary at column c0 + 1 */
                const float f = (c0f + 1.0f - lo) / (hi - lo);
                const float v1 = (c0 + 1 >= 0 && c0 + 1 < n) ? __ldg(img + (size_t) j * n + c0 + 1) : 0.0f;
                sum += len * (f * v0 + (1.0f - f) * v1);
            } else {
                sum += len * v0;
            }
            xa = xb;
        }
    } else {
        /* columns: Y(X) = (X cos - u0) / sin, |dY/dX| < 1 */
        const float len = 1.0f / fabsf(sn);
        const float slope = cs / sn;
        const float y0 = (-u0) / sn + (-half) * slope + half;   /* row coordinate at column i's left edge */
        float ya = y0;
        for (int i = 0; i < n; ++i) {
            const float yb = fmaf((float) (i + 1), slope, y0);
            const float lo = fminf(ya, yb), hi = fmaxf(ya, yb);
            const float r0f = floorf(lo);
            const int r0 = (int) r0f;
            float v0 = (r0 >= 0 && r0 < n) ? __ldg(img + (size_t) r0 * n + i) : 0.0f;
            if (hi > r0f + 1.0f) {
                const float f = (r0f + 1.0f - lo) / (hi - lo);
                const float v1 = (r0 + 1 >= 0 && r0 + 1 < n) ? __ldg(img + (size_t) (r0 + 1) * n + i) : 0.0f;
                sum += len * (f * v0 + (1.0f - f) * v1);
            } else {
                sum += len * v0;
            }
            ya = yb;
        }
    }
    const size_t oidx = (size_t) slice * P.sino_stride + (size_t) angle * n + k;
    float result = P.src ? P.src[oidx] : 0.0f;
    result += P.scale * sum;
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

/* Grid (ceil(n / 32), ceil(n / 8), slices), block 32 x 8: thread = pixel. */
__global__ void __launch_bounds__(256) siddon_bp_kernel(SiddonBpArgs P)
{
    const int i = (int) (blockIdx.x * blockDim.x + threadIdx.x);
    const int j = (int) (blockIdx.y * blockDim.y + threadIdx.y);
    const int slice = (int) blockIdx.z;
    const int n = P.n;
    if (i >= n || j >= n)
        return;
    const float half = 0.5f * (float) n;
    const float X = ((float) i + 0.5f) - half, Y = ((float) j + 0.5f) - half;
    const float *sino = P.sino + (size_t) slice * P.sino_stride;
    const size_t pix = (size_t) slice * P.vol_stride + (size_t) j * n + i;
    float v = P.base ? P.base[pix] : 0.0f;
    for (int s = 0; s < P.n_subsets; ++s) {
        float sum = 0.0f;
        for (unsigned int q = 0; q < P.sub_n[s]; ++q) {
            const int angle = (int) (P.sub_offset[s] + q);
            const float sr = __ldg(P.sinv + angle), cr = __ldg(P.cosv + angle);
            const float r = sqrtf(sr * sr + cr * cr), ir = 1.0f / r;
            const float a = fabsf(cr) * ir, b = fabsf(sr) * ir;
            /* X cos - Y sin, kept as s + e with both products' rounding errors
             * (exact by FMA) and the difference's (TwoSum), so that the small
             * offset of a bin from the centre is computed without cancellation */
            /* (explicit rounding: no contraction may merge these steps) */
            const float pa = __fmul_rn(X, cr), pb = __fmul_rn(Y, sr);
            const float ea = fmaf(X, cr, -pa), eb = fmaf(Y, sr, -pb);
            const float s = __fsub_rn(pa, pb);
            const float bv = __fsub_rn(s, pa);
            const float es = __fadd_rn(__fsub_rn(pa, __fsub_rn(s, bv)), __fsub_rn(-pb, bv));
            const float e = __fadd_rn(es, __fsub_rn(ea, eb));
            const float uc = s + P.axis;                    /* bin coordinate of the centre (bounds only) */
            const float w = 0.5f * (a + b), p = 0.5f * fabsf(a - b);
            const float h = 1.0f / fmaxf(a, b);
            const float ab = a * b;
            /* bins k with |k + 0.5 - uc| / r < w: at most two */
            const int k0 = max(0, (int) ceilf(uc - w * r - 0.5f));
            const int k1 = min(n - 1, (int) floorf(uc + w * r - 0.5f));
            const float *row = sino + (size_t) angle * n;
            for (int k = k0; k <= k1; ++k) {
                const float dd = fabsf(__fsub_rn(__fsub_rn(__fsub_rn((float) k + 0.5f, P.axis), s), e)) * ir;
                float L;
                if (dd <= p)
                    L = h;
                else if (dd < w)
                    L = (w - dd) / ab;
                else
                    L = 0.0f;
                sum += L * __ldg(row + k);
            }
        }
        v += P.relax * sum;
    }
    P.dst[pix] = v;
}

}  // namespace

extern "C" int udev_siddon_fp(udev *d, const udev_geom *g, int a0, int na, const float *vol, const float *src,
                              const float *w, int w_shared, float *out, float scale, int n_slices)
{
    if (n_slices <= 0 || na <= 0)
        return UFOIR_OK;
    const int n = g->n_dets;
    if (a0 < 0 || a0 + na > g->n_angles || n < 1 || n_slices > 65535 || na > 65535) {
        udev_set_error(d, "siddon_fp: angles [%d, %d) of %d, %d slices out of range", a0, a0 + na, g->n_angles,
                       n_slices);
        return UFOIR_ERR_INVALID;
    }
    UDEV_BIND(d);
    SiddonFpArgs A;
    A.vol = vol;
    A.src = src;
    A.w = w;
    A.out = out;
    A.sinv = g->d_sin;
    A.cosv = g->d_cos;
    A.n = n;
    A.a0 = a0;
    A.na = na;
    A.axis = g->axis;
    A.scale = scale;
    A.vol_stride = (long long) n * n;
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
    dim3 grid(udev_div_up(n, 32), udev_div_up(n, 8), (unsigned int) n_slices);
    siddon_bp_kernel<<<grid, dim3(32, 8), 0, d->stream>>>(A);
    return udev_after_launch(d, "siddon_bp_kernel");
}
