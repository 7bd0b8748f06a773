/*
 * udev_project.cu - Joseph forward projector, pixel-driven backprojector and
 * the volume transpose used by the forward projector.
 *
 * Forward projection (replaces FP_hor / FP_vert, projector-parallel-joseph.cl:36-156):
 * one thread per ray walks the rows of a row-major image. Vertical rays
 * (|sin| <= |cos|) walk the rows of the volume and interpolate along x;
 * horizontal rays walk the rows of the transposed volume, so both kinds
 * read along rows and a warp's 32 neighbouring detectors touch a few
 * consecutive cache lines per step. Samples are summed per ray in blocks of
 * 64 in the reference's order, with the float coordinate recurrence, so the
 * sum is the reference's to the last bit.
 *
 * Backprojection (replaces BP, projector-parallel-joseph.cl:158-218): one
 * thread per pixel gathers every angle of every subset in order; no atomics,
 * deterministic. The epilogue fuses the SIRT/SART updates
 * (v * pixel_weight + x) so a method iteration is one FP and one BP launch.
 */
#include <cuda_runtime.h>

#include "joseph.cuh"
#include "udev_internal.cuh"

namespace {

constexpr int kMaxSubsetsPerLaunch = 16;

struct FpArgs {
    const float *vol;
    const float *volT;
    const float *src;
    const float *w;
    float *out;
    const float *sinv;
    const float *cosv;
    const unsigned char *dir;
    int n;
    int a0;
    int dir_override;
    int have_volT;
    float axis;
    float scale;
    long long vol_stride;
    long long sino_stride;
    long long w_stride;
};

__global__ void __launch_bounds__(128) fp_rows_kernel(FpArgs A)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int a = A.a0 + (int) blockIdx.y;
    const int slice = (int) blockIdx.z;
    const int n = A.n;
    if (s >= n)
        return;

    const size_t oidx = (size_t) slice * A.sino_stride + (size_t) a * n + s;
    const float srcv = A.src[oidx];
    const joseph::AxisConsts k = joseph::axis_consts(n, A.axis);

    float result;
    if (joseph::detector_inactive(k, s)) {
        result = srcv;
    } else {
        const int dir = A.dir_override >= 0 ? A.dir_override : (int) A.dir[a];
        float det_step, slice_step;
        joseph::ray_steps(dir, A.sinv[a], A.cosv[a], det_step, slice_step);
        /* Row-major walk: vertical rays on vol, horizontal rays on volT;
         * without volT horizontal rays read vol column by column. */
        const bool transposed_read = dir == 0 && !A.have_volT;
        const float *img = (dir == 0 && A.have_volT ? A.volT : A.vol) + (size_t) slice * A.vol_stride;
        const size_t row_step = transposed_read ? 1 : (size_t) n;
        const int col_step = transposed_read ? n : 1;
        float c = joseph::ray_start(k, s, n, det_step, slice_step);

        /* Rows beyond the image (the 64-block padding) read only the zero
         * border and add nothing; the walk stops at row n - 1. */
        float detected = 0.0f;
        int row = 0;
        const int nb = joseph::n_blocks(n);
        for (int j = 0; j < nb && row < n; ++j) {
            float inner = 0.0f;
            const int end = min(row + 64, n);
#pragma unroll 4
            for (; row < end; ++row) {
                const float *r = img + (size_t) row * row_step;
                int i0;
                float t;
                joseph::lerp_coord(c, i0, t);
                const float t0 = (i0 >= 0 && i0 < n) ? __ldg(r + (size_t) i0 * col_step) : 0.0f;
                const float t1 = (i0 + 1 >= 0 && i0 + 1 < n) ? __ldg(r + (size_t) (i0 + 1) * col_step) : 0.0f;
                inner = __fadd_rn(inner, joseph::lerp(t, t0, t1));
                c = __fadd_rn(c, slice_step);
            }
            detected = __fadd_rn(detected, inner);
        }
        result = __fadd_rn(srcv, __fmul_rn(detected, A.scale));
    }
    if (A.w)
        result = __fmul_rn(result, A.w[(size_t) slice * A.w_stride + (size_t) a * n + s]);
    A.out[oidx] = result;
}

struct BpArgs {
    const float *sino;
    const float *base;
    const float *cw;
    const float *add;
    float *dst;
    const float *sinv;
    const float *cosv;
    int n;
    float axis;
    float relax;
    long long vol_stride;
    long long sino_stride;
    long long cw_stride;
    int n_subsets;
    unsigned int sub_offset[kMaxSubsetsPerLaunch];
    unsigned int sub_n[kMaxSubsetsPerLaunch];
};

__global__ void __launch_bounds__(256) bp_gather_kernel(BpArgs A)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int slice = (int) blockIdx.z;
    const int n = A.n;
    if (x >= n || y >= n)
        return;

    const joseph::AxisConsts k = joseph::axis_consts(n, A.axis);
    float e0, e1;
    joseph::bp_edges(k, n, A.axis, e0, e1);
    const float shift = __fsub_rn(k.os, k.ros);
    const float fX = __fsub_rn(__fadd_rn((float) x, 0.5f), k.os);
    const float fY = __fsub_rn(__fadd_rn((float) y, 0.5f), k.os);

    const size_t p = (size_t) slice * A.vol_stride + (size_t) y * n + x;
    const float *sino = A.sino + (size_t) slice * A.sino_stride;
    float v = A.base ? A.base[p] : 0.0f;

    for (int si = 0; si < A.n_subsets; ++si) {
        float sum = 0.0f;
        const unsigned int off = A.sub_offset[si];
        const unsigned int cnt = A.sub_n[si];
        for (unsigned int i = 0; i < cnt; ++i) {
            const unsigned int a = off + i;
            const float sn = __ldg(A.sinv + a);
            const float cs = __ldg(A.cosv + a);
            float sc = __fadd_rn(__fsub_rn(__fmul_rn(fX, cs), __fmul_rn(fY, sn)), shift);
            if (sc > e1)
                sc = e1;
            else if (sc < e0)
                sc = e0;
            int i0;
            float t;
            joseph::lerp_coord(sc, i0, t);
            const float *r = sino + (size_t) a * n;
            sum = __fadd_rn(sum, joseph::lerp(t, joseph::texel(r, i0, n), joseph::texel(r, i0 + 1, n)));
        }
        v = __fadd_rn(v, __fmul_rn(A.relax, sum));
    }
    if (A.cw)
        v = __fmul_rn(v, A.cw[(size_t) slice * A.cw_stride + (size_t) y * n + x]);
    if (A.add)
        v = __fadd_rn(v, A.add[p]);
    A.dst[p] = v;
}

__global__ void __launch_bounds__(256) transpose_kernel(const float *__restrict__ in,
                                                        float *__restrict__ out, int n,
                                                        long long stride)
{
    __shared__ float tile[32][33];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    const size_t base = (size_t) blockIdx.z * stride;
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int x = bx + threadIdx.x, y = by + j;
        if (x < n && y < n)
            tile[j][threadIdx.x] = in[base + (size_t) y * n + x];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int x = by + threadIdx.x, y = bx + j;
        if (x < n && y < n)
            out[base + (size_t) y * n + x] = tile[threadIdx.x][j];
    }
}

}  // namespace

extern "C" int udev_fp(udev *d, const udev_geom *g, int a0, int na, int dir_override,
                       const float *vol, const float *volT, const float *src, const float *w,
                       int w_shared, float *out, float scale, int n_slices)
{
    if (na <= 0 || n_slices <= 0)
        return UFOIR_OK;
    if (a0 < 0 || a0 + na > g->n_angles) {
        udev_set_error(d, "fp: angle range [%d, %d) outside [0, %d)", a0, a0 + na, g->n_angles);
        return UFOIR_ERR_INVALID;
    }
    UDEV_BIND(d);
    FpArgs A;
    A.vol = vol;
    A.volT = volT ? volT : vol;
    A.have_volT = volT != nullptr;
    A.src = src;
    A.w = w;
    A.out = out;
    A.sinv = g->d_sin;
    A.cosv = g->d_cos;
    A.dir = g->d_dir;
    A.n = g->n_dets;
    A.a0 = a0;
    A.dir_override = dir_override;
    A.axis = g->axis;
    A.scale = scale;
    A.vol_stride = (long long) g->n_dets * g->n_dets;
    A.sino_stride = (long long) g->n_angles * g->n_dets;
    A.w_stride = w_shared ? 0 : A.sino_stride;
    for (int done = 0; done < n_slices;) {
        const int chunk = n_slices - done > 65535 ? 65535 : n_slices - done;
        FpArgs B = A;
        B.vol += (size_t) done * A.vol_stride;
        B.volT += (size_t) done * A.vol_stride;
        B.src += (size_t) done * A.sino_stride;
        if (B.w)
            B.w += (size_t) done * A.w_stride;
        B.out += (size_t) done * A.sino_stride;
        dim3 grid(udev_div_up(g->n_dets, 128), (unsigned int) na, (unsigned int) chunk);
        fp_rows_kernel<<<grid, 128, 0, d->stream>>>(B);
        int rc = udev_after_launch(d, "fp_rows_kernel");
        if (rc)
            return rc;
        done += chunk;
    }
    return UFOIR_OK;
}

extern "C" int udev_transpose(udev *d, const float *in, float *out, int n, int n_slices)
{
    if (n_slices <= 0)
        return UFOIR_OK;
    UDEV_BIND(d);
    const long long stride = (long long) n * n;
    for (int done = 0; done < n_slices;) {
        const int chunk = n_slices - done > 65535 ? 65535 : n_slices - done;
        dim3 grid(udev_div_up(n, 32), udev_div_up(n, 32), (unsigned int) chunk);
        transpose_kernel<<<grid, dim3(32, 8), 0, d->stream>>>(in + (size_t) done * stride,
                                                            out + (size_t) done * stride, n, stride);
        int rc = udev_after_launch(d, "transpose_kernel");
        if (rc)
            return rc;
        done += chunk;
    }
    return UFOIR_OK;
}

extern "C" int udev_bp(udev *d, const udev_geom *g, const ufoir_subset *subsets, int n_subsets,
                       const float *sino, const float *base, const float *cw, int cw_shared,
                       const float *add, float *dst, float relax, int n_slices)
{
    if (n_slices <= 0)
        return UFOIR_OK;
    size_t total = 0;
    for (int i = 0; i < n_subsets; i++) {
        if (subsets[i].offset + (size_t) subsets[i].n > (size_t) g->n_angles) {
            udev_set_error(d, "bp: subset [%u, %u) outside [0, %d)", subsets[i].offset,
                           subsets[i].offset + subsets[i].n, g->n_angles);
            return UFOIR_ERR_INVALID;
        }
        total += subsets[i].n;
    }
    /* The tiled kernel clamps with min/max, which equals the reference's
     * if / else-if clamp (…joseph.cl:206-210) only while e0 <= e1; an axis
     * within half a pixel of the image edge gives e0 > e1 and goes to the
     * gather kernel, which follows the reference's form. */
    const float n_f = (float) g->n_dets;
    const float half = n_f - g->axis * 2.0f < 0.0f ? n_f - g->axis : g->axis;
    const bool edges_ordered = g->axis - half + 0.5f <= g->axis + half - 0.5f;
    /* many angles: the tiled kernel (shared-memory sinogram windows) */
    if (total >= 16 && n_subsets <= 16 && edges_ordered)
        return udev_bp_tiles(d, g, subsets, n_subsets, sino, base, cw, cw_shared, add, dst, relax, n_slices);
    UDEV_BIND(d);
    BpArgs A;
    A.sino = sino;
    A.cw = nullptr;
    A.add = nullptr;
    A.dst = dst;
    A.sinv = g->d_sin;
    A.cosv = g->d_cos;
    A.n = g->n_dets;
    A.axis = g->axis;
    A.relax = relax;
    A.vol_stride = (long long) g->n_dets * g->n_dets;
    A.sino_stride = (long long) g->n_angles * g->n_dets;
    A.cw_stride = cw_shared ? 0 : A.vol_stride;

    /* Subsets are applied in order; more than kMaxSubsetsPerLaunch are
     * chained through dst, and the epilogue runs in the last launch only. */
    int first = 0;
    do {
        const int cnt = n_subsets - first > kMaxSubsetsPerLaunch ? kMaxSubsetsPerLaunch : n_subsets - first;
        const bool last = first + cnt >= n_subsets;
        A.n_subsets = cnt;
        for (int i = 0; i < cnt; i++) {
            A.sub_offset[i] = subsets[first + i].offset;
            A.sub_n[i] = subsets[first + i].n;
        }
        A.base = first == 0 ? base : dst;
        A.cw = last ? cw : nullptr;
        A.add = last ? add : nullptr;
        for (int done = 0; done < n_slices;) {
            const int chunk = n_slices - done > 65535 ? 65535 : n_slices - done;
            BpArgs B = A;
            B.sino += (size_t) done * A.sino_stride;
            if (B.base)
                B.base += (size_t) done * A.vol_stride;
            if (B.cw)
                B.cw += (size_t) done * A.cw_stride;
            if (B.add)
                B.add += (size_t) done * A.vol_stride;
            B.dst += (size_t) done * A.vol_stride;
            dim3 grid(udev_div_up(g->n_dets, 32), udev_div_up(g->n_dets, 8), (unsigned int) chunk);
            bp_gather_kernel<<<grid, dim3(32, 8), 0, d->stream>>>(B);
            int rc = udev_after_launch(d, "bp_gather_kernel");
            if (rc)
                return rc;
            done += chunk;
        }
        first += cnt;
    } while (first < n_subsets);
    return UFOIR_OK;
}
