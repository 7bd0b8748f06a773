/*
 * udev_sart.cu - the per-angle projections of SART (and of ASD-POCS, whose
 * data-fidelity step is SART): one angle's forward projection, then one
 * angle's backprojection, n_angles times per sweep (sart-task.c:209-217).
 *
 * One angle is only n rays of n samples, so a ray-per-thread kernel leaves
 * the GPU idle. Here a ray is cut into its 64-sample blocks (the blocks the
 * reference sums separately, projector-parallel-joseph.cl:81-93) and every
 * (ray, block) pair is a thread. The coordinate at each block start is the
 * float recurrence c += step replayed from the ray start; it depends only on
 * the geometry, so it is tabulated once per job (block_starts_kernel) and a
 * block's thread starts from the table with the exact value the sequential
 * walk reaches. The block sums of a ray are then added in order in shared
 * memory, exactly as the reference adds its inner sums.
 *
 * Rays walk rows of a row-major image: vertical rays the volume, horizontal
 * rays its transpose. SART keeps the volume in the layout of the current
 * direction run (the angles of [0, pi) form three runs) and transposes it
 * at the two run boundaries; the per-angle backprojection updates either
 * layout in place.
 */
#include <cuda_runtime.h>

#include "joseph.cuh"
#include "udev_internal.cuh"

namespace {

constexpr int kBlock = 64;          /* samples per block (the reference's BLOCK_SIZE) */
constexpr int kRaysPerCta = 8;      /* lanes: 8 rays x 4 blocks per warp */
constexpr int kMaxBlocks = 128;     /* n <= 8192 */
constexpr int kMaxThreads = 512;          /* 16 warps: blocks beyond them loop */

__global__ void __launch_bounds__(256) block_starts_kernel(const float *__restrict__ sinv,
                                                           const float *__restrict__ cosv,
                                                           const unsigned char *__restrict__ dirs, int n,
                                                           int n_blocks, float axis, float *__restrict__ table)
{
    const int s = (int) (blockIdx.x * blockDim.x + threadIdx.x);
    const int a = (int) blockIdx.y;
    if (s >= n)
        return;
    const joseph::AxisConsts k = joseph::axis_consts(n, axis);
    float det_step, step;
    joseph::ray_steps((int) dirs[a], sinv[a], cosv[a], det_step, step);
    float c = joseph::ray_start(k, s, n, det_step, step);
    float *t = table + (size_t) a * n_blocks * n + s;
    for (int b = 0; b < n_blocks; ++b) {
        t[(size_t) b * n] = c;
#pragma unroll 8
        for (int r = 0; r < kBlock; ++r)
            c = __fadd_rn(c, step);
    }
}

struct FpAngleArgs {
    const float *img;       /* rows walked by this angle's rays */
    const float *table;     /* [n_angles][n_blocks][n] block-start coordinates */
    const float *src;
    const float *w;
    float *out;
    const float *sinv;
    const float *cosv;
    int n;
    int n_blocks;
    int angle;
    int dir;
    float axis;
    float scale;
    long long img_stride;
    long long sino_stride;
    long long w_stride;
};

/*
 * out = (src + scale * S) [* w] for the rays of one angle.
 *
 * A warp takes one 64-sample block of 8 adjacent rays; lane = 8 * q + ray,
 * and quarter q computes samples 16q .. 16q + 15 of the block. The quarter's
 * start coordinate is the block start (table) advanced by 16q steps of the
 * same float recurrence. The 16 sample values are computed independently
 * (all loads in flight together); the block's in-order sum is then folded
 * through the quarters with shuffles, so the additions happen in exactly the
 * reference's order. Samples in rows >= n read the zero border and add 0,
 * as in the reference's fixed 64-sample blocks.
 * Grid (ceil(n / 8), slices); block 32 * min(kMaxWarps, n_blocks) threads.
 */
__global__ void __launch_bounds__(kMaxThreads) fp_angle_kernel(FpAngleArgs P)
{
    __shared__ float bsum[kMaxBlocks][kRaysPerCta];
    const int lane = (int) (threadIdx.x & 31);
    const int ray = lane & (kRaysPerCta - 1);
    const int q = lane >> 3;
    const int s = (int) blockIdx.x * kRaysPerCta + ray;
    const int sc = min(s, P.n - 1);          /* lanes past the last ray compute a copy and write nothing */
    const int slice = (int) blockIdx.y;
    const int n = P.n;
    float det_step, step;
    joseph::ray_steps(P.dir, P.sinv[P.angle], P.cosv[P.angle], det_step, step);
    const float *img = P.img + (size_t) slice * P.img_stride;

    for (int b = (int) (threadIdx.x >> 5); b < P.n_blocks; b += (int) (blockDim.x >> 5)) {
        float c = P.table[((size_t) P.angle * P.n_blocks + b) * n + sc];
        for (int k = 0; k < 16 * q; ++k)
            c = __fadd_rn(c, step);
        const int row0 = b * kBlock + 16 * q;
        int i0[16];
        float t[16], va[16], vb[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            joseph::lerp_coord(c, i0[k], t[k]);
            c = __fadd_rn(c, step);
        }
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const float *rr = img + (size_t) min(row0 + k, n - 1) * n;
            va[k] = __ldg(rr + min(max(i0[k], 0), n - 1));
            vb[k] = __ldg(rr + min(max(i0[k] + 1, 0), n - 1));
        }
        float v[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const bool in_row = row0 + k < n;
            const float t0 = in_row && (unsigned) i0[k] < (unsigned) n ? va[k] : 0.0f;
            const float t1 = in_row && (unsigned) (i0[k] + 1) < (unsigned) n ? vb[k] : 0.0f;
            v[k] = joseph::lerp(t[k], t0, t1);
        }
        /* inner = (((0 + v_0) + v_1) + ... + v_63), quarter by quarter */
        float run = 0.0f;
#pragma unroll
        for (int stage = 0; stage < 4; ++stage) {
            if (q == stage) {
#pragma unroll
                for (int k = 0; k < 16; ++k)
                    run = __fadd_rn(run, v[k]);
            }
            const float from_prev = __shfl_up_sync(0xffffffffu, run, kRaysPerCta);
            if (q == stage + 1)
                run = from_prev;
        }
        if (q == 3)
            bsum[b][ray] = run;
    }
    __syncthreads();
    if (threadIdx.x < kRaysPerCta && s < n) {
        const size_t oidx = (size_t) slice * P.sino_stride + (size_t) P.angle * n + s;
        float result = P.src[oidx];
        const joseph::AxisConsts k = joseph::axis_consts(n, P.axis);
        if (!joseph::detector_inactive(k, s)) {
            float detected = 0.0f;
            for (int j = 0; j < P.n_blocks; ++j)
                detected = __fadd_rn(detected, bsum[j][ray]);
            result = __fadd_rn(result, __fmul_rn(detected, P.scale));
        }
        if (P.w)
            result = __fmul_rn(result, P.w[(size_t) slice * P.w_stride + (size_t) P.angle * n + s]);
        P.out[oidx] = result;
    }
}

struct BpAngleArgs {
    const float *sino;
    float *vol;
    int n;
    int angle;
    int transposed;     /* vol holds the transpose: element (i, j) is pixel x = i, y = j */
    float os, shift, e0, e1;   /* origin shift, os - ros, clamp edges (…joseph.cl:174-187) */
    float sn, cs;
    float relax;
    const float *relax_dev;
    long long vol_stride;
    long long sino_stride;
};

/* vol = vol + relax * (0 + sample) for one angle (…joseph.cl:158-218 with a
 * one-angle subset). Grid (ceil(n / 128), ceil(n / 8), slices), block 32 x 8;
 * a thread updates 4 consecutive storage columns of one storage row, with
 * 16-byte loads and stores when rows are 16-byte aligned (VEC). */
template <bool VEC>
__global__ void __launch_bounds__(256) bp_angle_kernel(BpAngleArgs P)
{
    const int j = (int) (blockIdx.y * blockDim.y + threadIdx.y);   /* storage row */
    const int i_first = (int) (blockIdx.x * blockDim.x + threadIdx.x) * 4;
    const int slice = (int) blockIdx.z;
    const int n = P.n;
    if (j >= n || i_first >= n)
        return;
    const float *r = P.sino + (size_t) slice * P.sino_stride + (size_t) P.angle * n;
    const float relax = P.relax_dev ? *P.relax_dev : P.relax;
    const float fJ = __fsub_rn(__fadd_rn((float) j, 0.5f), P.os);
    float *row = P.vol + (size_t) slice * P.vol_stride + (size_t) j * n;
    float v[4];
    if (VEC) {
        const float4 x4 = *reinterpret_cast<const float4 *>(row + i_first);
        v[0] = x4.x;
        v[1] = x4.y;
        v[2] = x4.z;
        v[3] = x4.w;
    } else {
#pragma unroll
        for (int h = 0; h < 4; ++h)
            v[h] = i_first + h < n ? row[i_first + h] : 0.0f;
    }
#pragma unroll
    for (int h = 0; h < 4; ++h) {
        const int i = i_first + h;   /* storage column */
        const float fI = __fsub_rn(__fadd_rn((float) i, 0.5f), P.os);
        const float fX = P.transposed ? fJ : fI;
        const float fY = P.transposed ? fI : fJ;
        float sc = __fadd_rn(__fsub_rn(__fmul_rn(fX, P.cs), __fmul_rn(fY, P.sn)), P.shift);
        if (sc > P.e1)
            sc = P.e1;
        else if (sc < P.e0)
            sc = P.e0;
        int i0;
        float t;
        joseph::lerp_coord(sc, i0, t);
        const float sum =
            __fadd_rn(0.0f, joseph::lerp(t, joseph::texel(r, i0, n), joseph::texel(r, i0 + 1, n)));
        v[h] = __fadd_rn(v[h], __fmul_rn(relax, sum));
    }
    if (VEC) {
        *reinterpret_cast<float4 *>(row + i_first) = make_float4(v[0], v[1], v[2], v[3]);
    } else {
#pragma unroll
        for (int h = 0; h < 4; ++h)
            if (i_first + h < n)
                row[i_first + h] = v[h];
    }
}

}  // namespace

extern "C" size_t udev_fp_block_starts_floats(int n, int n_angles)
{
    const int nb = (n + kBlock - 1) / kBlock;
    return (size_t) n_angles * nb * n;
}

extern "C" int udev_fp_block_starts(udev *d, const udev_geom *g, float *table)
{
    const int n = g->n_dets;
    if (n <= 0 || g->n_angles <= 0)
        return UFOIR_OK;
    if (n > kMaxBlocks * kBlock || g->n_angles > 65535) {
        udev_set_error(d, "sart: n = %d, n_angles = %d beyond the per-angle kernels' limits (%d, 65535)", n,
                       g->n_angles, kMaxBlocks * kBlock);
        return UFOIR_ERR_UNSUPPORTED;
    }
    UDEV_BIND(d);
    const int nb = (n + kBlock - 1) / kBlock;
    dim3 grid(udev_div_up(n, 256), (unsigned int) g->n_angles);
    block_starts_kernel<<<grid, 256, 0, d->stream>>>(g->d_sin, g->d_cos, g->d_dir, n, nb, g->axis, table);
    return udev_after_launch(d, "block_starts_kernel");
}

extern "C" int udev_fp_angle(udev *d, const udev_geom *g, int angle, int dir, const float *table, const float *img,
                             const float *src, const float *w, int w_shared, float *out, float scale, int n_slices)
{
    if (n_slices <= 0)
        return UFOIR_OK;
    const int n = g->n_dets;
    if (angle < 0 || angle >= g->n_angles || n > kMaxBlocks * kBlock || n_slices > 65535) {
        udev_set_error(d, "fp_angle: angle %d of %d, n = %d, %d slices out of range", angle, g->n_angles, n,
                       n_slices);
        return UFOIR_ERR_INVALID;
    }
    UDEV_BIND(d);
    FpAngleArgs A;
    A.img = img;
    A.table = table;
    A.src = src;
    A.w = w;
    A.out = out;
    A.sinv = g->d_sin;
    A.cosv = g->d_cos;
    A.n = n;
    A.n_blocks = (n + kBlock - 1) / kBlock;
    A.angle = angle;
    A.dir = dir;
    A.axis = g->axis;
    A.scale = scale;
    A.img_stride = (long long) n * n;
    A.sino_stride = (long long) g->n_angles * n;
    A.w_stride = w_shared ? 0 : A.sino_stride;
    const int warps = A.n_blocks < kMaxThreads / 32 ? A.n_blocks : kMaxThreads / 32;
    const int threads = 32 * warps;
    dim3 grid(udev_div_up(n, kRaysPerCta), (unsigned int) n_slices);
    fp_angle_kernel<<<grid, threads, 0, d->stream>>>(A);
    return udev_after_launch(d, "fp_angle_kernel");
}

extern "C" int udev_bp_angle(udev *d, const udev_geom *g, int angle, float sn, float cs, const float *sino,
                             float *vol, int transposed, float relax, const float *relax_dev, int n_slices)
{
    if (n_slices <= 0)
        return UFOIR_OK;
    const int n = g->n_dets;
    if (angle < 0 || angle >= g->n_angles || n_slices > 65535) {
        udev_set_error(d, "bp_angle: angle %d of %d, %d slices out of range", angle, g->n_angles, n_slices);
        return UFOIR_ERR_INVALID;
    }
    UDEV_BIND(d);
    /* the per-launch constants of …joseph.cl:174-187 (float arithmetic,
     * the multiplications and divisions by 2 exact) */
    const float w = (float) n, axis = g->axis;
    const float required_width = axis * 2.0f;
    const float diff = w - required_width;
    const float ros = diff / 2.0f, os = w / 2.0f;
    const float half = diff < 0.0f ? w - axis : axis;
    BpAngleArgs A;
    A.sino = sino;
    A.vol = vol;
    A.n = n;
    A.angle = angle;
    A.transposed = transposed;
    A.os = os;
    A.shift = os - ros;
    A.e0 = axis - half + 0.5f;
    A.e1 = axis + half - 0.5f;
    A.sn = sn;
    A.cs = cs;
    A.relax = relax;
    A.relax_dev = relax_dev;
    A.vol_stride = (long long) n * n;
    A.sino_stride = (long long) g->n_angles * n;
    dim3 grid(udev_div_up(n, 128), udev_div_up(n, 8), (unsigned int) n_slices);
    const bool vec = (n % 4) == 0 && (reinterpret_cast<uintptr_t>(vol) & 15) == 0;
    if (vec)
        bp_angle_kernel<true><<<grid, dim3(32, 8), 0, d->stream>>>(A);
    else
        bp_angle_kernel<false><<<grid, dim3(32, 8), 0, d->stream>>>(A);
    return udev_after_launch(d, "bp_angle_kernel");
}
