/*
 * udev_sart.cu - the per-angle projections of SART (and of ASD-POCS, whose
 * data-fidelity step is SART): one angle's forward projection, then one
 * angle's backprojection, n_angles times per sweep (sart-task.c:209-217).
 *
 * One angle is only n rays of n samples, so a ray-per-thread kernel leaves
 * the GPU idle. A ray is cut into its 64-sample blocks (the blocks the
 * reference sums separately, projector-parallel-joseph.cl:81-93), and the
 * blocks are computed in parallel. The coordinate at each block start is the
 * float recurrence c += step replayed from the ray start; it depends only on
 * the geometry, so it is tabulated once per job (block_starts_kernel), and a
 * block starts from the table with the exact value the sequential walk
 * reaches. The block sums of a ray are then added in order, exactly as the
 * reference adds its inner sums.
 *
 * Rays walk rows of a row-major image: vertical rays the volume, horizontal
 * rays its transpose. SART keeps the volume in the layout of the current
 * direction run (the angles of [0, pi) form three runs) and transposes it at
 * the two run boundaries; the per-angle backprojection updates either layout
 * in place. Two sets of kernels:
 *  - the padded path (sart_fp_kernel, sart_bp_kernel, sart_copy_kernel):
 *    zero-padded copies of the volume, a cluster of CTAs per group of 64
 *    rays whose block sums meet in distributed shared memory, and a tiled
 *    backprojection with the tile's sinogram span in shared memory;
 *  - the general kernels (fp_angle_kernel, bp_angle_kernel) on the
 *    unpadded volume, for geometries whose backprojection clamp edges cross
 *    (an axis within half a pixel of the image edge).
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

/*
 * The padded sweep layout. While a sweep runs, the volume lives in one of
 * two padded copies: V (row y holds the pixels of row y) for vertical
 * angles, H (row x holds column x, the transpose) for horizontal ones. A
 * padded row has kSartPadL zero columns, the n pixels (16-byte aligned),
 * and at least 3 zero columns; the rows run up to whole 64-row blocks, the
 * rows beyond n zero. Forward-projection rays then read their taps without
 * bounds checks: the coordinate is clamped to [-1, n + 1], where both taps
 * outside the image are pad zeros, as the reference's zero border gives, and
 * samples in rows >= n read zero rows (…joseph.cl:81-93 sums fixed
 * 64-sample blocks). The backprojection updates only the pixels, so the
 * pads stay zero.
 */
constexpr int kSartPadL = 4;
constexpr int kErrSpan = 4;      /* error word: a backprojection span exceeded its buffer */

__host__ __device__ inline int sart_pitch(int n)
{
    return (n + kSartPadL + 3 + 3) / 4 * 4;
}

__host__ __device__ inline int sart_rows(int n)
{
    return (n + kBlock - 1) / kBlock * kBlock;
}

/* dst = src (or its transpose) for n x n interiors, each addressed by a row
 * pitch and a column offset. Grid (ceil(n/32), ceil(n/32), slices), block 32 x 8. */
__global__ void __launch_bounds__(256) sart_copy_kernel(const float *__restrict__ src, int sp, int so,
                                                        long long sstride, float *__restrict__ dst, int dp, int dof,
                                                        long long dstride, int n, int transpose)
{
    __shared__ float tile[32][33];
    const int bx = (int) blockIdx.x * 32, by = (int) blockIdx.y * 32;
    const int tx = (int) threadIdx.x;
    src += (size_t) blockIdx.z * sstride;
    dst += (size_t) blockIdx.z * dstride;
    if (!transpose) {
        for (int k = (int) threadIdx.y; k < 32; k += 8) {
            const int y = by + k, x = bx + tx;
            if (x < n && y < n)
                dst[(size_t) y * dp + dof + x] = src[(size_t) y * sp + so + x];
        }
        return;
    }
    for (int k = (int) threadIdx.y; k < 32; k += 8) {
        const int y = by + k, x = bx + tx;
        tile[k][tx] = (x < n && y < n) ? src[(size_t) y * sp + so + x] : 0.0f;
    }
    __syncthreads();
    for (int k = (int) threadIdx.y; k < 32; k += 8) {
        const int y = bx + k, x = by + tx;   /* dst(y, x) = src(x, y) */
        if (x < n && y < n)
            dst[(size_t) y * dp + dof + x] = tile[tx][k];
    }
}

struct SartFpArgs {
    const float *img;          /* padded layout walked by this angle's rays, [slices][rows][pitch] */
    const float *table;        /* [n_angles][n_blocks][n] block-start coordinates */
    const float *next_table;   /* the next launch's rows of it, pulled into L2 ahead (or null) */
    const float *src;
    const float *w;
    float *out;
    const float *sinv;
    const float *cosv;
    int n;
    int n_blocks;
    int angle;
    int dir;
    int pitch;
    int cluster;               /* CTAs per ray group (the cluster size) */
    float axis;
    float scale;
    float neg_zero;
    long long img_stride;
    long long sino_stride;
    long long w_stride;
};

constexpr int kFpCluster = 8;                       /* CTAs per ray group at most (portable cluster) */
constexpr int kFpWideCluster = 16;                  /* the same, non-portable, for the segment form */
constexpr int kFpLocal = kMaxBlocks / kFpCluster;   /* blocks per CTA at most */
constexpr int kRemoteBatch = 16;                    /* block sums read over DSMEM per round */
constexpr size_t kPrefetchTableBytes = (size_t) 64 << 20;   /* block-start tables above this are prefetched */

/* Programmatic dependent launch: let the next kernel in the stream launch
 * now, and wait here until the previous one has completed and its writes are
 * visible (both return at once when the launch did not allow overlap). */
__device__ __forceinline__ void pdl_launch_next()
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__device__ __forceinline__ void pdl_wait_previous()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

__device__ __forceinline__ void cluster_sync_all()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

/* A float of CTA `rank`'s shared memory, at the address `local` has here.
 * Ordering against the writes comes from the cluster barrier before it, so
 * the loads may be issued back to back. */
__device__ __forceinline__ float ld_cluster(const float *local, int rank)
{
    uint32_t remote;
    float v;
    asm("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"((uint32_t) __cvta_generic_to_shared(local)), "r"(rank));
    asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(remote));
    return v;
}

/* The samples [row0, row0 + ROWS) of rays (s0, s1) of one block, from the
 * coordinates c at row0, in batches of K samples whose loads are all in
 * flight together: appended to the running sum (STREAM) or stored in v. */
template <int ROWS, int K, bool STREAM>
__device__ __forceinline__ void sart_fp_samples(const float *img, int pitch, float2 c, float2 st, float hi,
                                                float2 z2, float2 &run, float2 *v)
{
#pragma unroll 1
    for (int k0 = 0; k0 < ROWS; k0 += K) {
        float2 t[K];
        int ia[K], ib[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const float2 cc = make_float2(fminf(fmaxf(c.x, -1.0f), hi), fminf(fmaxf(c.y, -1.0f), hi));
            const float2 y = joseph::floor_any2(cc, t[k]);
            const int roff = (k0 + k) * pitch;
            ia[k] = __float_as_int(y.x) + roff;
            ib[k] = __float_as_int(y.y) + roff;
            c = joseph::add2(c, st);
        }
        float2 t0[K], t1[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            t0[k] = make_float2(__ldg(img + ia[k]), __ldg(img + ib[k]));
            t1[k] = make_float2(__ldg(img + ia[k] + 1), __ldg(img + ib[k] + 1));
        }
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if (STREAM)
                run = joseph::add2(run, joseph::lerp2(t[k], t0[k], t1[k], z2));
            else
                v[k] = joseph::lerp2(t[k], t0[k], t1[k], z2);
        }
    }
}

/* One batch of K samples of rays (s0, s1): fractions and both taps, loads
 * in flight until the batch is consumed. */
template <int K>
struct FpBatch {
    float2 t[K], t0[K], t1[K];
};

/* Issues the loads of rows [row0, row0 + K) and advances c past them. */
template <int K>
__device__ __forceinline__ void fp_batch_issue(FpBatch<K> &B, const float *img, int pitch, int row0, float2 &c,
                                               float2 st, float hi)
{
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const float2 cc = make_float2(fminf(fmaxf(c.x, -1.0f), hi), fminf(fmaxf(c.y, -1.0f), hi));
        const float2 y = joseph::floor_any2(cc, B.t[k]);
        const int roff = (row0 + k) * pitch;
        const int ia = __float_as_int(y.x) + roff, ib = __float_as_int(y.y) + roff;
        B.t0[k] = make_float2(__ldg(img + ia), __ldg(img + ib));
        B.t1[k] = make_float2(__ldg(img + ia + 1), __ldg(img + ib + 1));
        c = joseph::add2(c, st);
    }
}

template <int K>
__device__ __forceinline__ void fp_batch_add(const FpBatch<K> &B, float2 &run, float2 z2)
{
#pragma unroll
    for (int k = 0; k < K; ++k)
        run = joseph::add2(run, joseph::lerp2(B.t[k], B.t0[k], B.t1[k], z2));
}

/* The STREAM form of sart_fp_samples with two batches in flight: the loads
 * of batch b + 1 are issued before batch b is added. ROWS % (2 K) == 0. */
template <int ROWS, int K>
__device__ __forceinline__ void sart_fp_samples_2x(const float *img, int pitch, float2 c, float2 st, float hi,
                                                   float2 z2, float2 &run)
{
    static_assert(ROWS % (2 * K) == 0, "two whole batches per step");
    FpBatch<K> A, B;
    fp_batch_issue<K>(A, img, pitch, 0, c, st, hi);
#pragma unroll 1
    for (int k0 = 0; k0 < ROWS; k0 += 2 * K) {
        fp_batch_issue<K>(B, img, pitch, k0 + K, c, st, hi);
        fp_batch_add<K>(A, run, z2);
        if (k0 + 2 * K < ROWS)
            fp_batch_issue<K>(A, img, pitch, k0 + 2 * K, c, st, hi);
        fp_batch_add<K>(B, run, z2);
    }
}

/*
 * out = (src + scale * S) [* w] for the rays of one angle, on the padded layout.
 *
 * Lane l walks rays 64g + l and 64g + l + 32 together in packed FP32, so
 * every load instruction of a warp reads 32 adjacent rays' taps in one
 * image row. A ray's block starts at its table coordinate and advances by
 * the float recurrence c += step; each block's inner sum adds its 64
 * samples in order (…joseph.cl:84-92).
 *
 * The blocks of one group of 64 rays are spread over a cluster of C CTAs
 * (block b on CTA b mod C), each keeping its block sums in shared memory.
 * SEG == 4: the CTA's four warps cut each of its blocks into four 16-row
 * segments, computed with all loads in flight together, and fold the inner
 * sum through the segments in order (warp q continues the running sum of
 * warp q - 1), for few blocks per CTA. SEG == 1: each warp adds whole
 * blocks, for many. After a cluster barrier, CTA 0 reads the block sums
 * over distributed shared memory, adds them in block order and writes the
 * rays' results (…joseph.cl:93-100); a second barrier keeps every CTA's
 * shared memory alive until then. Grid (groups * C, 1, slices), cluster
 * (C, 1, 1), 32 W threads; K samples per batch of loads.
 */
template <int SEG, int K, int W, int MINB, bool PIPE = false>
__global__ void __launch_bounds__(32 * W, MINB) sart_fp_kernel(SartFpArgs P)
{
    __shared__ float bs_local[kFpLocal][64];
    __shared__ float2 run_s[32];
    const int lane = (int) (threadIdx.x & 31);
    const int warp = (int) (threadIdx.x >> 5);
    const int C = P.cluster;
    const int g = (int) blockIdx.x / C, rank = (int) blockIdx.x % C;
    const int slice = (int) blockIdx.z;
    const int n = P.n, nb = P.n_blocks;
    const int s0 = g * 64 + lane, s1 = s0 + 32;
    pdl_launch_next();
    /* The next angle's block starts (n_blocks x n floats, read once per sweep,
     * so from DRAM when the table outgrows L2) are pulled into L2 a BP ahead of
     * the FP that reads them: one 128-byte line per thread of the grid, within
     * the rows (the grid always has at least n_blocks * n / 32 threads). */
    if (P.next_table && slice == 0) {
        const size_t line = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
        if (line * 32 < (size_t) nb * n)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(P.next_table + line * 32));
    }

    /* CTA 0 fetches its rays' src and w early, before the grid dependency
     * wait. This is safe because src (the sinogram b) and w (the ray weights
     * R) are written only by kernels that do not trigger their dependents
     * early: every padded sweep starts with sart_copy_kernel, launched
     * without programmatic dependency, after the last write to b and R. A
     * kernel that updates b or R inside the sweep must move these loads
     * after pdl_wait_previous(). */
    const int sr = g * 64 + (int) threadIdx.x;
    const bool writer = rank == 0 && threadIdx.x < 64 && sr < n;
    const size_t oidx = (size_t) slice * P.sino_stride + (size_t) P.angle * n + sr;
    float src_v = 0.0f, w_v = 0.0f;
    if (writer) {
        src_v = P.src[oidx];
        if (P.w)
            w_v = P.w[(size_t) slice * P.w_stride + (size_t) P.angle * n + sr];
    }

    float det_step, step;
    joseph::ray_steps(P.dir, __ldg(P.sinv + P.angle), __ldg(P.cosv + P.angle), det_step, step);
    const float2 st = joseph::splat(step), z2 = joseph::splat(P.neg_zero);
    const float hi = (float) (n + 1);
    const float *tab = P.table + (size_t) P.angle * nb * n;
    const float *img0 = P.img + (size_t) slice * P.img_stride + kSartPadL - joseph::kFloorMagicBits;
    /* the volume was written by the previous kernel */
    pdl_wait_previous();

    if (SEG == 4) {
        for (int i = 0; rank + C * i < nb; ++i) {
            const int b = rank + C * i;
            const float *tb = tab + (size_t) b * n;
            float2 c = make_float2(__ldg(tb + min(s0, n - 1)), __ldg(tb + min(s1, n - 1)));
            for (int k = 0; k < 16 * warp; ++k)
                c = joseph::add2(c, st);
            float2 v[16], run = joseph::splat(0.0f);
            sart_fp_samples<16, 16, false>(img0 + (size_t) (b * kBlock + 16 * warp) * P.pitch, P.pitch, c, st, hi, z2,
                                       run, v);
            /* inner = (((0 + v_0) + v_1) + ... + v_63), segment by segment */
#pragma unroll
            for (int stage = 0; stage < 4; ++stage) {
                if (warp == stage) {
                    if (stage > 0)
                        run = run_s[lane];
#pragma unroll
                    for (int k = 0; k < 16; ++k)
                        run = joseph::add2(run, v[k]);
                    if (stage < 3)
                        run_s[lane] = run;
                }
                __syncthreads();
            }
            if (warp == 3) {
                bs_local[i][lane] = run.x;
                bs_local[i][lane + 32] = run.y;
            }
        }
    } else {
        for (int i = warp; rank + C * i < nb; i += W) {
            const int b = rank + C * i;
            const float *tb = tab + (size_t) b * n;
            const float2 c = make_float2(__ldg(tb + min(s0, n - 1)), __ldg(tb + min(s1, n - 1)));
            float2 run = joseph::splat(0.0f);
            if (PIPE)
                sart_fp_samples_2x<kBlock, K>(img0 + (size_t) b * kBlock * P.pitch, P.pitch, c, st, hi, z2, run);
            else
                sart_fp_samples<kBlock, K, true>(img0 + (size_t) b * kBlock * P.pitch, P.pitch, c, st, hi, z2, run,
                                              nullptr);
            bs_local[i][lane] = run.x;
            bs_local[i][lane + 32] = run.y;
        }
    }
    cluster_sync_all();
    if (writer) {
        float result = src_v;
        const joseph::AxisConsts kc = joseph::axis_consts(n, P.axis);
        if (!joseph::detector_inactive(kc, sr)) {
            /* block sums in block order, 16 remote loads in flight at a time;
             * block j sits on CTA j mod C in slot j / C, stepped without a
             * division (on this path after the barrier, a division per block
             * cost more than the loads) */
            float detected = 0.0f;
            int rk = 0, slot = 0;
            for (int j0 = 0; j0 < nb; j0 += kRemoteBatch) {
                float bsv[kRemoteBatch];
#pragma unroll
                for (int k = 0; k < kRemoteBatch; ++k) {
                    bsv[k] = j0 + k < nb ? ld_cluster(&bs_local[slot][threadIdx.x], rk) : 0.0f;
                    if (++rk == C) {
                        rk = 0;
                        ++slot;
                    }
                }
#pragma unroll
                for (int k = 0; k < kRemoteBatch; ++k)
                    if (j0 + k < nb)
                        detected = __fadd_rn(detected, bsv[k]);
            }
            result = __fadd_rn(result, __fmul_rn(detected, P.scale));
        }
        if (P.w)
            result = __fmul_rn(result, w_v);
        P.out[oidx] = result;
    }
    cluster_sync_all();
}

struct SartBpArgs {
    const float *sino;
    float *vol;             /* padded layout, [slices][rows][pitch] */
    int n;
    int angle;
    int pitch;
    float os, shift, e0, e1;
    float sn, cs;
    float relax;
    float neg_zero;
    const float *relax_dev;
    int *err;
    long long vol_stride;
    long long sino_stride;
};

constexpr int kBpTileW = 128;   /* storage columns per CTA: 32 threads x 4 */
constexpr int kBpSpan = 256;    /* sinogram values staged per CTA */

/* The backprojection's detector coordinate of storage pixel (i, j), clamp
 * excluded (…joseph.cl:189-195); with T the storage holds the transpose. */
template <bool T>
__device__ __forceinline__ float sart_bp_coord(const SartBpArgs &P, int i, int j)
{
    const float fI = __fsub_rn(__fadd_rn((float) i, 0.5f), P.os);
    const float fJ = __fsub_rn(__fadd_rn((float) j, 0.5f), P.os);
    const float fX = T ? fJ : fI;
    const float fY = T ? fI : fJ;
    return __fadd_rn(__fsub_rn(__fmul_rn(fX, P.cs), __fmul_rn(fY, P.sn)), P.shift);
}

/* The pixel updates of one thread: rows j0 + 8m (m < ROWS, clamped to the
 * image), column pairs with products pc; CLAMP for tiles that reach past
 * the clamp edges. */
template <bool T, int ROWS, bool CLAMP>
__device__ __forceinline__ void sart_bp_rows(const SartBpArgs &P, float (&x)[ROWS][4], const float2 (&pc)[2],
                                             int j0, uint32_t rbase, float relax, float2 z2)
{
#pragma unroll
    for (int m = 0; m < ROWS; ++m) {
        const int j = min(j0 + 8 * m, P.n - 1);
        const float fJ = __fsub_rn(__fadd_rn((float) j, 0.5f), P.os);
        const float q = __fmul_rn(fJ, T ? P.cs : P.sn);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const float2 d = T ? joseph::sub2(joseph::splat(q), pc[h]) : joseph::sub2(pc[h], joseph::splat(q));
            float2 c = joseph::add2(d, joseph::splat(P.shift));
            if (CLAMP)
                c = make_float2(fminf(fmaxf(c.x, P.e0), P.e1), fminf(fmaxf(c.y, P.e0), P.e1));
            float2 t;
            const float2 y = joseph::floor_half2(c, t);
            const uint32_t aa = rbase + 4u * (uint32_t) __float_as_int(y.x);
            const uint32_t ab = rbase + 4u * (uint32_t) __float_as_int(y.y);
            const float2 t0 = make_float2(joseph::lds(aa), joseph::lds(ab));
            const float2 t1 = make_float2(joseph::lds(aa + 4u), joseph::lds(ab + 4u));
            const float2 sum = joseph::add2(joseph::splat(0.0f), joseph::lerp2(t, t0, t1, z2));
            const float2 upd = joseph::add2(make_float2(x[m][2 * h], x[m][2 * h + 1]),
                                            joseph::mul2z(joseph::splat(relax), sum, z2));
            x[m][2 * h] = upd.x;
            x[m][2 * h + 1] = upd.y;
        }
    }
}

/*
 * vol = vol + relax * (0 + sample) for one angle on the padded layout
 * (…joseph.cl:158-218 with a one-angle subset); requires e0 <= e1.
 *
 * A CTA updates an (8 ROWS) x 128 storage tile; thread (tx, ty) the columns
 * tx + 32h (h = 0..3) of rows ty + 8m (m < ROWS), so the 32 lanes of a warp
 * read 32 adjacent columns (coalesced) and, for one h, detector bins at most
 * one apart (no shared-memory bank conflicts). Columns h and h + 1 form one
 * packed pair. The coordinate is monotone in each pixel index (every
 * rounding step is), so over the tile it lies between its values at the
 * four corners (four lanes of each warp compute them): the CTA stages the
 * sinogram values between those bounds in shared memory, and tiles whose
 * corners lie within [e0, e1] skip the clamp. The row product is computed
 * once per row, the column products once per thread.
 * Grid (ceil(n/128), ceil(n/(8 ROWS)), slices), block 32 x 8.
 */
template <bool T, int ROWS>
__global__ void __launch_bounds__(256) sart_bp_kernel(SartBpArgs P)
{
    __shared__ __align__(16) float rs[kBpSpan];
    pdl_launch_next();
    const int n = P.n;
    const int lane = (int) threadIdx.x;
    const int i_base = (int) blockIdx.x * kBpTileW, j_base = (int) blockIdx.y * (8 * ROWS);
    /* lane k < 4 computes corner (k & 1, k >> 1); min and max over the four */
    const int ci = (lane & 1) ? min(i_base + kBpTileW - 1, n - 1) : i_base;
    const int cj = (lane & 2) ? min(j_base + 8 * ROWS - 1, n - 1) : j_base;
    const float cc = sart_bp_coord<T>(P, ci, cj);
    float umin = lane < 4 ? cc : INFINITY, umax = lane < 4 ? cc : -INFINITY;
    umin = fminf(umin, __shfl_xor_sync(0xffffffffu, umin, 1));
    umax = fmaxf(umax, __shfl_xor_sync(0xffffffffu, umax, 1));
    umin = fminf(umin, __shfl_xor_sync(0xffffffffu, umin, 2));
    umax = fmaxf(umax, __shfl_xor_sync(0xffffffffu, umax, 2));
    umin = __shfl_sync(0xffffffffu, umin, 0);
    umax = __shfl_sync(0xffffffffu, umax, 0);
    const bool interior = umin >= P.e0 && umax <= P.e1;
    const float cmin = fminf(fmaxf(umin, P.e0), P.e1), cmax = fminf(fmaxf(umax, P.e0), P.e1);
    const int lo = (int) floorf(__fsub_rn(cmin, 0.5f));
    const int span = (int) floorf(__fsub_rn(cmax, 0.5f)) + 2 - lo;
    const int tid = (int) (threadIdx.y * 32 + threadIdx.x);
    if (span > kBpSpan) {      /* cannot happen for |sin|, |cos| <= 1; uniform per CTA */
        if (tid == 0)
            atomicOr(P.err, kErrSpan);
        return;
    }
    /* the residual row and the volume were written by earlier kernels */
    pdl_wait_previous();
    /* the tile's pixels first: their loads overlap the staging below */
    const int i0 = i_base + lane;
    bool okc[4];
#pragma unroll
    for (int h = 0; h < 4; ++h)
        okc[h] = i0 + 32 * h < n;
    float *vcol = P.vol + (size_t) blockIdx.z * P.vol_stride + (size_t) (j_base + (int) threadIdx.y) * P.pitch +
                  kSartPadL + i0;
    const int rows_left = n - j_base - (int) threadIdx.y;     /* rows m with 8m < rows_left exist */
    /* a tile wholly inside the image (uniform per CTA) loads and stores
     * every pixel without the per-pixel checks */
    const bool full = i_base + kBpTileW <= n && j_base + 8 * ROWS <= n;
    float x[ROWS][4];
    if (full) {
#pragma unroll
        for (int m = 0; m < ROWS; ++m) {
            const float *row = vcol + (size_t) (8 * m) * P.pitch;
#pragma unroll
            for (int h = 0; h < 4; ++h)
                x[m][h] = row[32 * h];
        }
    } else {
#pragma unroll
        for (int m = 0; m < ROWS; ++m) {
            const float *row = vcol + (size_t) (8 * m) * P.pitch;
#pragma unroll
            for (int h = 0; h < 4; ++h)
                x[m][h] = okc[h] && 8 * m < rows_left ? row[32 * h] : 0.0f;
        }
    }
    const float *r = P.sino + (size_t) blockIdx.z * P.sino_stride + (size_t) P.angle * n;
    for (int k = tid; k < span; k += 256) {
        const int idx = lo + k;
        rs[k] = (idx >= 0 && idx < n) ? __ldg(r + idx) : 0.0f;
    }
    __syncthreads();
    if (!okc[0] || rows_left <= 0)
        return;

    const float relax = P.relax_dev ? *P.relax_dev : P.relax;
    const float2 z2 = joseph::splat(P.neg_zero);
    /* column products; columns past n repeat column n - 1 and are not stored */
    float2 pc[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int ia = min(i0 + 64 * h, n - 1), ib = min(i0 + 64 * h + 32, n - 1);
        const float2 fI = make_float2(__fsub_rn(__fadd_rn((float) ia, 0.5f), P.os),
                                      __fsub_rn(__fadd_rn((float) ib, 0.5f), P.os));
        pc[h] = joseph::mul2z(fI, joseph::splat(T ? P.sn : P.cs), z2);
    }
    const uint32_t rbase = (uint32_t) __cvta_generic_to_shared(rs) -
                           4u * (uint32_t) (joseph::kHalfFloorBits + lo);
    const int j0 = j_base + (int) threadIdx.y;
    if (interior)
        sart_bp_rows<T, ROWS, false>(P, x, pc, j0, rbase, relax, z2);
    else
        sart_bp_rows<T, ROWS, true>(P, x, pc, j0, rbase, relax, z2);
    if (full) {
#pragma unroll
        for (int m = 0; m < ROWS; ++m) {
            float *row = vcol + (size_t) (8 * m) * P.pitch;
#pragma unroll
            for (int h = 0; h < 4; ++h)
                row[32 * h] = x[m][h];
        }
        return;
    }
#pragma unroll
    for (int m = 0; m < ROWS; ++m) {
        if (8 * m < rows_left) {
            float *row = vcol + (size_t) (8 * m) * P.pitch;
#pragma unroll
            for (int h = 0; h < 4; ++h)
                if (okc[h])
                    row[32 * h] = x[m][h];
        }
    }
}

}  // namespace

/* Lets the segment-form FP run in clusters of 16 CTAs and counts how many
 * such clusters fit on this GPU at once (0 where the size is refused). */
int udev_sart_init(udev *d)
{
    const void *func = (const void *) sart_fp_kernel<4, 16, 4, 3>;
    d->sart_wide_clusters = 0;
    if (cudaFuncSetAttribute(func, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        cudaGetLastError();
        return UFOIR_OK;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned int) kFpWideCluster, 1, 1);
    cfg.blockDim = dim3(128, 1, 1);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned int) kFpWideCluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, func, &cfg) != cudaSuccess) {
        cudaGetLastError();
        clusters = 0;
    }
    d->sart_wide_clusters = clusters;
    return UFOIR_OK;
}

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

/* ---- the padded sweep layout ---- */

extern "C" int udev_sart_pitch(int n)
{
    return sart_pitch(n);
}

extern "C" size_t udev_sart_work_floats(int n, int n_slices)
{
    const size_t plane = (size_t) sart_rows(n) * (size_t) sart_pitch(n);
    return (size_t) n_slices * 2 * plane;
}

/* The clamp edges of the backprojection (…joseph.cl:174-187), computed as
 * the host side of udev_bp_angle does. */
static void sart_bp_consts(const udev_geom *g, float *os, float *shift, float *e0, float *e1)
{
    const float w = (float) g->n_dets, axis = g->axis;
    const float required_width = axis * 2.0f;
    const float diff = w - required_width;
    const float ros = diff / 2.0f;
    const float half = diff < 0.0f ? w - axis : axis;
    *os = w / 2.0f;
    *shift = *os - ros;
    *e0 = axis - half + 0.5f;
    *e1 = axis + half - 0.5f;
}

/* The padded kernels' arithmetic needs e0 <= e1 and n <= 8192. */
static bool sart_geometry_ok(const udev_geom *g)
{
    float os, shift, e0, e1;
    if (g->n_dets < 1 || g->n_dets > kMaxBlocks * kBlock)
        return false;
    sart_bp_consts(g, &os, &shift, &e0, &e1);
    return e0 <= e1;
}

/* Launch shape of the one-angle forward projection: up to 16 blocks,
 * clusters of up to 8 CTAs with one or two blocks each, four segment warps
 * (16 rows each) per block; else, where it fits in one wave, one block per
 * warp: two 8-sample batches in flight in 4-warp CTAs (3 per SM; 4-6 %
 * faster at 1448^2 than one 16-sample batch at a time), or one 8-sample
 * batch at a time (fewer registers) in 16-warp CTAs (one per SM) or 8-warp
 * CTAs (2 per SM), where a second batch in flight (128 registers) was 1 %
 * slower at 2900^2; else clusters of 8 CTAs with several blocks per warp. */
struct SartFpShape {
    int shape;      /* 0: segments; 1, 2, 3: whole blocks per warp (4, 8, 16 warps per CTA) */
    int cluster;
    int threads;
    const void *func;
};

static SartFpShape sart_fp_shape(udev *d, int n, int n_slices)
{
    const int nb = (n + kBlock - 1) / kBlock, groups = (n + 63) / 64;
    const long long sms = udev_sm_count(d);
    SartFpShape f;
    if (nb > kFpCluster && nb <= 2 * kFpWideCluster && (long long) groups * n_slices <= d->sart_wide_clusters) {
        /* one or two blocks per CTA over a non-portable cluster of up to 16
         * CTAs, where every ray group's cluster fits on the GPU at once */
        f.shape = 0;
        f.cluster = nb < kFpWideCluster ? nb : kFpWideCluster;
    } else if (nb <= 2 * kFpCluster) {
        f.shape = 0;
        f.cluster = nb < kFpCluster ? nb : kFpCluster;
    } else if (udev_div_up(nb, 4) <= kFpCluster && (long long) groups * udev_div_up(nb, 4) * n_slices <= 3 * sms) {
        f.shape = 1;
        f.cluster = (int) udev_div_up(nb, 4);
    } else if (udev_div_up(nb, 16) <= kFpCluster && (long long) groups * udev_div_up(nb, 16) * n_slices <= sms) {
        f.shape = 3;
        f.cluster = (int) udev_div_up(nb, 16);
    } else if (udev_div_up(nb, 8) <= kFpCluster && (long long) groups * udev_div_up(nb, 8) * n_slices <= 2 * sms) {
        f.shape = 2;
        f.cluster = (int) udev_div_up(nb, 8);
    } else {
        f.shape = 1;
        f.cluster = kFpCluster;
    }
    f.threads = f.shape == 3 ? 512 : f.shape == 2 ? 256 : 128;
    f.func = f.shape == 0   ? (const void *) sart_fp_kernel<4, 16, 4, 3>
             : f.shape == 1 ? (const void *) sart_fp_kernel<1, 8, 4, 3, true>
             : f.shape == 2 ? (const void *) sart_fp_kernel<1, 8, 8, 2>
                            : (const void *) sart_fp_kernel<1, 8, 16, 1>;
    return f;
}

/* Overlap each per-angle kernel's launch and geometry prologue with the end
 * of the previous one (programmatic dependent launch) when both kernels'
 * grids fit on the GPU together: then a waiting CTA takes no SM another
 * one needs (with larger grids that overlap was measured slower). */
static bool sart_pdl(udev *d, int n, int n_slices)
{
    const SartFpShape f = sart_fp_shape(d, n, n_slices);
    const long long fp_ctas = (long long) ((n + 63) / 64) * f.cluster * n_slices;
    const long long bp_ctas = (long long) udev_div_up(n, kBpTileW) * udev_div_up(n, 32) * n_slices;
    return fp_ctas + bp_ctas <= udev_sm_count(d);
}

extern "C" int udev_sart_padded(udev *d, const udev_geom *g, int n_slices)
{
    if (!sart_geometry_ok(g) || n_slices < 1 || n_slices > 65535)
        return 0;
    /* one cluster of the forward projection's shape must fit on this GPU
     * (a partition with few SMs may not hold it) */
    if (cudaSetDevice(d->device) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    const SartFpShape f = sart_fp_shape(d, g->n_dets, n_slices);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned int) f.cluster, 1, 1);
    cfg.blockDim = dim3((unsigned int) f.threads, 1, 1);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned int) f.cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, f.func, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return clusters > 0;
}

/* Copies between the user's n x n slices (place -1) and the padded copies
 * V (place 0) and H (place 1, the transpose). */
extern "C" int udev_sart_move(udev *d, int n, float *x, float *work, int from, int to, int n_slices)
{
    if (n_slices <= 0 || n <= 0)
        return UFOIR_OK;
    if (from == to || from < -1 || from > 1 || to < -1 || to > 1 || n_slices > 65535) {
        udev_set_error(d, "sart_move: bad places %d -> %d or %d slices", from, to, n_slices);
        return UFOIR_ERR_INVALID;
    }
    UDEV_BIND(d);
    const int pitch = sart_pitch(n);
    const long long plane = (long long) sart_rows(n) * pitch;
    float *place[2] = {work, work + (size_t) n_slices * plane};
    const float *src = from < 0 ? x : place[from];
    float *dst = to < 0 ? x : place[to];
    const int sp = from < 0 ? n : pitch, so = from < 0 ? 0 : kSartPadL;
    const int dp = to < 0 ? n : pitch, dof = to < 0 ? 0 : kSartPadL;
    const long long ss = from < 0 ? (long long) n * n : plane, ds = to < 0 ? (long long) n * n : plane;
    /* H is the transpose of V and of the user's layout */
    const int transpose = (from == 1) != (to == 1);
    dim3 grid(udev_div_up(n, 32), udev_div_up(n, 32), (unsigned int) n_slices);
    sart_copy_kernel<<<grid, dim3(32, 8), 0, d->stream>>>(src, sp, so, ss, dst, dp, dof, ds, n, transpose);
    return udev_after_launch(d, "sart_copy_kernel");
}

extern "C" int udev_sart_fp(udev *d, const udev_geom *g, int angle, int dir, const float *table, float *work,
                            int place, const float *src, const float *w, int w_shared, float *out, float scale,
                            int n_slices)
{
    if (n_slices <= 0)
        return UFOIR_OK;
    const int n = g->n_dets;
    if (angle < 0 || angle >= g->n_angles || n < 1 || n > kMaxBlocks * kBlock || n_slices > 65535 ||
        (place != 0 && place != 1)) {
        udev_set_error(d, "sart_fp: angle %d of %d, n = %d, %d slices, place %d out of range", angle, g->n_angles,
                       n, n_slices, place);
        return UFOIR_ERR_INVALID;
    }
    UDEV_BIND(d);
    const int pitch = sart_pitch(n);
    const size_t plane = (size_t) sart_rows(n) * pitch;
    const int nb = (n + kBlock - 1) / kBlock, groups = (n + 63) / 64;
    SartFpArgs A;
    A.img = work + (size_t) place * n_slices * plane;
    A.table = table;
    /* the sweep runs the angles in order (the last one's FP pulls in the
     * first's rows); only where the table outgrows what L2 keeps beside the
     * volume: 1 % per angle at 1448^2 x 1200 and 2900^2 x 360 (A/B), nothing
     * to gain below */
    const size_t table_bytes = udev_fp_block_starts_floats(n, g->n_angles) * sizeof(float);
    A.next_table = table_bytes > kPrefetchTableBytes ? table + (size_t) ((angle + 1) % g->n_angles) * nb * n : nullptr;
    A.src = src;
    A.w = w;
    A.out = out;
    A.sinv = g->d_sin;
    A.cosv = g->d_cos;
    A.n = n;
    A.n_blocks = nb;
    A.angle = angle;
    A.dir = dir;
    A.pitch = pitch;
    A.axis = g->axis;
    A.scale = scale;
    A.neg_zero = -0.0f;
    A.img_stride = (long long) plane;
    A.sino_stride = (long long) g->n_angles * n;
    A.w_stride = w_shared ? 0 : A.sino_stride;
    const SartFpShape f = sart_fp_shape(d, n, n_slices);
    A.cluster = f.cluster;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned int) (groups * A.cluster), 1, (unsigned int) n_slices);
    cfg.blockDim = dim3((unsigned int) f.threads, 1, 1);
    cfg.stream = d->stream;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned int) A.cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (sart_pdl(d, n, n_slices)) {
        attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[1].val.programmaticStreamSerializationAllowed = 1;
        cfg.numAttrs = 2;
    }
    cudaError_t e = f.shape == 0   ? cudaLaunchKernelEx(&cfg, sart_fp_kernel<4, 16, 4, 3>, A)
                    : f.shape == 1 ? cudaLaunchKernelEx(&cfg, sart_fp_kernel<1, 8, 4, 3, true>, A)
                    : f.shape == 2 ? cudaLaunchKernelEx(&cfg, sart_fp_kernel<1, 8, 8, 2>, A)
                                   : cudaLaunchKernelEx(&cfg, sart_fp_kernel<1, 8, 16, 1>, A);
    if (e != cudaSuccess) {
        cudaGetLastError();
        udev_set_error(d, "sart_fp_kernel launch: %s", cudaGetErrorString(e));
        return UFOIR_ERR_CUDA;
    }
    return udev_after_launch(d, "sart_fp_kernel");
}

extern "C" int udev_sart_bp(udev *d, const udev_geom *g, int angle, float sn, float cs, const float *sino,
                            float *work, int place, float relax, const float *relax_dev, int n_slices)
{
    if (n_slices <= 0)
        return UFOIR_OK;
    const int n = g->n_dets;
    if (angle < 0 || angle >= g->n_angles || n < 1 || n_slices > 65535 || (place != 0 && place != 1) ||
        !sart_geometry_ok(g)) {
        udev_set_error(d, "sart_bp: angle %d of %d, n = %d, %d slices, place %d out of range", angle, g->n_angles,
                       n, n_slices, place);
        return UFOIR_ERR_INVALID;
    }
    UDEV_BIND(d);
    const int pitch = sart_pitch(n);
    const size_t plane = (size_t) sart_rows(n) * pitch;
    SartBpArgs A;
    sart_bp_consts(g, &A.os, &A.shift, &A.e0, &A.e1);
    A.sino = sino;
    A.vol = work + (size_t) place * n_slices * plane;
    A.n = n;
    A.angle = angle;
    A.pitch = pitch;
    A.sn = sn;
    A.cs = cs;
    A.relax = relax;
    A.neg_zero = -0.0f;
    A.relax_dev = relax_dev;
    A.err = d->d_err;
    A.vol_stride = (long long) plane;
    A.sino_stride = (long long) g->n_angles * n;
    /* 32-row tiles at every size: at 2900^2 they took 1 us off each angle against
     * 64-row tiles (2.3 waves of those at three CTAs per SM left a thin last wave) */
    dim3 grid(udev_div_up(n, kBpTileW), udev_div_up(n, 32), (unsigned int) n_slices);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(32, 8, 1);
    cfg.stream = d->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = sart_pdl(d, n, n_slices) ? 1 : 0;
    const cudaError_t e = place == 1 ? cudaLaunchKernelEx(&cfg, sart_bp_kernel<true, 4>, A)
                                     : cudaLaunchKernelEx(&cfg, sart_bp_kernel<false, 4>, A);
    if (e != cudaSuccess) {
        cudaGetLastError();
        udev_set_error(d, "sart_bp_kernel launch: %s", cudaGetErrorString(e));
        return UFOIR_ERR_CUDA;
    }
    return udev_after_launch(d, "sart_bp_kernel");
}
