/*
 * udev_bp_tiles.cu - pixel-driven backprojection over many angles, with the
 * sinogram windows of a pixel tile staged in shared memory.
 *
 * One CTA owns a 32 x 32 pixel tile; thread (tx, ty) owns the 4 pixels
 * (x0 + tx, y0 + ty + 8p), p < 4, which share fX * cos(theta). For a chunk of
 * 32 angles the CTA copies, per angle, the 64 detector values that the tile
 * can reach (cp.async, double buffered; detectors outside [0, n) read 0),
 * so every sample reads shared memory and a warp's 32 lanes (adjacent x)
 * touch adjacent words.
 *
 * Arithmetic is the reference's BP (projector-parallel-joseph.cl:158-218):
 * s = fX * cos - fY * sin + (os - ros), clamped to the active detector
 * edges, linear interpolation along s at the row centre, per-subset float
 * sums over the angles in order, then v = v + relax * sum per subset; the
 * epilogue optionally applies v * cw + add (SIRT update).
 */
#include <cuda_runtime.h>

#include "joseph.cuh"
#include "udev_internal.cuh"

namespace {

constexpr int kTX = 32;
constexpr int kTY = 8;
constexpr int kPY = 4;               /* pixels per thread (one column) */
constexpr int kTile = kTX;           /* tile is kTile x kTile pixels */
constexpr int kAC = 32;              /* angles per chunk */
constexpr int kWin = 64;             /* detector window per angle */
constexpr int kMaxSub = 16;
constexpr float kFloorMagic = 12582912.0f;
constexpr int kFloorMagicBits = 0x4B400000;

struct BpTileArgs {
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
    int total_angles;
    unsigned int sub_offset[kMaxSub];
    unsigned int sub_n[kMaxSub];
};

struct __align__(16) BpSmem {
    float win[2][kAC][kWin];
    float cs[2][kAC];
    float sn[2][kAC];
    int w0[2][kAC];
};

__device__ __forceinline__ void cp_async4(float *dst, const float *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t) __cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}

__device__ __forceinline__ void cp_async_commit()
{
    asm volatile("cp.async.commit_group;" ::: "memory");
}

template <int N>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

/* Angle of virtual index vi (angles of the subsets, in order). */
__device__ __forceinline__ int angle_of(const BpTileArgs &P, int vi)
{
    for (int k = 0; k < P.n_subsets; ++k) {
        if (vi < (int) P.sub_n[k])
            return (int) P.sub_offset[k] + vi;
        vi -= (int) P.sub_n[k];
    }
    return 0;
}

/* Detector coordinate of pixel (x, y) for one angle, exactly as the reference. */
__device__ __forceinline__ float det_coord(float fX, float fY, float cs, float sn, float shift)
{
    return __fadd_rn(__fsub_rn(__fmul_rn(fX, cs), __fmul_rn(fY, sn)), shift);
}

__device__ void load_chunk(const BpTileArgs &P, BpSmem &S, int buf, int chunk, const float *sino, int x0, int y0,
                           const joseph::AxisConsts &k, float e0, float e1, float shift)
{
    const int tid = threadIdx.y * kTX + threadIdx.x;
    const int first = chunk * kAC;
    const int count = min(kAC, P.total_angles - first);
    /* one thread per angle: LUT values and window start */
    if (tid < count) {
        const int a = angle_of(P, first + tid);
        const float cs = __ldg(P.cosv + a), sn = __ldg(P.sinv + a);
        S.cs[buf][tid] = cs;
        S.sn[buf][tid] = sn;
        const float fx0 = __fsub_rn(__fadd_rn((float) x0, 0.5f), k.os);
        const float fx1 = __fsub_rn(__fadd_rn((float) (x0 + kTile - 1), 0.5f), k.os);
        const float fy0 = __fsub_rn(__fadd_rn((float) y0, 0.5f), k.os);
        const float fy1 = __fsub_rn(__fadd_rn((float) (y0 + kTile - 1), 0.5f), k.os);
        const float c00 = det_coord(fx0, fy0, cs, sn, shift), c10 = det_coord(fx1, fy0, cs, sn, shift);
        const float c01 = det_coord(fx0, fy1, cs, sn, shift), c11 = det_coord(fx1, fy1, cs, sn, shift);
        float lo = fminf(fminf(c00, c10), fminf(c01, c11));
        lo = fminf(fmaxf(lo, e0), e1);
        S.w0[buf][tid] = (int) floorf(__fsub_rn(lo, 0.5f)) - 2;
    }
    __syncthreads();
    /* windows: 256 threads, 4 angles x 64 detectors per round */
    for (int idx = tid; idx < count * kWin; idx += kTX * kTY) {
        const int slot = idx / kWin, e = idx % kWin;
        const int a = angle_of(P, first + slot);
        const int d = S.w0[buf][slot] + e;
        float *dst = &S.win[buf][slot][e];
        if (d >= 0 && d < P.n)
            cp_async4(dst, sino + (size_t) a * P.n + d);
        else
            *dst = 0.0f;
    }
}

template <bool CLAMP>
__device__ __forceinline__ void sample_chunk(const BpSmem &S, int buf, int count, int first_vi, const BpTileArgs &P,
                                             float fX, const float fY[kPY], float shift, float e0, float e1,
                                             float sum[kPY], float v[kPY], int &sub, int &sub_end)
{
    for (int i = 0; i < count; ++i) {
        const int vi = first_vi + i;
        if (vi == sub_end) {
            /* end of a subset: v = v + relax * sum (one BP launch of the reference) */
#pragma unroll
            for (int p = 0; p < kPY; ++p) {
                v[p] = __fadd_rn(v[p], __fmul_rn(P.relax, sum[p]));
                sum[p] = 0.0f;
            }
            ++sub;
            sub_end += (int) P.sub_n[sub];
        }
        const float cs = S.cs[buf][i], sn = S.sn[buf][i];
        const int w0 = S.w0[buf][i];
        const float *win = S.win[buf][i];
        const float fxc = __fmul_rn(fX, cs);
#pragma unroll
        for (int p = 0; p < kPY; ++p) {
            float sc = __fadd_rn(__fsub_rn(fxc, __fmul_rn(fY[p], sn)), shift);
            if (CLAMP)
                sc = fminf(fmaxf(sc, e0), e1);
            const float cm = __fsub_rn(sc, 0.5f);
            const float y = __fadd_rd(cm, kFloorMagic);
            const float fi = __fsub_rn(y, kFloorMagic);
            const int j = __float_as_int(y) - kFloorMagicBits - w0;
            const float t = __fsub_rn(cm, fi);
            sum[p] = __fadd_rn(sum[p], joseph::lerp(t, win[j], win[j + 1]));
        }
    }
}

__global__ void __launch_bounds__(kTX * kTY) bp_tiles_kernel(BpTileArgs P)
{
    __shared__ BpSmem S;
    const int n = P.n;
    const int tiles_x = (n + kTile - 1) / kTile;
    const int x0 = (int) (blockIdx.x % tiles_x) * kTile;
    const int y0 = (int) (blockIdx.x / tiles_x) * kTile;
    const int slice = (int) blockIdx.y;
    const float *sino = P.sino + (size_t) slice * P.sino_stride;

    const joseph::AxisConsts k = joseph::axis_consts(n, P.axis);
    float e0, e1;
    joseph::bp_edges(k, n, P.axis, e0, e1);
    const float shift = __fsub_rn(k.os, k.ros);

    const int x = x0 + (int) threadIdx.x;
    const float fX = __fsub_rn(__fadd_rn((float) x, 0.5f), k.os);
    float fY[kPY], sum[kPY], v[kPY];
#pragma unroll
    for (int p = 0; p < kPY; ++p) {
        const int y = y0 + (int) threadIdx.y + kTY * p;
        fY[p] = __fsub_rn(__fadd_rn((float) y, 0.5f), k.os);
        sum[p] = 0.0f;
        const size_t pix = (size_t) slice * P.vol_stride + (size_t) y * n + x;
        v[p] = (P.base && x < n && y < n) ? P.base[pix] : 0.0f;
    }

    /* A tile whose every pixel lies within distance (n/2 - 2) of the centre
     * never reaches the clamp edges (on-axis geometry), so the clamp can be
     * skipped without changing any result. */
    bool clamp = true;
    if (k.diff == 0.0f) {
        const float r = 0.5f * (float) n - 2.0f;
        const float ax = fmaxf(fabsf((float) x0 - k.os), fabsf((float) (x0 + kTile) - k.os));
        const float ay = fmaxf(fabsf((float) y0 - k.os), fabsf((float) (y0 + kTile) - k.os));
        clamp = ax * ax + ay * ay > r * r;
    }

    const int nchunks = (P.total_angles + kAC - 1) / kAC;
    int sub = 0;
    int sub_end = P.n_subsets > 0 ? (int) P.sub_n[0] : 0;
    if (nchunks > 0) {
        load_chunk(P, S, 0, 0, sino, x0, y0, k, e0, e1, shift);
        cp_async_commit();
    }
    for (int ch = 0; ch < nchunks; ++ch) {
        const int buf = ch & 1;
        if (ch + 1 < nchunks) {
            load_chunk(P, S, buf ^ 1, ch + 1, sino, x0, y0, k, e0, e1, shift);
            cp_async_commit();
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const int count = min(kAC, P.total_angles - ch * kAC);
        if (clamp)
            sample_chunk<true>(S, buf, count, ch * kAC, P, fX, fY, shift, e0, e1, sum, v, sub, sub_end);
        else
            sample_chunk<false>(S, buf, count, ch * kAC, P, fX, fY, shift, e0, e1, sum, v, sub, sub_end);
        __syncthreads();
    }
    if (P.n_subsets > 0) {
#pragma unroll
        for (int p = 0; p < kPY; ++p)
            v[p] = __fadd_rn(v[p], __fmul_rn(P.relax, sum[p]));
    }
    if (x >= n)
        return;
#pragma unroll
    for (int p = 0; p < kPY; ++p) {
        const int y = y0 + (int) threadIdx.y + kTY * p;
        if (y >= n)
            continue;
        float r = v[p];
        if (P.cw)
            r = __fmul_rn(r, P.cw[(size_t) slice * P.cw_stride + (size_t) y * n + x]);
        const size_t pix = (size_t) slice * P.vol_stride + (size_t) y * n + x;
        if (P.add)
            r = __fadd_rn(r, P.add[pix]);
        P.dst[pix] = r;
    }
}

}  // namespace

extern "C" int udev_bp_tiles(udev *d, const udev_geom *g, const ufoir_subset *subsets, int n_subsets,
                             const float *sino, const float *base, const float *cw, int cw_shared, const float *add,
                             float *dst, float relax, int n_slices)
{
    if (n_slices <= 0)
        return UFOIR_OK;
    if (n_subsets > kMaxSub) {
        udev_set_error(d, "bp_tiles: %d subsets (at most %d)", n_subsets, kMaxSub);
        return UFOIR_ERR_UNSUPPORTED;
    }
    int total = 0;
    for (int i = 0; i < n_subsets; i++) {
        if (subsets[i].offset + (size_t) subsets[i].n > (size_t) g->n_angles) {
            udev_set_error(d, "bp: subset [%u, %u) outside [0, %d)", subsets[i].offset,
                           subsets[i].offset + subsets[i].n, g->n_angles);
            return UFOIR_ERR_INVALID;
        }
        total += (int) subsets[i].n;
    }
    UDEV_BIND(d);
    BpTileArgs A;
    A.sino = sino;
    A.base = base;
    A.cw = cw;
    A.add = add;
    A.dst = dst;
    A.sinv = g->d_sin;
    A.cosv = g->d_cos;
    A.n = g->n_dets;
    A.axis = g->axis;
    A.relax = relax;
    A.vol_stride = (long long) g->n_dets * g->n_dets;
    A.sino_stride = (long long) g->n_angles * g->n_dets;
    A.cw_stride = cw_shared ? 0 : A.vol_stride;
    A.n_subsets = n_subsets;
    A.total_angles = total;
    for (int i = 0; i < kMaxSub; i++) {
        A.sub_offset[i] = i < n_subsets ? subsets[i].offset : 0;
        A.sub_n[i] = i < n_subsets ? subsets[i].n : 0;
    }
    const int tiles_x = (g->n_dets + kTile - 1) / kTile;
    const unsigned int n_tiles = (unsigned int) (tiles_x * tiles_x);
    for (int done = 0; done < n_slices;) {
        const int chunk = n_slices - done > 65535 ? 65535 : n_slices - done;
        BpTileArgs B = A;
        B.sino += (size_t) done * A.sino_stride;
        if (B.base)
            B.base += (size_t) done * A.vol_stride;
        if (B.cw)
            B.cw += (size_t) done * A.cw_stride;
        if (B.add)
            B.add += (size_t) done * A.vol_stride;
        B.dst += (size_t) done * A.vol_stride;
        bp_tiles_kernel<<<dim3(n_tiles, (unsigned int) chunk), dim3(kTX, kTY), 0, d->stream>>>(B);
        int rc = udev_after_launch(d, "bp_tiles_kernel");
        if (rc)
            return rc;
        done += chunk;
    }
    return UFOIR_OK;
}
