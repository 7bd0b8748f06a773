/*
 * udev_bp_tiles.cu - pixel-driven backprojection over many angles, with the
 * sinogram windows of a pixel tile staged in shared memory.
 *
 * One CTA owns a 32 x 128 pixel tile; thread (tx, ty) owns the 16 pixels
 * (x0 + tx, y0 + ty + 8p), p < 16, which share fX * cos(theta) and the
 * per-angle set-up (16 pixels amortise it better than 8: 2.3 % on the C2
 * backprojection; 32 pixels, 32 x 256 tiles, need 139 KB of shared memory
 * and 132 registers, one CTA per SM, and were 23 % slower; a 64-register
 * build with 16-angle chunks, four CTAs per SM, was 6 % slower). Launches
 * with fewer than three waves of such tiles (a single slice of 1448^2: 552
 * tiles for 456 CTA slots) use 32 x 64 tiles, 8 pixels per thread, whose
 * last wave is fuller. For a chunk of
 * 32 angles the CTA copies, per angle, the
 * 160 detector values that the tile can reach (cp.async, double buffered;
 * detectors outside [0, n) read 0), so every sample reads shared memory and
 * a warp's 32 lanes (adjacent x) touch adjacent words.
 *
 * Arithmetic is the reference's BP (projector-parallel-joseph.cl:158-218):
 * s = fX * cos - fY * sin + (os - ros), clamped to the active detector
 * edges, linear interpolation along s at the row centre, per-subset float
 * sums over the angles in order, then v = v + relax * sum per subset; the
 * epilogue optionally applies v * cw + add (SIRT update).
 */
#include <cuda_runtime.h>

#include <cstring>

#include "joseph.cuh"
#include "udev_internal.cuh"

namespace {

constexpr int kTX = 32;
constexpr int kTY = 8;
constexpr int kPY = 16;              /* pixels per thread (one column); 8 for few-tile launches */
constexpr int kTileX = kTX;          /* tile is kTileX x (kTY * PY) pixels */
constexpr int kTileY = kTY * kPY;
constexpr int kAC = 32;              /* angles per chunk */
constexpr int kWin = 160;            /* detector window per angle (tile span <= 131, +5 margin, +3 alignment) */
constexpr int kMaxSub = 16;



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
    int contiguous;      /* subsets cover [first_angle, first_angle + total) in order */
    int first_angle;
    float neg_zero;      /* -0.0f: the addend of unfusable packed products */
    unsigned int sub_offset[kMaxSub];
    unsigned int sub_n[kMaxSub];
};

/* Per angle of a chunk: cos, sin, and the first detector of its window
 * (as int bits); one 16-byte shared load. */
template <int PY>
struct __align__(16) BpSmemT {
    float win[2][kAC][kWin];
    float4 ang[2][kAC];
    /* (-fY) * sin for the tile's rows, [angle][ty][pixel p of the thread's
     * column, 4 per float4]: the same for all 32 lanes of a warp */
    float4 nys[2][kAC][kTY][PY / 4];
};
typedef BpSmemT<kPY> BpSmem;

__device__ __forceinline__ void cp_async4(float *dst, const float *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t) __cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}

__device__ __forceinline__ void cp_async16(float *dst, const float *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t) __cvta_generic_to_shared(dst)),
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
    if (P.contiguous)
        return P.first_angle + vi;
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

/*
 * Stages the windows of one chunk of angles. Each window starts at a detector
 * whose global address is 16-byte aligned, at most 3 before the leftmost
 * reachable tap, so the bulk of it moves in 16-byte cp.async copies; groups
 * that cross the ends of the detector row go element by element, with zeros
 * outside [0, n).
 */
template <bool FM, int PY>
__device__ void load_chunk(const BpTileArgs &P, BpSmemT<PY> &S, int buf, int chunk, const float *sino, int x0, int y0,
                           const joseph::AxisConsts &k, float e0, float e1, float shift)
{
    constexpr int kTileH = kTY * PY;
    const int tid = threadIdx.y * kTX + threadIdx.x;
    const int first = chunk * kAC;
    const int count = min(kAC, P.total_angles - first);
    if (tid < count) {
        const int a = angle_of(P, first + tid);
        const float cs = __ldg(P.cosv + a), sn = __ldg(P.sinv + a);
        const float fx0 = __fsub_rn(__fadd_rn((float) x0, 0.5f), k.os);
        const float fx1 = __fsub_rn(__fadd_rn((float) (x0 + kTileX - 1), 0.5f), k.os);
        const float fy0 = __fsub_rn(__fadd_rn((float) y0, 0.5f), k.os);
        const float fy1 = __fsub_rn(__fadd_rn((float) (y0 + kTileH - 1), 0.5f), k.os);
        const float c00 = det_coord(fx0, fy0, cs, sn, shift), c10 = det_coord(fx1, fy0, cs, sn, shift);
        const float c01 = det_coord(fx0, fy1, cs, sn, shift), c11 = det_coord(fx1, fy1, cs, sn, shift);
        float lo = fminf(fminf(c00, c10), fminf(c01, c11));
        lo = fminf(fmaxf(lo, e0), e1);
        int w0 = (int) floorf(__fsub_rn(lo, 0.5f)) - 2;
        const int mis = (int) ((reinterpret_cast<uintptr_t>(sino + (size_t) a * P.n) >> 2) & 3);
        w0 -= (w0 + mis) & 3;
        S.ang[buf][tid] = make_float4(cs, sn, __int_as_float(w0), 0.0f);
    }
    __syncthreads();
    /* row products of the chunk's angles, rounded as the in-loop product
     * (fast arithmetic: with the shift already added) */
    float *nys = reinterpret_cast<float *>(&S.nys[buf][0][0][0]);
    for (int idx = tid; idx < count * kTileH; idx += kTX * kTY) {
        const int slot = idx / kTileH, r = idx % kTileH;      /* row r = ty + kTY * p */
        const float nfy = -__fsub_rn(__fadd_rn((float) (y0 + r), 0.5f), k.os);
        const float prod = __fmul_rn(nfy, S.ang[buf][slot].y);
        nys[(slot * kTY + r % kTY) * PY + r / kTY] = FM ? __fadd_rn(prod, shift) : prod;
    }
    constexpr int kGroups = kWin / 4;
    for (int idx = tid; idx < count * kGroups; idx += kTX * kTY) {
        const int slot = idx / kGroups, g = idx % kGroups;
        const int a = angle_of(P, first + slot);
        const int d = __float_as_int(S.ang[buf][slot].z) + 4 * g;
        float *dst = &S.win[buf][slot][4 * g];
        const float *src = sino + (size_t) a * P.n + d;
        if (d >= 0 && d + 4 <= P.n) {
            cp_async16(dst, src);
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                if (d + e >= 0 && d + e < P.n)
                    cp_async4(dst + e, src + e);
                else
                    dst[e] = 0.0f;
            }
        }
    }
}

/*
 * All angles of one staged chunk for the thread's 16 pixels, two pixels per
 * packed instruction. FAST: every clamped coordinate is >= 0.5, so the
 * three-step floor applies.
 */
template <bool CLAMP, bool FAST, bool FM, int PY>
__device__ __forceinline__ void sample_chunk(const BpSmemT<PY> &S, int buf, int count, int first_vi,
                                             const BpTileArgs &P, float fX, float shift, float e0, float e1,
                                             float2 sum[PY / 2], float2 v[PY / 2], int &sub, int &sub_end)
{
    const uint32_t win0 = (uint32_t) __cvta_generic_to_shared(&S.win[buf][0][0]);
    const uint32_t bits = FAST ? (uint32_t) joseph::kHalfFloorBits : (uint32_t) joseph::kFloorMagicBits;
    const float2 shift2 = joseph::splat(shift);
    const float2 z2 = joseph::splat(P.neg_zero);
    for (int i = 0; i < count; ++i) {
        const int vi = first_vi + i;
        if (vi == sub_end) {
            /* end of a subset: v = v + relax * sum (one BP launch of the reference) */
#pragma unroll
            for (int q = 0; q < PY / 2; ++q) {
                v[q] = joseph::add2(v[q], joseph::mul2z(joseph::splat(P.relax), sum[q], joseph::splat(P.neg_zero)));
                sum[q] = make_float2(0.0f, 0.0f);
            }
            ++sub;
            sub_end += (int) P.sub_n[sub];
        }
        const float4 ang = S.ang[buf][i];
        float2 nys[PY / 2];
#pragma unroll
        for (int f = 0; f < PY / 4; ++f) {
            const float4 ny = S.nys[buf][i][threadIdx.y][f];
            nys[2 * f] = make_float2(ny.x, ny.y);
            nys[2 * f + 1] = make_float2(ny.z, ny.w);
        }
        /* shared address of detector 0 of this angle's window, less the floor bits */
        const uint32_t base = win0 + 4u * (uint32_t) (i * kWin) - 4u * ((uint32_t) __float_as_int(ang.z) + bits);
        const float2 fxc = joseph::splat(__fmul_rn(fX, ang.x));
#pragma unroll
        for (int q = 0; q < PY / 2; ++q) {
            /* fX * cos - fY * sin + shift, as fX*cos + (-fY)*sin + shift
             * (fast arithmetic: fX*cos + ((-fY)*sin + shift)) */
            float2 sc = FM ? joseph::add2(fxc, nys[q]) : joseph::add2(joseph::add2(fxc, nys[q]), shift2);
            if (CLAMP) {
                sc.x = fminf(fmaxf(sc.x, e0), e1);
                sc.y = fminf(fmaxf(sc.y, e0), e1);
            }
            float2 t;
            const float2 y = FAST ? joseph::floor_half2(sc, t) : joseph::floor_any2(sc, t);
            const uint32_t a0 = base + 4u * (uint32_t) __float_as_int(y.x);
            const uint32_t a1 = base + 4u * (uint32_t) __float_as_int(y.y);
            const float2 t0 = make_float2(joseph::lds(a0), joseph::lds(a1));
            const float2 t1 = make_float2(joseph::lds(a0 + 4u), joseph::lds(a1 + 4u));
            sum[q] = FM ? joseph::lerp_acc_fast2(sum[q], t, t0, t1) : joseph::add2(sum[q], joseph::lerp2(t, t0, t1, z2));
        }
    }
}

/* One CTA's work: pixel tile `tile` of slice `slice`. */
template <bool FM, int PY>
__device__ __forceinline__ void bp_tile(const BpTileArgs &P, BpSmemT<PY> &S, int tile, int slice)
{
    constexpr int kTileH = kTY * PY;
    const int n = P.n;
    const int tiles_x = (n + kTileX - 1) / kTileX;
    const int x0 = (tile % tiles_x) * kTileX;
    const int y0 = (tile / tiles_x) * kTileH;
    const float *sino = P.sino + (size_t) slice * P.sino_stride;

    const joseph::AxisConsts k = joseph::axis_consts(n, P.axis);
    float e0, e1;
    joseph::bp_edges(k, n, P.axis, e0, e1);
    const float shift = __fsub_rn(k.os, k.ros);

    const int x = x0 + (int) threadIdx.x;
    const float fX = __fsub_rn(__fadd_rn((float) x, 0.5f), k.os);
    /* pixel pairs (p, p + 1) of the thread's column */
    float2 sum[PY / 2], v[PY / 2];
#pragma unroll
    for (int q = 0; q < PY / 2; ++q) {
        float b[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int y = y0 + (int) threadIdx.y + kTY * (2 * q + h);
            const size_t pix = (size_t) slice * P.vol_stride + (size_t) y * n + x;
            b[h] = (P.base && x < n && y < n) ? P.base[pix] : 0.0f;
        }
        v[q] = make_float2(b[0], b[1]);
        sum[q] = make_float2(0.0f, 0.0f);
    }

    /* A tile whose every pixel lies within distance (n/2 - 2) of the centre
     * never reaches the clamp edges (on-axis geometry), so the clamp can be
     * skipped without changing any result; its coordinates lie in
     * [2, n - 2]. */
    bool clamp = true;
    if (k.diff == 0.0f) {
        const float r = 0.5f * (float) n - 2.0f;
        const float ax = fmaxf(fabsf((float) x0 - k.os), fabsf((float) (x0 + kTileX) - k.os));
        const float ay = fmaxf(fabsf((float) y0 - k.os), fabsf((float) (y0 + kTileH) - k.os));
        clamp = ax * ax + ay * ay > r * r;
    }
    /* clamped coordinates are >= min(e0, e1) */
    const bool fast = fminf(e0, e1) >= 0.5f;

    const int nchunks = (P.total_angles + kAC - 1) / kAC;
    int sub = 0;
    int sub_end = P.n_subsets > 0 ? (int) P.sub_n[0] : 0;
    if (nchunks > 0) {
        load_chunk<FM, PY>(P, S, 0, 0, sino, x0, y0, k, e0, e1, shift);
        cp_async_commit();
    }
    for (int ch = 0; ch < nchunks; ++ch) {
        const int buf = ch & 1;
        if (ch + 1 < nchunks) {
            load_chunk<FM, PY>(P, S, buf ^ 1, ch + 1, sino, x0, y0, k, e0, e1, shift);
            cp_async_commit();
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const int count = min(kAC, P.total_angles - ch * kAC);
        if (!clamp)
            sample_chunk<false, true, FM, PY>(S, buf, count, ch * kAC, P, fX, shift, e0, e1, sum, v, sub, sub_end);
        else if (fast)
            sample_chunk<true, true, FM, PY>(S, buf, count, ch * kAC, P, fX, shift, e0, e1, sum, v, sub, sub_end);
        else
            sample_chunk<true, false, FM, PY>(S, buf, count, ch * kAC, P, fX, shift, e0, e1, sum, v, sub, sub_end);
        __syncthreads();
    }
    if (P.n_subsets > 0) {
#pragma unroll
        for (int q = 0; q < PY / 2; ++q)
            v[q] = joseph::add2(v[q], joseph::mul2z(joseph::splat(P.relax), sum[q], joseph::splat(P.neg_zero)));
    }
    if (x >= n)
        return;
#pragma unroll
    for (int p = 0; p < PY; ++p) {
        const int y = y0 + (int) threadIdx.y + kTY * p;
        if (y >= n)
            continue;
        float r = (p & 1) ? v[p >> 1].y : v[p >> 1].x;
        if (P.cw)
            r = __fmul_rn(r, P.cw[(size_t) slice * P.cw_stride + (size_t) y * n + x]);
        const size_t pix = (size_t) slice * P.vol_stride + (size_t) y * n + x;
        if (P.add)
            r = __fadd_rn(r, P.add[pix]);
        P.dst[pix] = r;
    }
}

template <bool FM, int PY>
__global__ void __launch_bounds__(kTX * kTY) bp_tiles_kernel(const __grid_constant__ BpTileArgs P)
{
    __shared__ BpSmemT<PY> S;
    bp_tile<FM, PY>(P, S, (int) blockIdx.x, (int) blockIdx.y);
}

/*
 * Mixed batch: the pixel tiles of many one-slice jobs (any size and angle
 * count) in one launch. CTA b belongs to the job j with item_start[j] <= b <
 * item_start[j + 1]; its record (the job's BpTileArgs) is staged in shared
 * memory. Jobs whose active flag is 0 are skipped.
 */
template <bool FM>
__global__ void __launch_bounds__(kTX * kTY, 3) bp_tiles_batch_kernel(const BpTileArgs *__restrict__ recs,
                                                                   const int *__restrict__ item_start, int n_jobs,
                                                                   const int *__restrict__ job_index,
                                                                   const int *__restrict__ active)
{
    __shared__ BpSmem S;
    __shared__ BpTileArgs rec;
    __shared__ int job_s;
    const int b = (int) blockIdx.x;
    const int tid = (int) (threadIdx.y * kTX + threadIdx.x);
    if (tid == 0) {
        int lo = 0, hi = n_jobs - 1;      /* last j with item_start[j] <= b */
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(item_start + mid) <= b)
                lo = mid;
            else
                hi = mid - 1;
        }
        job_s = lo;
    }
    __syncthreads();
    const int j = job_s;
    if (!__ldg(active + __ldg(job_index + j)))
        return;
    {
        const int *src = reinterpret_cast<const int *>(recs + j);
        int *dst = reinterpret_cast<int *>(&rec);
        for (int e = tid; e < (int) (sizeof(BpTileArgs) / sizeof(int)); e += kTX * kTY)
            dst[e] = __ldg(src + e);
    }
    __syncthreads();
    bp_tile<FM, kPY>(rec, S, b - __ldg(item_start + j), 0);
}

static_assert(sizeof(BpTileArgs) % sizeof(int) == 0, "records are copied as ints");

/* The arguments of one BP launch (udev_bp_tiles' contract) for one slice. */
static int fill_args(udev *d, const udev_geom *g, const ufoir_subset *subsets, int n_subsets, const float *sino,
                     const float *base, const float *cw, int cw_shared, const float *add, float *dst, float relax,
                     BpTileArgs &A)
{
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
    memset(&A, 0, sizeof(A));
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
    A.neg_zero = -0.0f;
    A.contiguous = 1;
    A.first_angle = n_subsets > 0 ? (int) subsets[0].offset : 0;
    for (int i = 1; i < n_subsets; i++)
        if (subsets[i].offset != subsets[i - 1].offset + subsets[i - 1].n)
            A.contiguous = 0;
    for (int i = 0; i < kMaxSub; i++) {
        A.sub_offset[i] = i < n_subsets ? subsets[i].offset : 0;
        A.sub_n[i] = i < n_subsets ? subsets[i].n : 0;
    }
    return UFOIR_OK;
}

}  // namespace

extern "C" size_t udev_bp_record_bytes(void)
{
    return sizeof(BpTileArgs);
}

extern "C" int udev_bp_record(udev *d, const udev_geom *g, const ufoir_subset *subsets, int n_subsets,
                              const float *sino, const float *base, const float *cw, const float *add, float *dst,
                              float relax, void *record, int *items)
{
    BpTileArgs A;
    const int rc = fill_args(d, g, subsets, n_subsets, sino, base, cw, 0, add, dst, relax, A);
    if (rc)
        return rc;
    memcpy(record, &A, sizeof(A));
    const int tiles_x = (g->n_dets + kTileX - 1) / kTileX;
    const int tiles_y = (g->n_dets + kTileY - 1) / kTileY;
    *items = tiles_x * tiles_y;
    return UFOIR_OK;
}

extern "C" int udev_bp_batch(udev *d, int fast_arith, const void *d_records, const int *d_item_start, int n_jobs,
                             const int *d_job_index, const int *d_active, int n_items)
{
    if (n_jobs <= 0 || n_items <= 0)
        return UFOIR_OK;
    UDEV_BIND(d);
    if (fast_arith)
        bp_tiles_batch_kernel<true><<<(unsigned int) n_items, dim3(kTX, kTY), 0, d->stream>>>(
            static_cast<const BpTileArgs *>(d_records), d_item_start, n_jobs, d_job_index, d_active);
    else
        bp_tiles_batch_kernel<false><<<(unsigned int) n_items, dim3(kTX, kTY), 0, d->stream>>>(
            static_cast<const BpTileArgs *>(d_records), d_item_start, n_jobs, d_job_index, d_active);
    return udev_after_launch(d, "bp_tiles_batch_kernel");
}

extern "C" int udev_bp_tiles(udev *d, const udev_geom *g, const ufoir_subset *subsets, int n_subsets,
                             const float *sino, const float *base, const float *cw, int cw_shared, const float *add,
                             float *dst, float relax, int n_slices)
{
    if (n_slices <= 0)
        return UFOIR_OK;
    BpTileArgs A;
    const int rc0 = fill_args(d, g, subsets, n_subsets, sino, base, cw, cw_shared, add, dst, relax, A);
    if (rc0)
        return rc0;
    UDEV_BIND(d);
    /* Tiles of 16 pixels per thread (32 x 128) unless the launch has fewer than
     * three waves of them (three CTAs per SM): then 8 per thread (32 x 64), whose
     * last wave is fuller. At 1448^2 x 1200 one slice's BP took 1.131 instead of
     * 1.194 ms, two slices' 2.155 instead of 2.266; three slices (3.6 waves)
     * keep the tall tiles (3.130 against 3.197 ms). */
    const int tiles_x = (g->n_dets + kTileX - 1) / kTileX;
    const long long tiles16 = (long long) tiles_x * ((g->n_dets + kTileY - 1) / kTileY);
    const bool short_tiles = tiles16 * n_slices < 3LL * 3 * udev_sm_count(d);
    const int tile_h = short_tiles ? kTY * 8 : kTileY;
    const unsigned int n_tiles = (unsigned int) (tiles_x * ((g->n_dets + tile_h - 1) / tile_h));
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
        const dim3 grid(n_tiles, (unsigned int) chunk), block(kTX, kTY);
        if (g->fast_arith && short_tiles)
            bp_tiles_kernel<true, 8><<<grid, block, 0, d->stream>>>(B);
        else if (g->fast_arith)
            bp_tiles_kernel<true, kPY><<<grid, block, 0, d->stream>>>(B);
        else if (short_tiles)
            bp_tiles_kernel<false, 8><<<grid, block, 0, d->stream>>>(B);
        else
            bp_tiles_kernel<false, kPY><<<grid, block, 0, d->stream>>>(B);
        int rc = udev_after_launch(d, "bp_tiles_kernel");
        if (rc)
            return rc;
        done += chunk;
    }
    return UFOIR_OK;
}
