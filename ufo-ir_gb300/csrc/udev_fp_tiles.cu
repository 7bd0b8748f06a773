/*
 * udev_fp_tiles.cu - the forward projector for whole angle sets (every
 * method's A x), streaming image rows through shared memory.
 *
 * Layout: the volume (for vertical rays) and its transpose (for horizontal
 * rays) are first written as padded copies, each row [2 zeros | n values |
 * zeros] of `pitch` floats (pitch % 4 == 0), so that every ray of either
 * direction walks the rows of a row-major image and a zero border needs no
 * bounds checks. One CTA owns a tile of up to A consecutive angles of one
 * direction and all n detectors (J per thread, lanes on adjacent
 * detectors). All of its A*n rays advance row by row in lockstep; chunks of
 * K rows (K | 64) are brought into shared memory by a single 1-D TMA bulk
 * copy each (cp.async.bulk + mbarrier, double buffered), and every row in
 * shared memory is sampled by all A*n rays, so the image is read from L2
 * once per tile instead of once per ray.
 *
 * When there are too few tiles to fill the GPU (one slice, few angles), a
 * tile's detectors are split over several CTAs. Each then stages only a
 * window of each chunk's rows: the columns its rays can reach, bounded by
 * the extreme rays of its angles (the coordinate is monotone in detector and
 * row), one 1-D copy per row, with two zero slots after the window for taps
 * outside it (they lie outside the image). 2900^2 x 90 angles: 925 -> 818 us.
 *
 * Arithmetic is the reference's: per ray, the float coordinate recurrence,
 * one linear-filter sample per row with (1 - t) * T0 + t * T1, samples
 * summed in blocks of 64, then sino = src + scale * sum
 * (projector-parallel-joseph.cl:36-156). floor() is taken with a
 * round-toward-minus-infinity add of 1.5 * 2^23 instead of conversion
 * instructions; for |x| < 2^22 it is exact.
 */
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "joseph.cuh"
#include "tma.cuh"
#include "udev_internal.cuh"

namespace {

constexpr int kPadL = 2;
constexpr int kHeader = 256;   /* shared bytes before the stages: barriers, window starts, extreme rays */
/* bits of floor(c - 0.5) + 1.5 * 2^23, less the padded column of index 0 */
constexpr int kColBits = joseph::kFloorMagicBits - kPadL;

struct FpTileArgs {
    const float *volP;
    const float *volTP;
    const float *src;
    const float *w;
    float *out;
    const float *sinv;
    const float *cosv;
    const int4 *tiles;     /* {first angle, angle count, direction, 0} */
    int n;
    int pitch;
    int rows_per_chunk;
    float axis;
    float scale;
    long long volp_stride;
    long long sino_stride;
    long long w_stride;
    float neg_zero;        /* -0.0f: the addend of unfusable packed products */
    int dsplit;            /* CTAs per angle tile, each on a range of dper detectors */
    int dper;
    int wcols;             /* columns staged per row: pitch (whole rows), or a window of the CTA's rays */
    int wstride;           /* shared floats per staged row (wcols + 4 for windows: 2 zero slots) */
    int margin;            /* window margin in columns (the recurrence's drift and the filter's taps) */
    int skip_chunk;        /* testing: row chunk whose barrier never completes (-1 = none) */
    int *err;
};

static_assert(sizeof(FpTileArgs) % sizeof(int) == 0, "records are copied as ints");
/* static shared memory of the batch kernel (its record and job index), rounded up */
constexpr size_t kBatchStatic = (sizeof(FpTileArgs) + 16 + 127) / 128 * 128;

constexpr int kMaxWinThreads = 448;   /* detector-split CTAs hold at most half the slots */

/* Windowed CTAs of the J = 1 variants made for large n (A <= 4) hold few
 * rays per thread: two of them per SM. (The A = 8 variant, the default at
 * n <= 768, measured 4 % slower held to that register budget.) */
/* One CTA's work: angle tile `tile_idx` of P.tiles, detector part `dpart`
 * of P.dsplit, slice `slice`; smem_raw is the dynamic shared memory. */
template <int J, int A, bool WIN, bool FM>
__device__ __forceinline__ void fp_tile(const FpTileArgs &P, int tile_idx, int dpart, int slice,
                                        unsigned char *smem_raw)
{
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem_raw);
    int *w0s = reinterpret_cast<int *>(smem_raw + 16);     /* window start of each stage */
    float *ext = reinterpret_cast<float *>(smem_raw + 32);   /* [3][A]: extreme rays' starts, steps */
    float *stage0 = reinterpret_cast<float *>(smem_raw + kHeader);
    const int K = P.rows_per_chunk;
    const int pitch = P.pitch;
    /* WIN: rows staged as column windows (wcols of them, stride wstride) */
    const int wcols = WIN ? P.wcols : pitch, wstride = WIN ? P.wstride : pitch;
    constexpr bool win = WIN;
    const size_t stage_floats = (size_t) K * wstride;

    const int4 tile = P.tiles[tile_idx];
    const int n = P.n;
    const int dir = tile.z;
    /* detector range of this CTA: [dstart, dend) */
    const int dstart = dpart * P.dper;
    const int dend = min(n, dstart + P.dper);
    const float *img = (dir == 0 ? P.volTP : P.volP) + (size_t) slice * P.volp_stride;

    const joseph::AxisConsts kc = joseph::axis_consts(n, P.axis);
    /* Lanes: each warp holds 16 detector slots x 2 adjacent angles (the
     * half-warp g takes the tile's angles g, g + 2, g + 4, ...). Rays of
     * adjacent angles through adjacent detectors meet a row within ~25
     * words, so a warp's shared loads stay free of bank conflicts, which 32
     * adjacent detectors of one angle (spread 1/|cos| apart) are not.
     * A thread owns A/2 angles x 2J detectors d0 + 16 i, so a warp's rays
     * are 32J adjacent detectors of A adjacent angles, which cross the
     * image together (see the chunk modes below); detectors (2m, 2m + 1) of
     * one angle travel as a pair through packed FP32. Slots past the tile's
     * angles or the CTA's detectors repeat its last angle or detector (their
     * sums are not written), so every slot holds a ray of the image. */
    constexpr int A2 = A / 2;
    const int lane = (int) (threadIdx.x & 31);
    const int g = lane >> 4;
    const int d0 = dstart + (int) (threadIdx.x >> 5) * 32 * J + (lane & 15);
    float2 c[A2][J], inner[A2][J], sum[A2][J], stp[A2];
#pragma unroll
    for (int k = 0; k < A2; ++k) {
        const int angle = tile.x + min(g + 2 * k, tile.y - 1);
        float st, det_step;
        joseph::ray_steps(dir, __ldg(P.sinv + angle), __ldg(P.cosv + angle), det_step, st);
        stp[k] = joseph::splat(st);
#pragma unroll
        for (int m = 0; m < J; ++m) {
            const int s0 = min(d0 + 32 * m, dend - 1), s1 = min(d0 + 32 * m + 16, dend - 1);
            c[k][m] = make_float2(joseph::ray_start(kc, s0, n, det_step, st), joseph::ray_start(kc, s1, n, det_step, st));
            inner[k][m] = make_float2(0.0f, 0.0f);
            sum[k][m] = make_float2(0.0f, 0.0f);
        }
    }

    const int nchunks = (n + K - 1) / K;
    /* Windowed rows (detector-split CTAs): a chunk stages only the columns
     * its rays can reach. The coordinate is monotone in the detector and in
     * the row, so over the CTA's rays and the chunk's rows it lies between
     * its values at the extreme detectors and rows, per angle; thread 0 keeps
     * those rays' starts and steps. Taps outside the window read two zero
     * slots after it, as taps outside the image read the zero border. */
    if (win && threadIdx.x < A) {
        const int a = (int) threadIdx.x;
        float det_step = 0.0f, st = 0.0f;
        if (a < tile.y)
            joseph::ray_steps(dir, __ldg(P.sinv + tile.x + a), __ldg(P.cosv + tile.x + a), det_step, st);
        ext[a] = a < tile.y ? joseph::ray_start(kc, dstart, n, det_step, st) : 0.0f;
        ext[A + a] = a < tile.y ? joseph::ray_start(kc, dend - 1, n, det_step, st) : 0.0f;
        ext[2 * A + a] = st;
    }
    /* window start (a multiple of 4 columns) of the chunk at row r0 */
    auto window = [&](int r0, int rows) -> int {
        /* in FP32: the rounding (< 1e-3 column here) is covered by the margin */
        float lo = 1e30f, hi = -1e30f;
        const float ya = (float) r0, yb = (float) (r0 + rows - 1);
        for (int a = 0; a < tile.y; ++a) {
            const float c0 = ext[a], c1 = ext[A + a], st = ext[2 * A + a];
            lo = fminf(lo, fminf(fminf(c0 + ya * st, c0 + yb * st), fminf(c1 + ya * st, c1 + yb * st)));
            hi = fmaxf(hi, fmaxf(fmaxf(c0 + ya * st, c0 + yb * st), fmaxf(c1 + ya * st, c1 + yb * st)));
        }
        const int clo = (int) floorf(lo - 0.5f) + kPadL - P.margin;
        const int chi = (int) floorf(hi - 0.5f) + kPadL + 1 + P.margin;
        int w0 = (clo >= 0 ? clo : clo - 3) / 4 * 4;
        w0 = max(0, min(w0, pitch - wcols));
        if (min(chi, kPadL + n - 1) >= w0 + wcols)
            atomicOr(P.err, tma::kErrWindow);      /* the host's width bound was too small */
        return w0;
    };
    if (threadIdx.x == 0) {
        tma::mbar_init(&bars[0], 1);
        tma::mbar_init(&bars[1], 1);
        tma::fence_mbar_init();
    }
    if (win)
        for (int e = (int) threadIdx.x; e < 2 * K * 4; e += (int) blockDim.x)
            stage0[(size_t) (e >> 2) * wstride + wcols + (e & 3)] = 0.0f;
    __syncthreads();

    /* issue the copy of chunk ch into stage ch & 1 */
    auto issue = [&](int ch) {
        const int r0 = ch * K, rows = min(K, n - r0);
        float *dst = stage0 + (ch & 1) * stage_floats;
        /* testing (ufoir_ctx_inject_copy_timeout): the barrier of chunk
         * skip_chunk expects 16 bytes more than its copies bring, so its
         * phase never completes, its waits run out and the error path runs.
         * (Written as arithmetic: a branch here cost the kernel 5 %.) */
        const uint32_t extra = ch == P.skip_chunk ? 16u : 0u;
        if (!win) {
            const uint32_t bytes = (uint32_t) (rows * pitch) * 4u;
            w0s[ch & 1] = 0;
            tma::mbar_arrive_expect_tx(&bars[ch & 1], bytes + extra);
            tma::bulk_g2s(dst, img + (size_t) r0 * pitch, bytes, &bars[ch & 1]);
        } else {
            const int w0 = window(r0, rows);
            w0s[ch & 1] = w0;
            tma::mbar_arrive_expect_tx(&bars[ch & 1], (uint32_t) (rows * wcols) * 4u + extra);
            for (int r = 0; r < rows; ++r)
                tma::bulk_g2s(dst + (size_t) r * wstride, img + (size_t) (r0 + r) * pitch + w0,
                              (uint32_t) wcols * 4u, &bars[ch & 1]);
        }
    };
    int issued = 0;
    if (threadIdx.x == 0)
        for (; issued < 2 && issued < nchunks; ++issued)
            issue(issued);

    /* A tap pair starts at padded column floor(c - 0.5) + kPadL; pairs that
     * start outside [0, n + 2] lie wholly in the zero border, so the start
     * is clamped (as unsigned) to n + 2, whose taps are two pad zeros.
     * Each warp picks one of three forms per chunk, from its rays'
     * coordinates at the chunk's first and last rows (monotone along a ray;
     * the float recurrence drifts < 0.03 columns over a chunk, and the
     * bounds keep 0.25):
     *  - inside: every coordinate lies in [0.5, n + 1.5) and in the staged
     *    columns, so floor(c - 0.5) takes the three-operation form
     *    (floor_half2) and the tap address is one multiply-add on its bits,
     *    with no clamp;
     *  - outside: every coordinate is below -0.5 or at least n + 0.5, where
     *    both taps are border zeros. Only the recurrence advances: adding
     *    +-0 leaves a block sum unchanged (it starts at +0 and a sum of
     *    finite floats in round-to-nearest is never -0);
     *  - otherwise the general form above. */
    const uint32_t col_lim = (uint32_t) n + 2u;
    const float2 z2 = joseph::splat(P.neg_zero);
    const uint32_t stage_s = (uint32_t) __cvta_generic_to_shared(stage0);
    bool ok = true;
    int waited = 0;
    for (int ch = 0; ch < nchunks; ++ch) {
        const int st = ch & 1;
        if (ok) {
            ok = tma::mbar_wait(&bars[st], (uint32_t) ((ch >> 1) & 1), P.err, tma::kErrWaitTimeout);
            if (ok)
                waited = ch + 1;   /* chunks [0, waited) have landed */
        }
        const int r0 = ch * K;
        const int rows = min(K, n - r0);
        if (ok) {
            const uint32_t row_s0 = stage_s + 4u * (uint32_t) (st * (int) stage_floats);
            /* padded column - window start, clamped (as unsigned) to the zero taps */
            const int w0 = WIN ? w0s[st] : 0;
            const int colbits = kColBits + w0;
            const uint32_t lim = WIN ? (uint32_t) wcols : col_lim;
            /* the chunk's form */
            const float span = (float) (rows - 1);
            const float in_lo = fmaxf(0.5f, (float) (w0 - kPadL) + 0.5f) + 0.25f;
            const float in_hi = (float) ((int) lim - kPadL + w0) + 1.25f;
            const float out_hi = (float) n + 0.75f;
            bool inside = true, outside = true;
#pragma unroll
            for (int k = 0; k < A2; ++k)
#pragma unroll
                for (int m = 0; m < J; ++m) {
                    const float ex = fmaf(span, stp[k].x, c[k][m].x), ey = fmaf(span, stp[k].y, c[k][m].y);
                    const float lo = fminf(fminf(c[k][m].x, ex), fminf(c[k][m].y, ey));
                    const float hi = fmaxf(fmaxf(c[k][m].x, ex), fmaxf(c[k][m].y, ey));
                    inside = inside && lo >= in_lo && hi < in_hi;
                    const bool xo = fmaxf(c[k][m].x, ex) < -0.75f || fminf(c[k][m].x, ex) >= out_hi;
                    const bool yo = fmaxf(c[k][m].y, ey) < -0.75f || fminf(c[k][m].y, ey) >= out_hi;
                    outside = outside && xo && yo;
                }
            inside = __all_sync(0xffffffffu, inside);
            outside = !inside && __all_sync(0xffffffffu, outside);
            if (inside) {
                /* address = row + 4 (floor(c - 0.5) + kPadL - w0) = base + 4 bits(y) */
                uint32_t base = row_s0 + 4u * (uint32_t) (kPadL - w0) - 4u * (uint32_t) joseph::kHalfFloorBits;
                for (int r = 0; r < rows; ++r, base += 4u * (uint32_t) wstride) {
#pragma unroll
                    for (int k = 0; k < A2; ++k) {
#pragma unroll
                        for (int m = 0; m < J; ++m) {
                            float2 t;
                            const float2 y = joseph::floor_half2(c[k][m], t);
                            const uint32_t a0 = base + 4u * (uint32_t) __float_as_int(y.x);
                            const uint32_t a1 = base + 4u * (uint32_t) __float_as_int(y.y);
                            const float2 t0 = make_float2(joseph::lds(a0), joseph::lds(a1));
                            const float2 t1 = make_float2(joseph::lds(a0 + 4u), joseph::lds(a1 + 4u));
                            inner[k][m] = FM ? joseph::lerp_acc_fast2(inner[k][m], t, t0, t1)
                                             : joseph::add2(inner[k][m], joseph::lerp2(t, t0, t1, z2));
                            c[k][m] = joseph::add2(c[k][m], stp[k]);
                        }
                    }
                }
            } else if (outside) {
                for (int r = 0; r < rows; ++r) {
#pragma unroll
                    for (int k = 0; k < A2; ++k)
#pragma unroll
                        for (int m = 0; m < J; ++m)
                            c[k][m] = joseph::add2(c[k][m], stp[k]);
                }
            } else {
                uint32_t row_s = row_s0;
                for (int r = 0; r < rows; ++r, row_s += 4u * (uint32_t) wstride) {
#pragma unroll
                    for (int k = 0; k < A2; ++k) {
#pragma unroll
                        for (int m = 0; m < J; ++m) {
                            float2 t;
                            const float2 y = joseph::floor_any2(c[k][m], t);
                            const uint32_t p0 = min((uint32_t) (__float_as_int(y.x) - colbits), lim);
                            const uint32_t p1 = min((uint32_t) (__float_as_int(y.y) - colbits), lim);
                            const uint32_t a0 = row_s + 4u * p0, a1 = row_s + 4u * p1;
                            const float2 t0 = make_float2(joseph::lds(a0), joseph::lds(a1));
                            const float2 t1 = make_float2(joseph::lds(a0 + 4u), joseph::lds(a1 + 4u));
                            inner[k][m] = FM ? joseph::lerp_acc_fast2(inner[k][m], t, t0, t1)
                                             : joseph::add2(inner[k][m], joseph::lerp2(t, t0, t1, z2));
                            c[k][m] = joseph::add2(c[k][m], stp[k]);
                        }
                    }
                }
            }
            /* K divides 64: a 64-row block ends only at a chunk's last row */
            if (((r0 + rows) & 63) == 0) {
#pragma unroll
                for (int k = 0; k < A2; ++k)
#pragma unroll
                    for (int m = 0; m < J; ++m) {
                        sum[k][m] = joseph::add2(sum[k][m], inner[k][m]);
                        inner[k][m] = make_float2(0.0f, 0.0f);
                    }
            }
        }
        ok = __syncthreads_and(ok) != 0;
        if (threadIdx.x == 0 && ok && issued < nchunks) {
            /* every thread is done with this stage: refill it */
            tma::fence_proxy_async_smem();
            issue(issued);
            ++issued;
        }
    }
    if (!ok) {
        /* a copy did not arrive in time: drain what was issued (from the
         * first chunk this thread did not see land, the timed-out one
         * included), write nothing */
        if (threadIdx.x == 0)
            for (int ch = waited; ch < issued; ++ch)
                tma::mbar_wait(&bars[ch & 1], (uint32_t) ((ch >> 1) & 1), P.err, tma::kErrDrainTimeout);
        return;
    }

    if ((n & 63) != 0) {
#pragma unroll
        for (int k = 0; k < A2; ++k)
#pragma unroll
            for (int m = 0; m < J; ++m)
                sum[k][m] = joseph::add2(sum[k][m], inner[k][m]);
    }
#pragma unroll
    for (int k = 0; k < A2; ++k) {
        const int a = g + 2 * k;
        if (a >= tile.y)
            continue;
        const int angle = tile.x + a;
#pragma unroll
        for (int i = 0; i < 2 * J; ++i) {
            const int s = d0 + i * 16;
            if (s >= dend)
                continue;
            const size_t oidx = (size_t) slice * P.sino_stride + (size_t) angle * n + s;
            float result = P.src[oidx];
            const float ray = (i & 1) ? sum[k][i >> 1].y : sum[k][i >> 1].x;
            if (!joseph::detector_inactive(kc, s))
                result = __fadd_rn(result, __fmul_rn(ray, P.scale));
            if (P.w)
                result = __fmul_rn(result, P.w[(size_t) slice * P.w_stride + (size_t) angle * n + s]);
            P.out[oidx] = result;
        }
    }
}

template <int J, int A, bool WIN, bool FM>
__global__ void __launch_bounds__(WIN ? kMaxWinThreads : 768, (WIN && J == 1 && A <= 4) ? 2 : 1)
    fp_tiles_kernel(const __grid_constant__ FpTileArgs P)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    fp_tile<J, A, WIN, FM>(P, (int) (blockIdx.x / (unsigned) P.dsplit), (int) (blockIdx.x % (unsigned) P.dsplit),
                       (int) blockIdx.y, smem_raw);
}

/*
 * Mixed batch: the tiles of many one-slice jobs (any n_angles, same launch
 * shape) in one launch. CTA b belongs to the job j with item_start[j] <= b <
 * item_start[j + 1]; its record (the job's FpTileArgs) is staged in shared
 * memory. Jobs whose active flag is 0 are skipped.
 */
template <int J, int A, bool WIN, bool FM>
__global__ void __launch_bounds__(WIN ? kMaxWinThreads : 768, (WIN && J == 1 && A <= 4) ? 2 : 1)
    fp_tiles_batch_kernel(const FpTileArgs *__restrict__ recs, const int *__restrict__ item_start, int n_jobs,
                          const int *__restrict__ job_index, const int *__restrict__ active)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ FpTileArgs rec;
    __shared__ int job_s;
    const int b = (int) blockIdx.x;
    if (threadIdx.x == 0) {
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
        for (int e = (int) threadIdx.x; e < (int) (sizeof(FpTileArgs) / sizeof(int)); e += (int) blockDim.x)
            dst[e] = __ldg(src + e);
    }
    __syncthreads();
    const int local = b - __ldg(item_start + j);
    fp_tile<J, A, WIN, FM>(rec, local / rec.dsplit, local % rec.dsplit, 0, smem_raw);
}

/* Writes the padded copy and the padded transpose of n x n slices; the pad
 * columns are left as they are (zeroed once when the buffers are made). */
__global__ void __launch_bounds__(256) pad_transpose_kernel(const float *__restrict__ in, float *__restrict__ outP,
                                                            float *__restrict__ outTP, int n, int pitch,
                                                            long long in_stride, long long out_stride)
{
    __shared__ float tile[32][33];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    const float *src = in + (size_t) blockIdx.z * in_stride;
    float *dp = outP + (size_t) blockIdx.z * out_stride;
    float *dt = outTP + (size_t) blockIdx.z * out_stride;
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int x = bx + threadIdx.x, y = by + j;
        if (x < n && y < n) {
            const float v = src[(size_t) y * n + x];
            tile[j][threadIdx.x] = v;
            dp[(size_t) y * pitch + kPadL + x] = v;
        }
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int x = by + threadIdx.x, y = bx + j;
        if (x < n && y < n)
            dt[(size_t) y * pitch + kPadL + x] = tile[threadIdx.x][j];
    }
}

struct TileCfg {
    int J, A, threads, K;
    size_t smem;
};

constexpr int kMaxTileThreads = 768;

TileCfg tile_cfg(int n, int smem_optin)
{
    TileCfg c;
    c.J = n <= 768 ? 1 : (n <= 1536 ? 2 : (n <= 3072 ? 4 : 8));
    c.A = c.J <= 2 ? 8 : (c.J == 4 ? 4 : 2);
    /* 16 detector slots per warp and angle group, 2J detectors per slot */
    const int slots = (n + 2 * c.J - 1) / (2 * c.J);
    c.threads = (slots + 15) / 16 * 32;
    const int pitch = udev_fp_pitch(n);
    c.K = 32;
    while (c.K > 4 && kHeader + 2 * (size_t) c.K * pitch * 4 > (size_t) smem_optin)
        c.K /= 2;
    c.smem = kHeader + 2 * (size_t) c.K * pitch * 4;
    return c;
}

template <int J, int A, bool WIN, bool FM>
int launch_tiles(udev *d, const FpTileArgs &args, int n_tiles, int n_slices, int threads, size_t smem)
{
    for (int done = 0; done < n_slices;) {
        const int chunk = n_slices - done > 65535 ? 65535 : n_slices - done;
        FpTileArgs B = args;
        B.volP += (size_t) done * args.volp_stride;
        B.volTP += (size_t) done * args.volp_stride;
        B.src += (size_t) done * args.sino_stride;
        B.out += (size_t) done * args.sino_stride;
        if (B.w)
            B.w += (size_t) done * args.w_stride;
        const dim3 grid((unsigned int) (n_tiles * args.dsplit), (unsigned int) chunk);
        fp_tiles_kernel<J, A, WIN, FM><<<grid, threads, smem, d->stream>>>(B);
        int rc = udev_after_launch(d, "fp_tiles_kernel");
        if (rc)
            return rc;
        done += chunk;
    }
    return UFOIR_OK;
}

}  // namespace

extern "C" int udev_fp_pitch(int n)
{
    return (n + kPadL + 2 + 3) / 4 * 4;
}

static bool tiles_supported(const TileCfg &cfg, int smem_optin)
{
    return cfg.threads <= kMaxTileThreads && cfg.smem <= (size_t) smem_optin && cfg.K >= 8;
}

extern "C" int udev_fp_tile_angles(udev *d, int n)
{
    const TileCfg cfg = tile_cfg(n, d->smem_optin);
    return tiles_supported(cfg, d->smem_optin) ? cfg.A : 0;
}

template <bool FM>
static int kernels_init_fm(udev *d)
{
#define UDEV_TILE_ATTR(K_, bytes)                                                                              \
    UDEV_CHECK(d, cudaFuncSetAttribute(K_, cudaFuncAttributeMaxDynamicSharedMemorySize, (bytes)))
    UDEV_TILE_ATTR((fp_tiles_kernel<1, 8, false, FM>), d->smem_optin);
    UDEV_TILE_ATTR((fp_tiles_kernel<2, 8, false, FM>), d->smem_optin);
    UDEV_TILE_ATTR((fp_tiles_kernel<4, 4, false, FM>), d->smem_optin);
    UDEV_TILE_ATTR((fp_tiles_kernel<8, 2, false, FM>), d->smem_optin);
    UDEV_TILE_ATTR((fp_tiles_kernel<1, 8, true, FM>), d->smem_optin);
    UDEV_TILE_ATTR((fp_tiles_kernel<2, 8, true, FM>), d->smem_optin);
    UDEV_TILE_ATTR((fp_tiles_kernel<4, 4, true, FM>), d->smem_optin);
    UDEV_TILE_ATTR((fp_tiles_kernel<8, 2, true, FM>), d->smem_optin);
    UDEV_TILE_ATTR((fp_tiles_kernel<1, 4, true, FM>), d->smem_optin);
    UDEV_TILE_ATTR((fp_tiles_kernel<1, 2, true, FM>), d->smem_optin);
    /* the batch kernels also hold their record in static shared memory */
    const int batch_dyn = d->smem_optin - (int) kBatchStatic;
    UDEV_TILE_ATTR((fp_tiles_batch_kernel<1, 8, false, FM>), batch_dyn);
    UDEV_TILE_ATTR((fp_tiles_batch_kernel<2, 8, false, FM>), batch_dyn);
    UDEV_TILE_ATTR((fp_tiles_batch_kernel<4, 4, false, FM>), batch_dyn);
    UDEV_TILE_ATTR((fp_tiles_batch_kernel<8, 2, false, FM>), batch_dyn);
    UDEV_TILE_ATTR((fp_tiles_batch_kernel<1, 8, true, FM>), batch_dyn);
    UDEV_TILE_ATTR((fp_tiles_batch_kernel<2, 8, true, FM>), batch_dyn);
    UDEV_TILE_ATTR((fp_tiles_batch_kernel<4, 4, true, FM>), batch_dyn);
    UDEV_TILE_ATTR((fp_tiles_batch_kernel<8, 2, true, FM>), batch_dyn);
    UDEV_TILE_ATTR((fp_tiles_batch_kernel<1, 4, true, FM>), batch_dyn);
    UDEV_TILE_ATTR((fp_tiles_batch_kernel<1, 2, true, FM>), batch_dyn);
#undef UDEV_TILE_ATTR
    return UFOIR_OK;
}

int udev_kernels_init(udev *d)
{
    int rc = kernels_init_fm<false>(d);
    rc = rc ? rc : kernels_init_fm<true>(d);
    return rc ? rc : udev_sart_init(d);
}

extern "C" int udev_pad_transpose(udev *d, const float *vol, float *volP, float *volTP, int n, int n_slices)
{
    if (n_slices <= 0)
        return UFOIR_OK;
    UDEV_BIND(d);
    const int pitch = udev_fp_pitch(n);
    for (int done = 0; done < n_slices;) {
        const int chunk = n_slices - done > 65535 ? 65535 : n_slices - done;
        dim3 grid(udev_div_up(n, 32), udev_div_up(n, 32), (unsigned int) chunk);
        pad_transpose_kernel<<<grid, dim3(32, 8), 0, d->stream>>>(
            vol + (size_t) done * n * n, volP + (size_t) done * n * pitch, volTP + (size_t) done * n * pitch, n, pitch,
            (long long) n * n, (long long) n * pitch);
        int rc = udev_after_launch(d, "pad_transpose_kernel");
        if (rc)
            return rc;
        done += chunk;
    }
    return UFOIR_OK;
}

/* The template variants that exist: (J, A) with whole rows, and the
 * windowed ones of split tiles. */
static bool variant_exists(int J, int A, bool win)
{
    const int k = J * 16 + A;
    if (!win)
        return k == 1 * 16 + 8 || k == 2 * 16 + 8 || k == 4 * 16 + 4 || k == 8 * 16 + 2;
    return k == 1 * 16 + 2 || k == 1 * 16 + 4 || k == 1 * 16 + 8 || k == 2 * 16 + 8 || k == 4 * 16 + 4 ||
           k == 8 * 16 + 2;
}

extern "C" int udev_fp_cfg_finish(udev *d, const udev_geom *g, float tile_spread, udev_fp_cfg *c)
{
    const int n = g->n_dets, pitch = udev_fp_pitch(n);
    c->fm = g->fast_arith ? 1 : 0;
    if (!variant_exists(c->J, c->A, c->win != 0) || (c->K != 4 && c->K != 8 && c->K != 16 && c->K != 32) ||
        c->dsplit < 1 || c->dsplit > 64 || (c->win && c->dsplit < 2))
        return UFOIR_ERR_UNSUPPORTED;
    c->dper = (n + c->dsplit - 1) / c->dsplit;
    const int slots = (c->dper + 2 * c->J - 1) / (2 * c->J);
    c->threads = (slots + 15) / 16 * 32;
    if (c->threads > (c->win ? kMaxWinThreads : kMaxTileThreads))
        return UFOIR_ERR_UNSUPPORTED;
    c->margin = 4 + n / 512;
    c->wcols = c->wstride = pitch;
    if (c->win) {
        /* the columns a chunk's rays can reach: the detector range times
         * max |det_step| = sqrt 2, the chunk's rows times max |step| = 1,
         * the spread of the tile's angles, and a margin */
        const double need = (double) (c->dper - 1) * 1.41422 + (double) (c->K - 1) + (double) tile_spread +
                            2.0 * c->margin + 8.0;
        const int wc = ((int) ceil(need) + 3) / 4 * 4;
        if (wc >= pitch)
            return UFOIR_ERR_UNSUPPORTED;
        c->wcols = wc;
        c->wstride = wc + 4;
    }
    c->smem = kHeader + 2 * (size_t) c->K * c->wstride * 4;
    if (c->smem > (size_t) d->smem_optin)
        return UFOIR_ERR_UNSUPPORTED;
    return UFOIR_OK;
}

extern "C" int udev_fp_default_cfg(udev *d, const udev_geom *g, int n_tiles, int n_slices, float tile_spread,
                                   udev_fp_cfg *c)
{
    const int n = g->n_dets;
    const TileCfg cfg = tile_cfg(n, d->smem_optin);
    if (!tiles_supported(cfg, d->smem_optin)) {
        udev_set_error(d, "fp_tiles: n_dets %d needs %d threads / %zu B shared memory", n, cfg.threads, cfg.smem);
        return UFOIR_ERR_UNSUPPORTED;
    }
    const int pitch = udev_fp_pitch(n);
    c->fm = g->fast_arith ? 1 : 0;
    c->J = cfg.J;
    c->A = cfg.A;
    c->win = 0;
    c->K = cfg.K;
    c->dsplit = 1;
    c->dper = n;
    c->threads = cfg.threads;
    c->wcols = c->wstride = pitch;
    c->margin = 4 + n / 512;
    c->smem = cfg.smem;
    /* Too few tiles to fill the GPU (one slice, few angles): split each
     * angle tile's detectors over up to 8 CTAs, with chunks small enough
     * for two CTAs per SM. Every CTA walks all rows; it stages only the
     * window of columns its rays can reach (the detector range times
     * max |det_step| = sqrt 2, the chunk's rows times max |step| = 1, the
     * spread of the tile's angles, and a margin), unless that is the whole
     * row. */
    const long long ctas = (long long) n_tiles * n_slices;
    if (ctas < d->sm_count) {
        int split = (int) ((2LL * d->sm_count + ctas - 1) / ctas);
        split = split > 8 ? 8 : split;
        while (split > 1 && (n + split - 1) / split < 64)
            split--;
        int k2 = cfg.K;
        while (k2 > 4 && 2 * (kHeader + 2 * (size_t) k2 * pitch * 4) > (size_t) d->smem_optin)
            k2 /= 2;
        if (split > 1 && 2 * (kHeader + 2 * (size_t) k2 * pitch * 4) <= (size_t) d->smem_optin) {
            c->dsplit = split;
            c->dper = (n + split - 1) / split;
            const int slots = (c->dper + 2 * cfg.J - 1) / (2 * cfg.J);
            c->threads = (slots + 15) / 16 * 32;
            c->K = k2;
            c->smem = kHeader + 2 * (size_t) k2 * pitch * 4;
            /* Windowed CTAs take one detector pair per angle slot (J = 1)
             * where that fits: a split CTA holds few rays, and at J = 4
             * (n = 2900) it would run 3 warps of 16 rays per thread, too few
             * warps to hide the loads. The window: the largest chunk that
             * keeps two CTAs per SM. */
            const int slots1 = (c->dper + 1) / 2, threads1 = (slots1 + 15) / 16 * 32;
            for (int kw = 32; kw >= 4; kw /= 2) {
                udev_fp_cfg w = *c;
                w.win = 1;
                w.K = kw;
                w.J = threads1 <= kMaxWinThreads ? 1 : cfg.J;
                if (udev_fp_cfg_finish(d, g, tile_spread, &w) != UFOIR_OK) {
                    if (w.wcols >= pitch)
                        break;
                    continue;
                }
                if (2 * w.smem <= (size_t) d->smem_optin) {
                    *c = w;
                    break;
                }
            }
        }
    }
    return UFOIR_OK;
}

template <bool FM>
static int dispatch_tiles(udev *d, const FpTileArgs &A, const udev_fp_cfg *c, int n_tiles, int n_slices);

extern "C" int udev_fp_tiles_cfg(udev *d, const udev_geom *g, const udev_fp_cfg *c, const void *d_tiles,
                                 int n_tiles, const float *volP, const float *volTP, const float *src,
                                 const float *w, int w_shared, float *out, float scale, int n_slices)
{
    if (n_slices <= 0 || n_tiles <= 0)
        return UFOIR_OK;
    UDEV_BIND(d);
    const int n = g->n_dets;
    FpTileArgs A;
    A.volP = volP;
    A.volTP = volTP;
    A.src = src;
    A.w = w;
    A.out = out;
    A.sinv = g->d_sin;
    A.cosv = g->d_cos;
    A.tiles = static_cast<const int4 *>(d_tiles);
    A.n = n;
    A.pitch = udev_fp_pitch(n);
    A.rows_per_chunk = c->K;
    A.axis = g->axis;
    A.scale = scale;
    A.volp_stride = (long long) n * A.pitch;
    A.sino_stride = (long long) g->n_angles * n;
    A.w_stride = w_shared ? 0 : A.sino_stride;
    A.neg_zero = -0.0f;
    A.err = d->d_err;
    A.skip_chunk = d->inject_skip_chunk;   /* one-shot test injection */
    d->inject_skip_chunk = -1;
    A.dsplit = c->dsplit;
    A.dper = c->dper;
    A.wcols = c->wcols;
    A.wstride = c->wstride;
    A.margin = c->margin;
    return c->fm ? dispatch_tiles<true>(d, A, c, n_tiles, n_slices) : dispatch_tiles<false>(d, A, c, n_tiles, n_slices);
}

template <bool FM>
static int dispatch_tiles(udev *d, const FpTileArgs &A, const udev_fp_cfg *c, int n_tiles, int n_slices)
{
    if (c->win) {
        switch (c->J * 16 + c->A) {
        case 1 * 16 + 4: return launch_tiles<1, 4, true, FM>(d, A, n_tiles, n_slices, c->threads, c->smem);
        case 1 * 16 + 2: return launch_tiles<1, 2, true, FM>(d, A, n_tiles, n_slices, c->threads, c->smem);
        case 1 * 16 + 8: return launch_tiles<1, 8, true, FM>(d, A, n_tiles, n_slices, c->threads, c->smem);
        case 2 * 16 + 8: return launch_tiles<2, 8, true, FM>(d, A, n_tiles, n_slices, c->threads, c->smem);
        case 4 * 16 + 4: return launch_tiles<4, 4, true, FM>(d, A, n_tiles, n_slices, c->threads, c->smem);
        case 8 * 16 + 2: return launch_tiles<8, 2, true, FM>(d, A, n_tiles, n_slices, c->threads, c->smem);
        default: break;
        }
    } else {
        switch (c->J * 16 + c->A) {
        case 1 * 16 + 8: return launch_tiles<1, 8, false, FM>(d, A, n_tiles, n_slices, c->threads, c->smem);
        case 2 * 16 + 8: return launch_tiles<2, 8, false, FM>(d, A, n_tiles, n_slices, c->threads, c->smem);
        case 4 * 16 + 4: return launch_tiles<4, 4, false, FM>(d, A, n_tiles, n_slices, c->threads, c->smem);
        case 8 * 16 + 2: return launch_tiles<8, 2, false, FM>(d, A, n_tiles, n_slices, c->threads, c->smem);
        default: break;
        }
    }
    udev_set_error(d, "fp_tiles: no kernel for J=%d A=%d win=%d", c->J, c->A, c->win);
    return UFOIR_ERR_UNSUPPORTED;
}

extern "C" int udev_fp_tiles(udev *d, const udev_geom *g, const void *d_tiles, int n_tiles, float tile_spread,
                             const float *volP, const float *volTP, const float *src, const float *w, int w_shared,
                             float *out, float scale, int n_slices)
{
    if (n_slices <= 0 || n_tiles <= 0)
        return UFOIR_OK;
    udev_fp_cfg c;
    const int rc = udev_fp_default_cfg(d, g, n_tiles, n_slices, tile_spread, &c);
    if (rc)
        return rc;
    return udev_fp_tiles_cfg(d, g, &c, d_tiles, n_tiles, volP, volTP, src, w, w_shared, out, scale, n_slices);
}

/* ---- mixed batches ---- */

extern "C" size_t udev_fp_record_bytes(void)
{
    return sizeof(FpTileArgs);
}

extern "C" int udev_fp_batch_fits(const udev *d, const udev_fp_cfg *c)
{
    return c->smem + kBatchStatic <= (size_t) d->smem_optin;
}

extern "C" int udev_fp_record(udev *d, const udev_geom *g, const udev_fp_cfg *c, const void *d_tiles, int n_tiles,
                              const float *volP, const float *volTP, const float *src, const float *w,
                              float *out, float scale, void *record, int *items)
{
    if (n_tiles <= 0 || !variant_exists(c->J, c->A, c->win != 0) || !udev_fp_batch_fits(d, c))
        return UFOIR_ERR_UNSUPPORTED;
    FpTileArgs A;
    memset(&A, 0, sizeof(A));
    const int n = g->n_dets;
    A.volP = volP;
    A.volTP = volTP;
    A.src = src;
    A.w = w;
    A.out = out;
    A.sinv = g->d_sin;
    A.cosv = g->d_cos;
    A.tiles = static_cast<const int4 *>(d_tiles);
    A.n = n;
    A.pitch = udev_fp_pitch(n);
    A.rows_per_chunk = c->K;
    A.axis = g->axis;
    A.scale = scale;
    A.volp_stride = (long long) n * A.pitch;
    A.sino_stride = (long long) g->n_angles * n;
    A.w_stride = 0;
    A.neg_zero = -0.0f;
    A.err = d->d_err;
    A.skip_chunk = -1;
    A.dsplit = c->dsplit;
    A.dper = c->dper;
    A.wcols = c->wcols;
    A.wstride = c->wstride;
    A.margin = c->margin;
    memcpy(record, &A, sizeof(A));
    *items = n_tiles * c->dsplit;
    return UFOIR_OK;
}

template <int J, int A, bool WIN, bool FM>
static int launch_batch(udev *d, const udev_fp_cfg *c, const void *recs, const int *item_start, int n_jobs,
                        const int *job_index, const int *active, int n_items)
{
    fp_tiles_batch_kernel<J, A, WIN, FM><<<(unsigned int) n_items, c->threads, c->smem, d->stream>>>(
        static_cast<const FpTileArgs *>(recs), item_start, n_jobs, job_index, active);
    return udev_after_launch(d, "fp_tiles_batch_kernel");
}

template <bool FM>
static int dispatch_batch(udev *d, const udev_fp_cfg *c, const void *r, const int *st, int nj, const int *ji,
                          const int *ac, int ni)
{
    if (c->win) {
        switch (c->J * 16 + c->A) {
        case 1 * 16 + 4: return launch_batch<1, 4, true, FM>(d, c, r, st, nj, ji, ac, ni);
        case 1 * 16 + 2: return launch_batch<1, 2, true, FM>(d, c, r, st, nj, ji, ac, ni);
        case 1 * 16 + 8: return launch_batch<1, 8, true, FM>(d, c, r, st, nj, ji, ac, ni);
        case 2 * 16 + 8: return launch_batch<2, 8, true, FM>(d, c, r, st, nj, ji, ac, ni);
        case 4 * 16 + 4: return launch_batch<4, 4, true, FM>(d, c, r, st, nj, ji, ac, ni);
        case 8 * 16 + 2: return launch_batch<8, 2, true, FM>(d, c, r, st, nj, ji, ac, ni);
        default: break;
        }
    } else {
        switch (c->J * 16 + c->A) {
        case 1 * 16 + 8: return launch_batch<1, 8, false, FM>(d, c, r, st, nj, ji, ac, ni);
        case 2 * 16 + 8: return launch_batch<2, 8, false, FM>(d, c, r, st, nj, ji, ac, ni);
        case 4 * 16 + 4: return launch_batch<4, 4, false, FM>(d, c, r, st, nj, ji, ac, ni);
        case 8 * 16 + 2: return launch_batch<8, 2, false, FM>(d, c, r, st, nj, ji, ac, ni);
        default: break;
        }
    }
    udev_set_error(d, "fp_tiles batch: no kernel for J=%d A=%d win=%d", c->J, c->A, c->win);
    return UFOIR_ERR_UNSUPPORTED;
}

extern "C" int udev_fp_batch(udev *d, const udev_fp_cfg *c, const void *d_records, const int *d_item_start,
                             int n_jobs, const int *d_job_index, const int *d_active, int n_items)
{
    if (n_jobs <= 0 || n_items <= 0)
        return UFOIR_OK;
    if (!udev_fp_batch_fits(d, c)) {
        udev_set_error(d, "fp_tiles batch: %zu B of shared memory do not fit", c->smem);
        return UFOIR_ERR_UNSUPPORTED;
    }
    UDEV_BIND(d);
    return c->fm ? dispatch_batch<true>(d, c, d_records, d_item_start, n_jobs, d_job_index, d_active, n_items)
                 : dispatch_batch<false>(d, c, d_records, d_item_start, n_jobs, d_job_index, d_active, n_items);
}

/* Padded copies of the volumes of a mixed batch: one launch, 32 x 32 tiles. */
struct PadRec {
    const float *vol;
    float *P, *TP;
    int n, pitch, tiles_x, pad_;
};

__global__ void __launch_bounds__(256) pad_batch_kernel(const PadRec *__restrict__ recs,
                                                        const int *__restrict__ item_start, int n_jobs,
                                                        const int *__restrict__ job_index,
                                                        const int *__restrict__ active)
{
    __shared__ float tile[32][33];
    __shared__ int job_s;
    const int b = (int) blockIdx.x;
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        int lo = 0, hi = n_jobs - 1;
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
    const PadRec r = recs[j];
    const int local = b - __ldg(item_start + j);
    const int bx = (local % r.tiles_x) * 32, by = (local / r.tiles_x) * 32;
    for (int k = threadIdx.y; k < 32; k += 8) {
        const int x = bx + threadIdx.x, y = by + k;
        if (x < r.n && y < r.n) {
            const float v = r.vol[(size_t) y * r.n + x];
            tile[k][threadIdx.x] = v;
            r.P[(size_t) y * r.pitch + kPadL + x] = v;
        }
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += 8) {
        const int x = by + threadIdx.x, y = bx + k;
        if (x < r.n && y < r.n)
            r.TP[(size_t) y * r.pitch + kPadL + x] = tile[threadIdx.x][k];
    }
}

extern "C" size_t udev_pad_record_bytes(void)
{
    return sizeof(PadRec);
}

extern "C" int udev_pad_record(int n, const float *vol, float *volP, float *volTP, void *record, int *items)
{
    PadRec r;
    memset(&r, 0, sizeof(r));
    r.vol = vol;
    r.P = volP;
    r.TP = volTP;
    r.n = n;
    r.pitch = udev_fp_pitch(n);
    r.tiles_x = (n + 31) / 32;
    memcpy(record, &r, sizeof(r));
    *items = r.tiles_x * r.tiles_x;
    return UFOIR_OK;
}

extern "C" int udev_pad_batch(udev *d, const void *d_records, const int *d_item_start, int n_jobs,
                              const int *d_job_index, const int *d_active, int n_items)
{
    if (n_jobs <= 0 || n_items <= 0)
        return UFOIR_OK;
    UDEV_BIND(d);
    pad_batch_kernel<<<(unsigned int) n_items, dim3(32, 8), 0, d->stream>>>(
        static_cast<const PadRec *>(d_records), d_item_start, n_jobs, d_job_index, d_active);
    return udev_after_launch(d, "pad_batch_kernel");
}
