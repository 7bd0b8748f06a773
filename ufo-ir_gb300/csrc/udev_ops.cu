/*
 * udev_ops.cu - element-wise ops, TV subgradient, periodic differences and
 * the deterministic reductions used by the methods.
 *
 * Element-wise ops replace ufo-ir-basic-ops.cl:4-171,255-273 and the host
 * loops of ufo-ir-basic-ops-processor.c:324-430,544-604; every operation
 * rounds as the reference's (IEEE float, no contraction).
 * l1_grad replaces ufo-math-tvstd-method.cl:5-57, Dx/Dxt/Dy/Dyt replace
 * ufo-ir-gradient-processor.cl:1-51.
 *
 * Reductions (replacing the reference's host loops, ufo-ir-basic-ops.c:259-277
 * and ufo-ir-basic-ops-processor.c:148-247):
 *   COMPAT mode reproduces the float sequential sums bit for bit;
 *   FP64 mode sums the same terms in double with a fixed-shape tree (the
 *   same result on every run), then rounds to float.
 */
#include <cuda_runtime.h>

#include "udev_internal.cuh"

namespace {

__global__ void fill_kernel(float *p, size_t n, float v)
{
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n;
         i += (size_t) gridDim.x * blockDim.x)
        p[i] = v;
}

template <int OP>
__device__ __forceinline__ float binop(float a, float b, float m)
{
    if (OP == UDEV_MUL)
        return __fmul_rn(a, b);
    if (OP == UDEV_ADD)
        return __fadd_rn(a, b);
    if (OP == UDEV_SUB)
        return __fsub_rn(a, b);
    if (OP == UDEV_SUB_SCALED)
        return __fsub_rn(a, __fmul_rn(m, b));
    if (OP == UDEV_ADD_SCALED)
        return __fadd_rn(a, __fmul_rn(m, b));
    if (OP == UDEV_MAX)
        return fmaxf(a, b);
    return __fdiv_rn(a, b);
}

template <int OP>
__global__ void binary_kernel(const float *a, const float *b, float m, float *out, size_t n)
{
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n;
         i += (size_t) gridDim.x * blockDim.x)
        out[i] = binop<OP>(a[i], b[i], m);
}

template <int OP>
__device__ __forceinline__ float unop(float a, float m, float m2)
{
    if (OP == UDEV_INV)
        return a != 0.0f ? __fdiv_rn(1.0f, a) : 0.0f;
    if (OP == UDEV_POSC)
        return a > 0.0f ? a : 0.0f;
    if (OP == UDEV_SQRT)
        return __fsqrt_rn(a);
    if (OP == UDEV_SCALE)
        return __fmul_rn(a, m);
    if (OP == UDEV_ADDC)
        return __fadd_rn(m, a);
    if (OP == UDEV_MAXC)
        return fmaxf(a, m);
    /* UDEV_NORMALIZE: delta * v - min * delta (ufo-ir-basic-ops-processor.c:365) */
    return __fsub_rn(__fmul_rn(m, a), __fmul_rn(m2, m));
}

template <int OP>
__global__ void unary_kernel(const float *a, float m, float m2, float *out, size_t n)
{
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n;
         i += (size_t) gridDim.x * blockDim.x)
        out[i] = unop<OP>(a[i], m, m2);
}

__device__ __forceinline__ float tex0(const float *img, int x, int y, int w, int h)
{
    return (x >= 0 && y >= 0 && x < w && y < h) ? img[(size_t) y * w + x] : 0.0f;
}

/* l1_grad: 7-point isotropic-TV subgradient with EPS 0.001 and zero border.
 * A block computes a 32 x 32 tile, 4 rows per thread, from the tile and its
 * one-pixel halo staged in shared memory (zeros outside the image). */
constexpr int kGradTile = 32;

__global__ void __launch_bounds__(256) l1_grad_kernel(const float *in, float *out, int w, int h, long long stride)
{
    __shared__ float t[kGradTile + 2][kGradTile + 3];
    const int x0 = (int) blockIdx.x * kGradTile, y0 = (int) blockIdx.y * kGradTile;
    const float *img = in + (size_t) blockIdx.z * stride;
    const int tid = (int) (threadIdx.y * 32 + threadIdx.x);
    for (int e = tid; e < (kGradTile + 2) * (kGradTile + 2); e += 256) {
        const int ty = e / (kGradTile + 2), tx = e % (kGradTile + 2);
        t[ty][tx] = tex0(img, x0 - 1 + tx, y0 - 1 + ty, w, h);
    }
    __syncthreads();
    const int lx = (int) threadIdx.x + 1, x = x0 + (int) threadIdx.x;
    if (x >= w)
        return;
    const float eps = 0.001f;
#pragma unroll
    for (int m = 0; m < kGradTile / 8; ++m) {
        const int ly = (int) threadIdx.y + 8 * m + 1, y = y0 + ly - 1;
        if (y >= h)
            break;
        const float f3 = t[ly][lx];
        const float f1 = t[ly - 1][lx];
        const float f0 = t[ly - 1][lx - 1];
        const float f2 = t[ly][lx - 1];
        const float f4 = t[ly][lx + 1];
        const float f6 = t[ly + 1][lx + 1];
        const float f5 = t[ly + 1][lx];
        const float d32 = __fsub_rn(f3, f2), d35 = __fsub_rn(f3, f5);
        const float d43 = __fsub_rn(f4, f3), d46 = __fsub_rn(f4, f6);
        const float d13 = __fsub_rn(f1, f3), d10 = __fsub_rn(f1, f0);
        const float t1 = __fdiv_rn(__fsub_rn(__fsub_rn(__fmul_rn(2.0f, f3), f2), f5),
                                   __fsqrt_rn(__fadd_rn(__fadd_rn(eps, __fmul_rn(d32, d32)), __fmul_rn(d35, d35))));
        const float t2 = __fdiv_rn(d43, __fsqrt_rn(__fadd_rn(__fadd_rn(eps, __fmul_rn(d43, d43)), __fmul_rn(d46, d46))));
        const float t3 = __fdiv_rn(d13, __fsqrt_rn(__fadd_rn(__fadd_rn(eps, __fmul_rn(d13, d13)), __fmul_rn(d10, d10))));
        out[(size_t) blockIdx.z * stride + (size_t) y * w + x] = __fsub_rn(__fsub_rn(t1, t2), t3);
    }
}

template <int WHICH>
__global__ void diff_kernel(const float *in, float *out, int w, int h, long long stride)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h)
        return;
    const size_t base = (size_t) blockIdx.z * stride;
    const long long idx = (long long) y * w + x;
    const long long last = (long long) w * h;
    long long j;
    if (WHICH == UDEV_DX)
        j = idx - 1 + (x == 0 ? w : 0);
    else if (WHICH == UDEV_DXT)
        j = idx + 1 - (x == w - 1 ? w : 0);
    else if (WHICH == UDEV_DY)
        j = idx - w + (y == 0 ? last : 0);
    else
        j = idx + w - (y == h - 1 ? last : 0);
    out[base + idx] = __fsub_rn(in[base + idx], in[base + j]);
}

/* ---------------- reductions ---------------- */

constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 512;   /* partial sums per slice in FP64 mode */

__device__ __forceinline__ double block_sum_double(double v)
{
    __shared__ double warp_sums[kRedThreads / 32];
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        warp_sums[wid] = v;
    __syncthreads();
    double r = 0.0;
    if (wid == 0) {
        r = lane < kRedThreads / 32 ? warp_sums[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1)
            r += __shfl_down_sync(0xffffffffu, r, o);
    }
    return r;   /* valid in thread 0 */
}

/* COMPAT l1: one thread per slice, float sequential in index order i*h + j
 * (i < w, j < h), i.e. memory order. */
__global__ void l1_compat_kernel(const float *v, size_t count, long long stride, float *out)
{
    if (threadIdx.x != 0)
        return;
    const float *p = v + (size_t) blockIdx.x * stride;
    float norm = 0.0f;
    for (size_t i = 0; i < count; i++)
        norm = __fadd_rn(norm, fabsf(p[i]));
    out[blockIdx.x] = norm;
}

/* FP64 l1, pass 1: block b of slice s sums a fixed contiguous chunk. */
__global__ void __launch_bounds__(kRedThreads) l1_fp64_partial_kernel(const float *v, size_t count,
                                                                      long long stride, double *partials)
{
    const float *p = v + (size_t) blockIdx.y * stride;
    const size_t chunk = (count + gridDim.x - 1) / gridDim.x;
    const size_t lo = (size_t) blockIdx.x * chunk;
    const size_t hi = lo + chunk < count ? lo + chunk : count;
    double acc = 0.0;
    for (size_t i = lo + threadIdx.x; i < hi; i += kRedThreads)
        acc += (double) fabsf(p[i]);
    acc = block_sum_double(acc);
    if (threadIdx.x == 0)
        partials[(size_t) blockIdx.y * gridDim.x + blockIdx.x] = acc;
}

/* FP64 pass 2: one block per slice sums its partials in a fixed tree. */
__global__ void __launch_bounds__(kRedThreads) sum_partials_kernel(const double *partials, int per_slice,
                                                                   float *out)
{
    const double *p = partials + (size_t) blockIdx.x * per_slice;
    double acc = 0.0;
    for (int i = threadIdx.x; i < per_slice; i += kRedThreads)
        acc += p[i];
    acc = block_sum_double(acc);
    if (threadIdx.x == 0)
        out[blockIdx.x] = (float) acc;
}

/* dot product of ufo_ir_basic_ops_processor_dot_product: for part p < h,
 * partial[p] = sum_{i < w} a[p*i] * b[p*i]; the result sums the partials
 * in order. COMPAT: float sequential; FP64: double. One thread per part. */
template <bool FP64>
__global__ void dot_parts_kernel(const float *a, const float *b, unsigned int w, unsigned int h,
                                 long long stride, double *parts)
{
    const unsigned int part = blockIdx.x * blockDim.x + threadIdx.x;
    if (part >= h)
        return;
    const float *pa = a + (size_t) blockIdx.y * stride;
    const float *pb = b + (size_t) blockIdx.y * stride;
    double out;
    if (FP64) {
        double acc = 0.0;
        for (unsigned int i = 0; i < w; i++) {
            const unsigned int index = part * i;
            acc += (double) pa[index] * (double) pb[index];
        }
        out = acc;
    } else {
        float acc = 0.0f;
        for (unsigned int i = 0; i < w; i++) {
            const unsigned int index = part * i;
            acc = __fadd_rn(acc, __fmul_rn(pa[index], pb[index]));
        }
        out = (double) acc;
    }
    parts[(size_t) blockIdx.y * h + part] = out;
}

__global__ void dot_compat_sum_kernel(const double *parts, unsigned int h, float *out)
{
    if (threadIdx.x != 0)
        return;
    const double *p = parts + (size_t) blockIdx.x * h;
    float norm = 0.0f;
    for (unsigned int i = 0; i < h; i++)
        norm = __fadd_rn(norm, (float) p[i]);
    out[blockIdx.x] = norm;
}

__global__ void __launch_bounds__(kRedThreads) minmax_kernel(const float *v, size_t count, long long stride,
                                                             float *out)
{
    __shared__ float smin[kRedThreads], smax[kRedThreads];
    const float *p = v + (size_t) blockIdx.x * stride;
    float lo = 3.402823466e38f, hi = -3.402823466e38f;
    for (size_t i = threadIdx.x; i < count; i += kRedThreads) {
        lo = fminf(lo, p[i]);
        hi = fmaxf(hi, p[i]);
    }
    smin[threadIdx.x] = lo;
    smax[threadIdx.x] = hi;
    __syncthreads();
    for (int s = kRedThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            smin[threadIdx.x] = fminf(smin[threadIdx.x], smin[threadIdx.x + s]);
            smax[threadIdx.x] = fmaxf(smax[threadIdx.x], smax[threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[2 * blockIdx.x] = smin[0];
        out[2 * blockIdx.x + 1] = smax[0];
    }
}

unsigned int grid_for(udev *d, size_t n)
{
    size_t blocks = (n + 255) / 256;
    const size_t cap = (size_t) d->sm_count * 8;
    if (blocks > cap)
        blocks = cap;
    return (unsigned int) (blocks ? blocks : 1);
}

}  // namespace

extern "C" int udev_fill(udev *d, float *p, size_t n, float v)
{
    if (n == 0)
        return UFOIR_OK;
    UDEV_BIND(d);
    fill_kernel<<<grid_for(d, n), 256, 0, d->stream>>>(p, n, v);
    return udev_after_launch(d, "fill_kernel");
}

extern "C" int udev_binary(udev *d, int op, const float *a, const float *b, float m, float *out, size_t n)
{
    if (n == 0)
        return UFOIR_OK;
    UDEV_BIND(d);
    const unsigned int g = grid_for(d, n);
    switch (op) {
    case UDEV_MUL: binary_kernel<UDEV_MUL><<<g, 256, 0, d->stream>>>(a, b, m, out, n); break;
    case UDEV_ADD: binary_kernel<UDEV_ADD><<<g, 256, 0, d->stream>>>(a, b, m, out, n); break;
    case UDEV_SUB: binary_kernel<UDEV_SUB><<<g, 256, 0, d->stream>>>(a, b, m, out, n); break;
    case UDEV_SUB_SCALED: binary_kernel<UDEV_SUB_SCALED><<<g, 256, 0, d->stream>>>(a, b, m, out, n); break;
    case UDEV_ADD_SCALED: binary_kernel<UDEV_ADD_SCALED><<<g, 256, 0, d->stream>>>(a, b, m, out, n); break;
    case UDEV_MAX: binary_kernel<UDEV_MAX><<<g, 256, 0, d->stream>>>(a, b, m, out, n); break;
    case UDEV_DIV: binary_kernel<UDEV_DIV><<<g, 256, 0, d->stream>>>(a, b, m, out, n); break;
    default:
        udev_set_error(d, "unknown binary op %d", op);
        return UFOIR_ERR_INVALID;
    }
    return udev_after_launch(d, "binary_kernel");
}

extern "C" int udev_unary(udev *d, int op, const float *a, float m, float m2, float *out, size_t n)
{
    if (n == 0)
        return UFOIR_OK;
    UDEV_BIND(d);
    const unsigned int g = grid_for(d, n);
    switch (op) {
    case UDEV_INV: unary_kernel<UDEV_INV><<<g, 256, 0, d->stream>>>(a, m, m2, out, n); break;
    case UDEV_POSC: unary_kernel<UDEV_POSC><<<g, 256, 0, d->stream>>>(a, m, m2, out, n); break;
    case UDEV_SQRT: unary_kernel<UDEV_SQRT><<<g, 256, 0, d->stream>>>(a, m, m2, out, n); break;
    case UDEV_SCALE: unary_kernel<UDEV_SCALE><<<g, 256, 0, d->stream>>>(a, m, m2, out, n); break;
    case UDEV_ADDC: unary_kernel<UDEV_ADDC><<<g, 256, 0, d->stream>>>(a, m, m2, out, n); break;
    case UDEV_MAXC: unary_kernel<UDEV_MAXC><<<g, 256, 0, d->stream>>>(a, m, m2, out, n); break;
    case UDEV_NORMALIZE: unary_kernel<UDEV_NORMALIZE><<<g, 256, 0, d->stream>>>(a, m, m2, out, n); break;
    default:
        udev_set_error(d, "unknown unary op %d", op);
        return UFOIR_ERR_INVALID;
    }
    return udev_after_launch(d, "unary_kernel");
}

extern "C" int udev_l1_grad(udev *d, const float *in, float *out, int w, int h, int n_slices)
{
    if (n_slices <= 0)
        return UFOIR_OK;
    UDEV_BIND(d);
    dim3 grid(udev_div_up(w, kGradTile), udev_div_up(h, kGradTile), (unsigned int) n_slices);
    l1_grad_kernel<<<grid, dim3(32, 8), 0, d->stream>>>(in, out, w, h, (long long) w * h);
    return udev_after_launch(d, "l1_grad_kernel");
}

extern "C" int udev_diff(udev *d, int which, const float *in, float *out, int w, int h, int n_slices)
{
    if (n_slices <= 0)
        return UFOIR_OK;
    UDEV_BIND(d);
    dim3 grid(udev_div_up(w, 32), udev_div_up(h, 8), (unsigned int) n_slices);
    const long long stride = (long long) w * h;
    switch (which) {
    case UDEV_DX: diff_kernel<UDEV_DX><<<grid, dim3(32, 8), 0, d->stream>>>(in, out, w, h, stride); break;
    case UDEV_DXT: diff_kernel<UDEV_DXT><<<grid, dim3(32, 8), 0, d->stream>>>(in, out, w, h, stride); break;
    case UDEV_DY: diff_kernel<UDEV_DY><<<grid, dim3(32, 8), 0, d->stream>>>(in, out, w, h, stride); break;
    case UDEV_DYT: diff_kernel<UDEV_DYT><<<grid, dim3(32, 8), 0, d->stream>>>(in, out, w, h, stride); break;
    default:
        udev_set_error(d, "unknown difference %d", which);
        return UFOIR_ERR_INVALID;
    }
    return udev_after_launch(d, "diff_kernel");
}

extern "C" int udev_l1_norm(udev *d, const float *v, size_t w, size_t h, int n_slices, int mode,
                            float *host_out)
{
    if (n_slices <= 0)
        return UFOIR_OK;
    UDEV_BIND(d);
    const size_t count = w * h;
    int rc = udev_reduction_scratch(d, (size_t) kRedBlocks * n_slices, (size_t) n_slices);
    if (rc)
        return rc;
    if (mode == UFOIR_NORM_COMPAT) {
        l1_compat_kernel<<<n_slices, 32, 0, d->stream>>>(v, count, (long long) count, d->red_out);
        if ((rc = udev_after_launch(d, "l1_compat_kernel")))
            return rc;
    } else {
        l1_fp64_partial_kernel<<<dim3(kRedBlocks, n_slices), kRedThreads, 0, d->stream>>>(
            v, count, (long long) count, d->red_partials);
        if ((rc = udev_after_launch(d, "l1_fp64_partial_kernel")))
            return rc;
        sum_partials_kernel<<<n_slices, kRedThreads, 0, d->stream>>>(d->red_partials, kRedBlocks, d->red_out);
        if ((rc = udev_after_launch(d, "sum_partials_kernel")))
            return rc;
    }
    UDEV_CHECK(d, cudaMemcpyAsync(d->h_red, d->red_out, sizeof(float) * n_slices, cudaMemcpyDeviceToHost, d->stream));
    UDEV_CHECK(d, cudaStreamSynchronize(d->stream));
    for (int i = 0; i < n_slices; i++)
        host_out[i] = d->h_red[i];
    return UFOIR_OK;
}

extern "C" size_t udev_l1_partials(int n_slices)
{
    return (size_t) kRedBlocks * (size_t) (n_slices > 0 ? n_slices : 0);
}

extern "C" int udev_l1_norm_to(udev *d, const float *v, size_t w, size_t h, int n_slices, int mode, double *partials,
                               float *d_out)
{
    if (n_slices <= 0)
        return UFOIR_OK;
    UDEV_BIND(d);
    const size_t count = w * h;
    int rc;
    if (mode == UFOIR_NORM_COMPAT) {
        l1_compat_kernel<<<n_slices, 32, 0, d->stream>>>(v, count, (long long) count, d_out);
        return udev_after_launch(d, "l1_compat_kernel");
    }
    l1_fp64_partial_kernel<<<dim3(kRedBlocks, n_slices), kRedThreads, 0, d->stream>>>(v, count, (long long) count,
                                                                                       partials);
    if ((rc = udev_after_launch(d, "l1_fp64_partial_kernel")))
        return rc;
    sum_partials_kernel<<<n_slices, kRedThreads, 0, d->stream>>>(partials, kRedBlocks, d_out);
    return udev_after_launch(d, "sum_partials_kernel");
}

extern "C" int udev_dot(udev *d, const float *a, const float *b, size_t w, size_t h, int n_slices,
                        int mode, float *host_out)
{
    if (n_slices <= 0)
        return UFOIR_OK;
    if (w * h > 0xffffffffull) {
        udev_set_error(d, "dot: %zu elements exceed the 32-bit index of the reference", w * h);
        return UFOIR_ERR_INVALID;
    }
    UDEV_BIND(d);
    int rc = udev_reduction_scratch(d, h * (size_t) n_slices, (size_t) n_slices);
    if (rc)
        return rc;
    const long long stride = (long long) (w * h);
    dim3 grid(udev_div_up(h, 128), (unsigned int) n_slices);
    if (mode == UFOIR_NORM_COMPAT) {
        dot_parts_kernel<false><<<grid, 128, 0, d->stream>>>(a, b, (unsigned int) w, (unsigned int) h, stride,
                                                             d->red_partials);
        if ((rc = udev_after_launch(d, "dot_parts_kernel")))
            return rc;
        dot_compat_sum_kernel<<<n_slices, 32, 0, d->stream>>>(d->red_partials, (unsigned int) h, d->red_out);
        if ((rc = udev_after_launch(d, "dot_compat_sum_kernel")))
            return rc;
    } else {
        dot_parts_kernel<true><<<grid, 128, 0, d->stream>>>(a, b, (unsigned int) w, (unsigned int) h, stride,
                                                            d->red_partials);
        if ((rc = udev_after_launch(d, "dot_parts_kernel")))
            return rc;
        sum_partials_kernel<<<n_slices, kRedThreads, 0, d->stream>>>(d->red_partials, (int) h, d->red_out);
        if ((rc = udev_after_launch(d, "sum_partials_kernel")))
            return rc;
    }
    UDEV_CHECK(d, cudaMemcpyAsync(d->h_red, d->red_out, sizeof(float) * n_slices, cudaMemcpyDeviceToHost, d->stream));
    UDEV_CHECK(d, cudaStreamSynchronize(d->stream));
    for (int i = 0; i < n_slices; i++)
        host_out[i] = d->h_red[i];
    return UFOIR_OK;
}

extern "C" int udev_minmax(udev *d, const float *v, size_t n, int n_slices, float *host_min, float *host_max)
{
    if (n_slices <= 0)
        return UFOIR_OK;
    UDEV_BIND(d);
    int rc = udev_reduction_scratch(d, 1, (size_t) n_slices);
    if (rc)
        return rc;
    minmax_kernel<<<n_slices, kRedThreads, 0, d->stream>>>(v, n, (long long) n, d->red_out);
    if ((rc = udev_after_launch(d, "minmax_kernel")))
        return rc;
    UDEV_CHECK(d, cudaMemcpyAsync(d->h_red, d->red_out, 2 * sizeof(float) * n_slices, cudaMemcpyDeviceToHost, d->stream));
    UDEV_CHECK(d, cudaStreamSynchronize(d->stream));
    for (int i = 0; i < n_slices; i++) {
        host_min[i] = d->h_red[2 * i];
        host_max[i] = d->h_red[2 * i + 1];
    }
    return UFOIR_OK;
}
