/*
 * noalloc.cu - an L1-norm entry point that allocates no device memory.
 *
 * Some callers cannot call cudaMalloc where they need this reduction:
 *   - code that runs while its own stream is being captured into a CUDA
 *     graph (device allocation is not a capturable operation);
 *   - code whose device memory is owned by someone else, e.g. a host
 *     framework with its own pooling allocator or an MPS client with a hard
 *     memory limit, where a library must not grow its own footprint;
 *   - latency-critical loops that must not take the allocator's locks.
 * ufoir_l1_norm_fp64_noalloc computes what ufoir_l1_norm computes in FP64
 * mode (same kernels shape: 512 fixed chunks per slice, 256 threads, the
 * same fixed summation tree), but keeps its per-chunk partial sums in the
 * file-scope device array below instead of allocated scratch. The caller
 * passes the input and the output (both device memory) and a stream.
 */
#include <cuda_runtime.h>

#include <mutex>

#include "udev_internal.cuh"

namespace {

constexpr int kNaBlocks = 512;     /* partial sums per slice */
constexpr int kNaThreads = 256;
constexpr int kNaMaxDevices = 64;

/* 64 slices x 512 partials x 8 bytes = 256 KiB, held by every GPU that loads
 * the library until the process exits. */
static __device__ __align__(256) double g_noalloc_partials[UFOIR_NOALLOC_MAX_SLICES * kNaBlocks];

std::mutex g_noalloc_mutex;
double *g_noalloc_addr[kNaMaxDevices];

__device__ __forceinline__ double na_block_sum(double v)
{
    __shared__ double warp_sums[kNaThreads / 32];
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        warp_sums[wid] = v;
    __syncthreads();
    double r = 0.0;
    if (wid == 0) {
        r = lane < kNaThreads / 32 ? warp_sums[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1)
            r += __shfl_down_sync(0xffffffffu, r, o);
    }
    return r;
}

/* Pass 1: block b of slice s sums |v| over its fixed contiguous chunk. */
__global__ void __launch_bounds__(kNaThreads) na_l1_partial_kernel(const float *v, size_t count, double *partials)
{
    const float *p = v + (size_t) blockIdx.y * count;
    const size_t chunk = (count + gridDim.x - 1) / gridDim.x;
    const size_t lo = (size_t) blockIdx.x * chunk;
    const size_t hi = lo + chunk < count ? lo + chunk : count;
    double acc = 0.0;
    for (size_t i = lo + threadIdx.x; i < hi; i += kNaThreads)
        acc += (double) fabsf(p[i]);
    acc = na_block_sum(acc);
    if (threadIdx.x == 0)
        partials[(size_t) blockIdx.y * gridDim.x + blockIdx.x] = acc;
}

/* Pass 2: one block per slice sums its partials in a fixed tree. */
__global__ void __launch_bounds__(kNaThreads) na_sum_kernel(const double *partials, int per_slice, float *out)
{
    const double *p = partials + (size_t) blockIdx.x * per_slice;
    double acc = 0.0;
    for (int i = threadIdx.x; i < per_slice; i += kNaThreads)
        acc += p[i];
    acc = na_block_sum(acc);
    if (threadIdx.x == 0)
        out[blockIdx.x] = (float) acc;
}

/* Device address of the scratch array for the current device, looked up
 * once per device (cudaGetSymbolAddress with that device current). */
int scratch_for_current_device(double **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return UFOIR_ERR_CUDA;
    }
    if (dev < 0 || dev >= kNaMaxDevices)
        return UFOIR_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        double *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress((void **) &p, g_noalloc_partials);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return UFOIR_ERR_CUDA;
        }
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return UFOIR_OK;
}

}  // namespace

extern "C" int ufoir_l1_norm_fp64_noalloc(const float *d_v, size_t count, unsigned int n_slices, float *d_out,
                                          void *stream)
{
    if (!d_v || !d_out || count == 0 || n_slices == 0)
        return UFOIR_ERR_INVALID;
    if (n_slices > UFOIR_NOALLOC_MAX_SLICES)
        return UFOIR_ERR_INVALID;   /* beyond the fixed scratch: rejected, nothing launched */
    double *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc)
        return rc;
    cudaStream_t s = (cudaStream_t) stream;
    na_l1_partial_kernel<<<dim3(kNaBlocks, n_slices), kNaThreads, 0, s>>>(d_v, count, scratch);
    na_sum_kernel<<<n_slices, kNaThreads, 0, s>>>(scratch, kNaBlocks, d_out);
    if (cudaGetLastError() != cudaSuccess)
        return UFOIR_ERR_CUDA;
    return UFOIR_OK;
}
