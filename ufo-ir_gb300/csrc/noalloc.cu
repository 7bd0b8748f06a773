/*
 * noalloc.cu - an L1-norm entry point that allocates no device memory.
 *
 * Some callers must not allocate device memory where they need this
 * reduction:
 *   - code whose device memory is owned by someone else, e.g. a host
 *     framework with its own pooling allocator, or a process under a hard
 *     device-memory limit (an MPS client with a set limit), where a library
 *     must not grow its own footprint behind the owner's back;
 *   - latency-critical loops that must not take the allocator's locks or
 *     risk the implicit synchronisation that cudaMalloc/cudaFree can cause.
 * ufoir_l1_norm_fp64_noalloc computes what ufoir_l1_norm computes in FP64
 * mode (the same kernel shape: 512 fixed chunks per slice, 256 threads, the
 * same fixed summation tree), but keeps its per-chunk partial sums in the
 * file-scope device array below instead of allocated scratch. The caller
 * passes the input and the output (both device memory) and a stream.
 */
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "udev_internal.cuh"

namespace {

constexpr int kNaBlocks = 512;     /* partial sums per slice */
constexpr int kNaThreads = 256;
constexpr int kNaCacheSlots = 64;  /* contexts remembered at once */

/* 64 slices x 512 partials x 8 bytes = 256 KiB, held by every GPU that loads
 * the library until the process exits. */
static __device__ __align__(256) double g_noalloc_partials[UFOIR_NOALLOC_MAX_SLICES * kNaBlocks];

/* The array's device address belongs to a CUDA context (the module is loaded
 * per context), so it is cached per context id: after cudaDeviceReset, or
 * with another driver context current, the id differs and the address is
 * looked up again. Ids are unique for the life of the process. */
struct AddrSlot {
    unsigned long long ctx_id;
    double *addr;
};
std::mutex g_noalloc_mutex;
AddrSlot g_noalloc_cache[kNaCacheSlots];
int g_noalloc_next;

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);
CtxGetCurrentFn g_ctx_get_current;
CtxGetIdFn g_ctx_get_id;

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

/* Id of the context current on this thread. When none is current yet, the
 * runtime is made to bind the current device's primary context first (a
 * cudaMemGetInfo call, which allocates nothing). */
int current_context_id(unsigned long long *id)
{
    if (!g_ctx_get_current || !g_ctx_get_id) {
        void *f1 = nullptr, *f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) !=
                cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2) {
            cudaGetLastError();
            return UFOIR_ERR_CUDA;
        }
        g_ctx_get_current = (CtxGetCurrentFn) f1;
        g_ctx_get_id = (CtxGetIdFn) f2;
    }
    CUcontext c = nullptr;
    if (g_ctx_get_current(&c) != CUDA_SUCCESS || !c) {
        /* no context current yet: make the runtime bind the current device's
         * primary context, then ask again */
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaSetDevice(dev) != cudaSuccess) {
            cudaGetLastError();
            return UFOIR_ERR_CUDA;
        }
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {   /* forces context creation */
            cudaGetLastError();
            return UFOIR_ERR_CUDA;
        }
        if (g_ctx_get_current(&c) != CUDA_SUCCESS || !c)
            return UFOIR_ERR_CUDA;
    }
    return g_ctx_get_id(c, id) == CUDA_SUCCESS ? UFOIR_OK : UFOIR_ERR_CUDA;
}

/* Device address of the scratch array in the current context: looked up with
 * cudaGetSymbolAddress the first time a context is seen (so once per device
 * in the usual one-context-per-device program), then served from the cache. */
int scratch_for_current_context(double **out)
{
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    unsigned long long id = 0;
    int rc = current_context_id(&id);
    if (rc)
        return rc;
    for (int i = 0; i < kNaCacheSlots; i++)
        if (g_noalloc_cache[i].addr && g_noalloc_cache[i].ctx_id == id) {
            *out = g_noalloc_cache[i].addr;
            return UFOIR_OK;
        }
    double *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress((void **) &p, g_noalloc_partials);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return UFOIR_ERR_CUDA;
    }
    AddrSlot &slot = g_noalloc_cache[g_noalloc_next];
    g_noalloc_next = (g_noalloc_next + 1) % kNaCacheSlots;
    slot.ctx_id = id;
    slot.addr = p;
    *out = p;
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
    int rc = scratch_for_current_context(&scratch);
    if (rc)
        return rc;
    cudaStream_t s = (cudaStream_t) stream;
    /* cudaLaunchKernel returns this launch's own status, so an error the
     * caller left pending is neither reported as ours nor consumed, unless
     * one of these launches fails (then the pending state is cleared). */
    int blocks = kNaBlocks;
    void *a1[] = {(void *) &d_v, (void *) &count, (void *) &scratch};
    cudaError_t e = cudaLaunchKernel((const void *) na_l1_partial_kernel, dim3(kNaBlocks, n_slices),
                                     dim3(kNaThreads), a1, 0, s);
    if (e == cudaSuccess) {
        const double *cs = scratch;
        void *a2[] = {(void *) &cs, (void *) &blocks, (void *) &d_out};
        e = cudaLaunchKernel((const void *) na_sum_kernel, dim3(n_slices), dim3(kNaThreads), a2, 0, s);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return UFOIR_ERR_CUDA;
    }
    return UFOIR_OK;
}
