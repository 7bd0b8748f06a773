/*
 * udev_runtime.cu - context, memory, copies and CUDA-graph capture for the
 * C host library (declared in udev.h).
 */
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>

#include "udev_internal.cuh"

extern "C" {

void udev_set_error(udev *d, const char *fmt, ...)
{
    if (!d)
        return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(d->err, sizeof(d->err), fmt, ap);
    va_end(ap);
}

const char *udev_error(const udev *d)
{
    return d ? d->err : "no context";
}

int udev_create(int device, udev **out, char *err, size_t errlen)
{
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        snprintf(err, errlen, "no CUDA device available (%s)",
                 e != cudaSuccess ? cudaGetErrorString(e) : "0 devices");
        cudaGetLastError();
        return UFOIR_ERR_CUDA;
    }
    if (device < 0 || device >= count) {
        snprintf(err, errlen, "device %d out of range [0, %d)", device, count);
        return UFOIR_ERR_INVALID;
    }
    e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        snprintf(err, errlen, "cudaSetDevice(%d): %s", device, cudaGetErrorString(e));
        return UFOIR_ERR_CUDA;
    }
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, device);
    if (e != cudaSuccess) {
        snprintf(err, errlen, "cudaGetDeviceProperties: %s", cudaGetErrorString(e));
        return UFOIR_ERR_CUDA;
    }
    if (prop.major < 10) {
        snprintf(err, errlen, "device %d is sm_%d%d; this library is built for sm_103a only",
                 device, prop.major, prop.minor);
        return UFOIR_ERR_UNSUPPORTED;
    }
    udev *d = new (std::nothrow) udev();
    if (!d) {
        snprintf(err, errlen, "out of host memory");
        return UFOIR_ERR_NOMEM;
    }
    d->device = device;
    d->sm_count = prop.multiProcessorCount;
    d->smem_optin = (int) prop.sharedMemPerBlockOptin;
    e = cudaStreamCreateWithFlags(&d->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        snprintf(err, errlen, "cudaStreamCreate: %s", cudaGetErrorString(e));
        delete d;
        return UFOIR_ERR_CUDA;
    }
    d->stream = d->own_stream;
    /* Keep freed stream-ordered memory in the pool instead of returning it to
     * the driver after every synchronisation. */
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t threshold = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
    }
    cudaGetLastError();
    if (cudaMalloc(&d->d_err, sizeof(int)) != cudaSuccess || cudaMemset(d->d_err, 0, sizeof(int)) != cudaSuccess ||
        cudaMallocHost(&d->h_err, sizeof(int)) != cudaSuccess || udev_kernels_init(d) != UFOIR_OK) {
        snprintf(err, errlen, "context setup failed: %s", d->err[0] ? d->err : cudaGetErrorString(cudaGetLastError()));
        udev_destroy(d);
        return UFOIR_ERR_CUDA;
    }
    *out = d;
    return UFOIR_OK;
}

void udev_destroy(udev *d)
{
    if (!d)
        return;
    cudaSetDevice(d->device);
    cudaStreamSynchronize(d->stream);
    if (d->red_partials)
        cudaFree(d->red_partials);
    if (d->red_out)
        cudaFree(d->red_out);
    if (d->h_red)
        cudaFreeHost(d->h_red);
    if (d->ev_start)
        cudaEventDestroy(d->ev_start);
    if (d->ev_stop)
        cudaEventDestroy(d->ev_stop);
    if (d->d_err)
        cudaFree(d->d_err);
    if (d->h_err)
        cudaFreeHost(d->h_err);
    if (d->side) {
        cudaStreamSynchronize(d->side);
        cudaStreamDestroy(d->side);
    }
    if (d->side_go)
        cudaEventDestroy(d->side_go);
    if (d->side_done)
        cudaEventDestroy(d->side_done);
    for (int i = 0; i < UDEV_SIDE_SLOTS; ++i)
        if (d->side_mark[i])
            cudaEventDestroy(d->side_mark[i]);
    if (d->own_stream)
        cudaStreamDestroy(d->own_stream);
    delete d;
}

int udev_stream_create(udev *d, void **s)
{
    UDEV_BIND(d);
    cudaStream_t st = nullptr;
    UDEV_CHECK(d, cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    *s = (void *) st;
    return UFOIR_OK;
}

void udev_stream_destroy(udev *d, void *s)
{
    if (!s)
        return;
    cudaSetDevice(d->device);
    cudaStreamDestroy((cudaStream_t) s);
}

void udev_use_stream(udev *d, void *s)
{
    d->stream = s ? (cudaStream_t) s : d->own_stream;
}

int udev_event_create(udev *d, void **e)
{
    UDEV_BIND(d);
    cudaEvent_t ev = nullptr;
    UDEV_CHECK(d, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    *e = (void *) ev;
    return UFOIR_OK;
}

void udev_event_destroy(void *e)
{
    if (e)
        cudaEventDestroy((cudaEvent_t) e);
}

int udev_event_record(udev *d, void *e)
{
    UDEV_BIND(d);
    UDEV_CHECK(d, cudaEventRecord((cudaEvent_t) e, d->stream));
    return UFOIR_OK;
}

int udev_event_done(udev *d, void *e)
{
    const cudaError_t r = cudaEventQuery((cudaEvent_t) e);
    if (r == cudaSuccess)
        return 1;
    if (r == cudaErrorNotReady)
        return 0;
    cudaGetLastError();
    udev_set_error(d, "event query: %s", cudaGetErrorString(r));
    return UFOIR_ERR_CUDA;
}

int udev_device(const udev *d)
{
    return d->device;
}

int udev_sm_count(const udev *d)
{
    return d->sm_count;
}

void *udev_stream(udev *d)
{
    return (void *) d->stream;
}

uint64_t udev_launches(const udev *d)
{
    return d->launches;
}

int udev_sync(udev *d)
{
    UDEV_BIND(d);
    UDEV_CHECK(d, cudaStreamSynchronize(d->stream));
    return UFOIR_OK;
}

int udev_mem_info(udev *d, size_t *free_bytes, size_t *total_bytes)
{
    UDEV_BIND(d);
    UDEV_CHECK(d, cudaMemGetInfo(free_bytes, total_bytes));
    return UFOIR_OK;
}

int udev_malloc(udev *d, void **p, size_t bytes)
{
    UDEV_BIND(d);
    *p = nullptr;
    if (bytes == 0)
        bytes = 16;
    cudaError_t e = cudaMallocAsync(p, bytes, d->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        udev_set_error(d, "device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? UFOIR_ERR_NOMEM : UFOIR_ERR_CUDA;
    }
    return UFOIR_OK;
}

int udev_free(udev *d, void *p)
{
    if (!p)
        return UFOIR_OK;
    UDEV_BIND(d);
    UDEV_CHECK(d, cudaFreeAsync(p, d->stream));
    return UFOIR_OK;
}

int udev_host_malloc(udev *d, void **p, size_t bytes)
{
    UDEV_BIND(d);
    *p = nullptr;
    cudaError_t e = cudaMallocHost(p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        udev_set_error(d, "pinned host allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        return UFOIR_ERR_NOMEM;
    }
    return UFOIR_OK;
}

int udev_host_free(udev *d, void *p)
{
    if (!p)
        return UFOIR_OK;
    UDEV_BIND(d);
    UDEV_CHECK(d, cudaFreeHost(p));
    return UFOIR_OK;
}

int udev_is_device_ptr(udev *d, const void *p)
{
    cudaPointerAttributes attr;
    cudaError_t e = cudaPointerGetAttributes(&attr, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged)
        return attr.device == d->device ? 1 : 0;
    return 0;
}

int udev_memcpy_async(udev *d, void *dst, const void *src, size_t bytes)
{
    if (bytes == 0)
        return UFOIR_OK;
    UDEV_BIND(d);
    UDEV_CHECK(d, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, d->stream));
    return UFOIR_OK;
}

static int side_ensure(udev *d)
{
    if (d->side)
        return UFOIR_OK;
    UDEV_CHECK(d, cudaStreamCreateWithFlags(&d->side, cudaStreamNonBlocking));
    UDEV_CHECK(d, cudaEventCreateWithFlags(&d->side_go, cudaEventDisableTiming));
    UDEV_CHECK(d, cudaEventCreateWithFlags(&d->side_done, cudaEventDisableTiming));
    for (int i = 0; i < UDEV_SIDE_SLOTS; ++i)
        UDEV_CHECK(d, cudaEventCreateWithFlags(&d->side_mark[i], cudaEventDisableTiming));
    return UFOIR_OK;
}

int udev_side_fence(udev *d)
{
    UDEV_BIND(d);
    int rc = side_ensure(d);
    if (rc)
        return rc;
    UDEV_CHECK(d, cudaEventRecord(d->side_go, d->stream));
    UDEV_CHECK(d, cudaStreamWaitEvent(d->side, d->side_go, 0));
    return UFOIR_OK;
}

int udev_side_copy(udev *d, void *dst, const void *src, size_t bytes, int slot)
{
    if (slot < 0 || slot >= UDEV_SIDE_SLOTS) {
        udev_set_error(d, "side copy: slot %d out of range", slot);
        return UFOIR_ERR_INVALID;
    }
    UDEV_BIND(d);
    int rc = side_ensure(d);
    if (rc)
        return rc;
    if (bytes)
        UDEV_CHECK(d, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, d->side));
    UDEV_CHECK(d, cudaEventRecord(d->side_mark[slot], d->side));
    return UFOIR_OK;
}

int udev_side_wait(udev *d, int slot)
{
    if (slot < 0 || slot >= UDEV_SIDE_SLOTS || !d->side) {
        udev_set_error(d, "side wait: slot %d out of range or no side stream", slot);
        return UFOIR_ERR_INVALID;
    }
    UDEV_BIND(d);
    UDEV_CHECK(d, cudaStreamWaitEvent(d->stream, d->side_mark[slot], 0));
    return UFOIR_OK;
}

int udev_copy_after(udev *d, void *dst, const void *src, size_t bytes)
{
    if (bytes == 0)
        return UFOIR_OK;
    int rc = udev_side_fence(d);
    if (rc)
        return rc;
    UDEV_CHECK(d, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, d->side));
    return UFOIR_OK;
}

int udev_copy_join(udev *d)
{
    if (!d->side)
        return UFOIR_OK;
    UDEV_BIND(d);
    UDEV_CHECK(d, cudaEventRecord(d->side_done, d->side));
    UDEV_CHECK(d, cudaStreamWaitEvent(d->stream, d->side_done, 0));
    return UFOIR_OK;
}

int udev_memcpy(udev *d, void *dst, const void *src, size_t bytes)
{
    int rc = udev_memcpy_async(d, dst, src, bytes);
    if (rc)
        return rc;
    return udev_sync(d);
}

int udev_memset(udev *d, void *p, int value, size_t bytes)
{
    if (bytes == 0)
        return UFOIR_OK;
    UDEV_BIND(d);
    UDEV_CHECK(d, cudaMemsetAsync(p, value, bytes, d->stream));
    return UFOIR_OK;
}

int udev_take_kernel_error(udev *d)
{
    UDEV_BIND(d);
    UDEV_CHECK(d, cudaMemcpyAsync(d->h_err, d->d_err, sizeof(int), cudaMemcpyDeviceToHost, d->stream));
    UDEV_CHECK(d, cudaStreamSynchronize(d->stream));
    const int code = *d->h_err;
    if (code == 0)
        return UFOIR_OK;
    UDEV_CHECK(d, cudaMemsetAsync(d->d_err, 0, sizeof(int), d->stream));
    UDEV_CHECK(d, cudaStreamSynchronize(d->stream));
    if (code & 3) {
        udev_set_error(d, "a kernel gave up waiting for a shared-memory copy (code %d); results of that call are invalid",
                       code);
        return UFOIR_ERR_TIMEOUT;
    }
    udev_set_error(d, "a kernel found its staging buffer too small (code %d); results of that call are invalid", code);
    return UFOIR_ERR_CUDA;
}

void udev_inject_copy_skip(udev *d, int chunk)
{
    d->inject_skip_chunk = chunk < 0 ? -1 : chunk;
}

int udev_timer_begin(udev *d)
{
    UDEV_BIND(d);
    if (!d->ev_start) {
        UDEV_CHECK(d, cudaEventCreate(&d->ev_start));
        UDEV_CHECK(d, cudaEventCreate(&d->ev_stop));
    }
    UDEV_CHECK(d, cudaEventRecord(d->ev_start, d->stream));
    return UFOIR_OK;
}

int udev_timer_end(udev *d, float *ms)
{
    UDEV_BIND(d);
    UDEV_CHECK(d, cudaEventRecord(d->ev_stop, d->stream));
    UDEV_CHECK(d, cudaEventSynchronize(d->ev_stop));
    UDEV_CHECK(d, cudaEventElapsedTime(ms, d->ev_start, d->ev_stop));
    return UFOIR_OK;
}

int udev_capture_begin(udev *d)
{
    UDEV_BIND(d);
    UDEV_CHECK(d, cudaStreamBeginCapture(d->stream, cudaStreamCaptureModeThreadLocal));
    d->capturing = 1;
    d->capture_launches = 0;
    return UFOIR_OK;
}

int udev_capture_end(udev *d, void **exec, uint64_t *kernels)
{
    UDEV_BIND(d);
    cudaGraph_t graph = nullptr;
    d->capturing = 0;
    *exec = nullptr;
    cudaError_t e = cudaStreamEndCapture(d->stream, &graph);
    if (e != cudaSuccess) {
        cudaGetLastError();
        udev_set_error(d, "graph capture failed: %s", cudaGetErrorString(e));
        return UFOIR_ERR_CUDA;
    }
    cudaGraphExec_t ge = nullptr;
    e = cudaGraphInstantiate(&ge, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        cudaGetLastError();
        udev_set_error(d, "graph instantiate failed: %s", cudaGetErrorString(e));
        return UFOIR_ERR_CUDA;
    }
    *exec = (void *) ge;
    if (kernels)
        *kernels = d->capture_launches;
    return UFOIR_OK;
}

int udev_graph_launch(udev *d, void *exec, uint64_t kernels)
{
    UDEV_BIND(d);
    UDEV_CHECK(d, cudaGraphLaunch((cudaGraphExec_t) exec, d->stream));
    d->launches += kernels;
    return UFOIR_OK;
}

void udev_graph_destroy(void *exec)
{
    if (exec)
        cudaGraphExecDestroy((cudaGraphExec_t) exec);
}

}  /* extern "C" */

int udev_after_launch(udev *d, const char *what)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        udev_set_error(d, "launch of %s failed: %s", what, cudaGetErrorString(e));
        return UFOIR_ERR_CUDA;
    }
    if (d->capturing)
        d->capture_launches++;
    else
        d->launches++;
    return UFOIR_OK;
}

int udev_reduction_scratch(udev *d, size_t partials, size_t outs)
{
    if (partials > d->red_partials_cap) {
        if (d->red_partials)
            cudaFree(d->red_partials);
        d->red_partials = nullptr;
        d->red_partials_cap = 0;
        UDEV_CHECK(d, cudaMalloc(&d->red_partials, partials * sizeof(double)));
        d->red_partials_cap = partials;
    }
    if (outs > d->red_out_cap) {
        if (d->red_out)
            cudaFree(d->red_out);
        if (d->h_red)
            cudaFreeHost(d->h_red);
        d->red_out = nullptr;
        d->h_red = nullptr;
        d->red_out_cap = 0;
        UDEV_CHECK(d, cudaMalloc(&d->red_out, 2 * outs * sizeof(float)));
        UDEV_CHECK(d, cudaMallocHost(&d->h_red, 2 * outs * sizeof(float)));
        d->red_out_cap = outs;
    }
    return UFOIR_OK;
}
