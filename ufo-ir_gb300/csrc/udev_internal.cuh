/*
 * udev_internal.cuh - private state of the CUDA layer and shared helpers.
 */
#ifndef UFOIR_UDEV_INTERNAL_CUH
#define UFOIR_UDEV_INTERNAL_CUH

#include <cuda_runtime.h>

#include "udev.h"

struct udev {
    int device = 0;
    int sm_count = 0;
    int smem_optin = 0;
    cudaStream_t stream = nullptr;      /* where work goes now */
    cudaStream_t own_stream = nullptr;  /* the context's own stream */
    char err[1024] = {0};
    uint64_t launches = 0;          /* kernels launched eagerly or through graphs */
    int capturing = 0;
    uint64_t capture_launches = 0;  /* kernels recorded into the graph being captured */
    /* reduction scratch (grown on demand, outside of graph capture) */
    double *red_partials = nullptr;
    size_t red_partials_cap = 0;
    float *red_out = nullptr;
    float *h_red = nullptr;
    size_t red_out_cap = 0;
    cudaEvent_t ev_start = nullptr;
    cudaEvent_t ev_stop = nullptr;
    int *d_err = nullptr;           /* kernel error word (bounded-wait timeouts) */
    int *h_err = nullptr;
    int inject_skip_chunk = -1;     /* testing: see udev_inject_copy_skip */
    int sart_wide_clusters = 0;     /* 16-CTA clusters of the segment-form SART FP that fit at once */
    cudaStream_t side = nullptr;    /* side copies (udev_copy_after), created on first use */
    cudaEvent_t side_go = nullptr;  /* current stream -> side stream ordering */
    cudaEvent_t side_done = nullptr;/* side stream -> current stream ordering */
    cudaEvent_t side_mark[UDEV_SIDE_SLOTS] = {};  /* udev_side_copy marks */
};

/* One-time kernel attribute setup (dynamic shared memory opt-in). */
int udev_kernels_init(udev *d);

/* The same for the SART per-angle kernels (non-portable cluster sizes). */
int udev_sart_init(udev *d);

#define UDEV_BIND(d)                                                                   \
    do {                                                                               \
        cudaError_t _e = cudaSetDevice((d)->device);                                   \
        if (_e != cudaSuccess) {                                                       \
            udev_set_error((d), "cudaSetDevice: %s", cudaGetErrorString(_e));         \
            return UFOIR_ERR_CUDA;                                                     \
        }                                                                              \
    } while (0)

#define UDEV_CHECK(d, call)                                                            \
    do {                                                                               \
        cudaError_t _e = (call);                                                       \
        if (_e != cudaSuccess) {                                                       \
            cudaGetLastError();                                                        \
            udev_set_error((d), "%s:%d %s: %s", __FILE__, __LINE__, #call,            \
                           cudaGetErrorString(_e));                                    \
            return _e == cudaErrorMemoryAllocation ? UFOIR_ERR_NOMEM : UFOIR_ERR_CUDA; \
        }                                                                              \
    } while (0)

/* Checks the launch that was just issued and counts it. */
int udev_after_launch(udev *d, const char *what);
/* Ensures the reduction scratch holds `partials` doubles and `outs` results. */
int udev_reduction_scratch(udev *d, size_t partials, size_t outs);

static inline unsigned int udev_div_up(size_t a, size_t b)
{
    return (unsigned int) ((a + b - 1) / b);
}

#endif
