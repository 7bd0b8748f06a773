/*
 * udev_asd.cu - the scalar logic of ASD-POCS on the device, so that an outer
 * iteration runs without reading anything back to the host and can be
 * captured as CUDA graphs.
 *
 * The reference keeps these scalars on the host in float
 * (asdpocs-task.c:457-506, 550-580); each kernel here does the same float
 * operations, one at a time and rounded as the host does:
 *   begin:  if (beta in [0, 1]) relax = beta              (:459, the property's range)
 *   init:   if (it == 0) dtgv = alpha * dp                (:478-479)
 *   step:   x = x - (dtgv / l1) * grad                    (:571-577)
 *   end:    beta = beta * beta_red;
 *           if (dg > r_max * dp && dd > 0.001) dtgv = dtgv * alpha_red;  it = it + 1   (:488-503)
 */
#include <cuda_runtime.h>

#include "udev_internal.cuh"

namespace {

__global__ void asd_begin_kernel(udev_asd_scalars S)
{
    const float beta = *S.beta;
    if (beta >= 0.0f && beta <= 1.0f)
        *S.relax = beta;
}

__global__ void asd_init_kernel(udev_asd_scalars S, float alpha, int n_slices)
{
    const int i = (int) threadIdx.x;
    if (*S.it == 0 && i < n_slices)
        S.dtgv[i] = __fmul_rn(alpha, S.dp[i]);
}

/* grid (blocks, slices) */
__global__ void __launch_bounds__(256) tv_step_kernel(float *__restrict__ x, const float *__restrict__ grad,
                                                     udev_asd_scalars S, size_t per_slice)
{
    const size_t s = blockIdx.y;
    const float factor = __fdiv_rn(S.dtgv[s], S.l1[s]);
    float *xs = x + s * per_slice;
    const float *gs = grad + s * per_slice;
    for (size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x; i < per_slice;
         i += (size_t) gridDim.x * blockDim.x)
        xs[i] = __fsub_rn(xs[i], __fmul_rn(factor, gs[i]));
}

__global__ void asd_end_kernel(udev_asd_scalars S, float beta_red, float r_max, float alpha_red, int n_slices)
{
    const int i = (int) threadIdx.x;
    if (i < n_slices && S.dg[i] > __fmul_rn(r_max, S.dp[i]) && S.dd[i] > 0.001f)
        S.dtgv[i] = __fmul_rn(S.dtgv[i], alpha_red);
    __syncthreads();
    if (i == 0) {
        *S.beta = __fmul_rn(*S.beta, beta_red);
        *S.it = *S.it + 1;
    }
}

}  // namespace

extern "C" int udev_asd_begin(udev *d, const udev_asd_scalars *S)
{
    UDEV_BIND(d);
    asd_begin_kernel<<<1, 1, 0, d->stream>>>(*S);
    return udev_after_launch(d, "asd_begin_kernel");
}

extern "C" int udev_asd_init(udev *d, const udev_asd_scalars *S, float alpha, int n_slices)
{
    if (n_slices <= 0 || n_slices > 1024) {
        udev_set_error(d, "asd: %d slices (1..1024)", n_slices);
        return UFOIR_ERR_INVALID;
    }
    UDEV_BIND(d);
    asd_init_kernel<<<1, n_slices, 0, d->stream>>>(*S, alpha, n_slices);
    return udev_after_launch(d, "asd_init_kernel");
}

extern "C" int udev_asd_tv_step(udev *d, float *x, const float *grad, const udev_asd_scalars *S, size_t per_slice,
                                int n_slices)
{
    if (per_slice == 0 || n_slices <= 0)
        return UFOIR_OK;
    if (n_slices > 65535) {
        udev_set_error(d, "asd: %d slices (at most 65535)", n_slices);
        return UFOIR_ERR_INVALID;
    }
    UDEV_BIND(d);
    const size_t want = (per_slice + 255) / 256;
    const size_t cap = ((size_t) d->sm_count * 16 + (size_t) n_slices - 1) / (size_t) n_slices;
    const unsigned int blocks = (unsigned int) (want < cap ? want : (cap > 0 ? cap : 1));
    tv_step_kernel<<<dim3(blocks, (unsigned int) n_slices), 256, 0, d->stream>>>(x, grad, *S, per_slice);
    return udev_after_launch(d, "tv_step_kernel");
}

extern "C" int udev_asd_end(udev *d, const udev_asd_scalars *S, float beta_red, float r_max, float alpha_red,
                            int n_slices)
{
    if (n_slices <= 0 || n_slices > 1024) {
        udev_set_error(d, "asd: %d slices (1..1024)", n_slices);
        return UFOIR_ERR_INVALID;
    }
    UDEV_BIND(d);
    asd_end_kernel<<<1, n_slices, 0, d->stream>>>(*S, beta_red, r_max, alpha_red, n_slices);
    return udev_after_launch(d, "asd_end_kernel");
}
