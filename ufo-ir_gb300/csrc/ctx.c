/*
 * ctx.c - context, memory helpers and host/device staging.
 */
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "host.h"

static char g_create_err[512];

int ufoir__fail(ufoir_ctx *ctx, int status, const char *fmt, ...)
{
    char buf[900];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (ctx && ctx->dev)
        udev_set_error(ctx->dev, "%s", buf);
    return status;
}

int ufoir_ctx_create(int device, uint64_t hbm_budget_bytes, ufoir_ctx **out)
{
    if (!out)
        return UFOIR_ERR_INVALID;
    *out = NULL;
    ufoir_ctx *ctx = (ufoir_ctx *) calloc(1, sizeof(*ctx));
    if (!ctx) {
        snprintf(g_create_err, sizeof(g_create_err), "out of host memory");
        return UFOIR_ERR_NOMEM;
    }
    int rc = udev_create(device, &ctx->dev, g_create_err, sizeof(g_create_err));
    if (rc != UFOIR_OK) {
        free(ctx);
        return rc;
    }
    ctx->autotune = UFOIR_AUTOTUNE_AUTO;
    if (hbm_budget_bytes == 0) {
        size_t fr = 0, tot = 0;
        if (udev_mem_info(ctx->dev, &fr, &tot) == UFOIR_OK)
            hbm_budget_bytes = (uint64_t) ((double) fr * 0.9);
    }
    ctx->hbm_budget = hbm_budget_bytes;
    *out = ctx;
    return UFOIR_OK;
}

void ufoir_ctx_destroy(ufoir_ctx *ctx)
{
    if (!ctx)
        return;
    ufoir__tune_free(ctx);
    udev_destroy(ctx->dev);
    free(ctx);
}

int ufoir_ctx_sm_count(const ufoir_ctx *ctx)
{
    return ctx ? udev_sm_count(ctx->dev) : 0;
}

int ufoir_ctx_set_autotune(ufoir_ctx *ctx, int on)
{
    if (!ctx || (on != UFOIR_AUTOTUNE_OFF && on != UFOIR_AUTOTUNE_ON && on != UFOIR_AUTOTUNE_AUTO))
        return UFOIR_ERR_INVALID;
    ctx->autotune = on;
    return UFOIR_OK;
}

const char *ufoir_last_error(const ufoir_ctx *ctx)
{
    if (!ctx)
        return g_create_err;
    return udev_error(ctx->dev);
}

int ufoir_ctx_synchronize(ufoir_ctx *ctx)
{
    if (!ctx)
        return UFOIR_ERR_INVALID;
    return udev_sync(ctx->dev);
}

void *ufoir_ctx_stream(ufoir_ctx *ctx)
{
    return ctx ? udev_stream(ctx->dev) : NULL;
}

int ufoir_ctx_set_stream(ufoir_ctx *ctx, void *stream)
{
    if (!ctx)
        return UFOIR_ERR_INVALID;
    udev_use_stream(ctx->dev, stream);
    return UFOIR_OK;
}

uint64_t ufoir_ctx_kernel_launches(const ufoir_ctx *ctx)
{
    return ctx ? udev_launches(ctx->dev) : 0;
}

int ufoir_ctx_inject_copy_timeout(ufoir_ctx *ctx, int chunk)
{
    if (!ctx || chunk < -1)
        return UFOIR_ERR_INVALID;
    udev_inject_copy_skip(ctx->dev, chunk);
    return UFOIR_OK;
}

int ufoir_ctx_timer_begin(ufoir_ctx *ctx)
{
    if (!ctx)
        return UFOIR_ERR_INVALID;
    return udev_timer_begin(ctx->dev);
}

int ufoir_ctx_timer_end(ufoir_ctx *ctx, float *ms)
{
    if (!ctx || !ms)
        return UFOIR_ERR_INVALID;
    return udev_timer_end(ctx->dev, ms);
}

int ufoir_device_alloc(ufoir_ctx *ctx, size_t bytes, void **ptr)
{
    if (!ctx || !ptr)
        return UFOIR_ERR_INVALID;
    int rc = udev_malloc(ctx->dev, ptr, bytes);
    if (rc == UFOIR_OK)
        rc = udev_sync(ctx->dev);
    return rc;
}

int ufoir_device_free(ufoir_ctx *ctx, void *ptr)
{
    if (!ctx)
        return UFOIR_ERR_INVALID;
    int rc = udev_free(ctx->dev, ptr);
    if (rc == UFOIR_OK)
        rc = udev_sync(ctx->dev);
    return rc;
}

int ufoir_host_alloc(ufoir_ctx *ctx, size_t bytes, void **ptr)
{
    if (!ctx || !ptr)
        return UFOIR_ERR_INVALID;
    return udev_host_malloc(ctx->dev, ptr, bytes);
}

int ufoir_host_free(ufoir_ctx *ctx, void *ptr)
{
    if (!ctx)
        return UFOIR_ERR_INVALID;
    return udev_host_free(ctx->dev, ptr);
}

int ufoir_memcpy(ufoir_ctx *ctx, void *dst, const void *src, size_t bytes)
{
    if (!ctx || (bytes && (!dst || !src)))
        return UFOIR_ERR_INVALID;
    return udev_memcpy(ctx->dev, dst, src, bytes);
}

int ufoir__alloc(ufoir_ctx *ctx, float **p, size_t count)
{
    return udev_malloc(ctx->dev, (void **) p, count * sizeof(float));
}

void ufoir__free(ufoir_ctx *ctx, void *p)
{
    if (p)
        udev_free(ctx->dev, p);
}

int ufoir__buf_in(ufoir_ctx *ctx, ufoir_buf *b, const float *user, size_t count, int copy_in)
{
    b->user = (float *) user;
    b->count = count;
    b->owned = 0;
    b->dev = NULL;
    if (!user)
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "NULL data pointer");
    if (udev_is_device_ptr(ctx->dev, user)) {
        b->dev = (float *) user;
        return UFOIR_OK;
    }
    int rc = ufoir__alloc(ctx, &b->dev, count);
    if (rc)
        return rc;
    b->owned = 1;
    if (copy_in)
        rc = udev_memcpy_async(ctx->dev, b->dev, user, count * sizeof(float));
    return rc;
}

int ufoir__buf_out(ufoir_ctx *ctx, ufoir_buf *b, int copy_out)
{
    /* a kernel that gave up on a bounded wait invalidates the result */
    int rc = udev_take_kernel_error(ctx->dev);
    if (rc == UFOIR_OK && b->owned && copy_out)
        rc = udev_memcpy(ctx->dev, b->user, b->dev, b->count * sizeof(float));
    ufoir__buf_release(ctx, b);
    return rc;
}

void ufoir__buf_release(ufoir_ctx *ctx, ufoir_buf *b)
{
    if (b->owned && b->dev)
        udev_free(ctx->dev, b->dev);
    b->dev = NULL;
    b->owned = 0;
}

int ufoir_sample_ceiling(ufoir_ctx *ctx, double *samples_per_s)
{
    if (!ctx || !samples_per_s)
        return UFOIR_ERR_INVALID;
    return udev_sample_ceiling(ctx->dev, samples_per_s);
}

int ufoir_sample_ceiling_bp(ufoir_ctx *ctx, double *samples_per_s)
{
    if (!ctx || !samples_per_s)
        return UFOIR_ERR_INVALID;
    return udev_sample_ceiling_bp(ctx->dev, samples_per_s);
}
