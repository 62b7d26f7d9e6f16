/*
 * Context, logging and device checks (reference lib/craw.c:26-43 for the
 * logging contract, 453-519 for context creation, replaced by CUDA
 * device queries).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include <craw/cuda.h>
#include <craw/debug.h>

#include "internal.h"

CRAW_API uint32_t craw_version_int(void)
{
    return ((uint32_t)CRAW_VERSION_MAJOR << 16) | ((uint32_t)CRAW_VERSION_MINOR << 8) |
           (uint32_t)CRAW_VERSION_MICRO;
}

CRAW_API void craw_log(void *opaque, enum CRAWLogLevel level, const char *fmt, ...)
{
    CRAWContext *ctx = opaque;
    va_list ap;

    va_start(ap, fmt);
    if (ctx && ctx->opts.log_cb) {
        if (level <= ctx->opts.log_level)
            ctx->opts.log_cb(ctx->opts.log_opaque, level, fmt, ap);
    } else if (level <= CRAW_LOG_WARN && level != CRAW_LOG_QUIET) {
        vfprintf(stderr, fmt, ap);
    }
    va_end(ap);
}

static int craw_cuda_err(cudaError_t e)
{
    switch (e) {
    case cudaSuccess:            return 0;
    case cudaErrorMemoryAllocation: return CRAW_ERROR(ENOMEM);
    case cudaErrorInvalidValue:  return CRAW_ERROR(EINVAL);
    case cudaErrorNoDevice:
    case cudaErrorInvalidDevice: return CRAW_ERROR(ENODEV);
    default:                     return CRAW_ERROR(EIO);
    }
}

CRAW_API int craw_cuda_check_device(int device, const char **missing)
{
    struct cudaDeviceProp prop;
    const char *dummy;

    if (!missing)
        missing = &dummy;
    *missing = NULL;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
        (void)cudaGetLastError();
        *missing = "a CUDA device with that ordinal";
        return CRAW_ERROR(ENOTSUP);
    }
    /* The kernels are built for sm_103a only. */
    if (prop.major != 10 || prop.minor != 3) {
        *missing = "compute capability 10.3 (sm_103)";
        return CRAW_ERROR(ENOTSUP);
    }
    if (prop.sharedMemPerBlockOptin < 200 * 1024) {
        *missing = "200 KB of shared memory per block";
        return CRAW_ERROR(ENOTSUP);
    }
    return 0;
}

CRAW_API int craw_context_create(CRAWContext **out, const CRAWCudaInitParams *params,
                                 const CRAWContextOptions *opts)
{
    CRAWContext *ctx;
    const char *missing = NULL;
    int ret;

    if (!out || !params)
        return CRAW_ERROR(EINVAL);
    *out = NULL;
    ctx = calloc(1, sizeof(*ctx));
    if (!ctx)
        return CRAW_ERROR(ENOMEM);
    if (opts)
        ctx->opts = *opts;
    else
        ctx->opts.log_level = CRAW_LOG_WARN;

    ret = craw_cuda_check_device(params->device, &missing);
    if (ret < 0) {
        craw_log(ctx, CRAW_LOG_ERROR, "CUDA device %d cannot run craw: needs %s\n",
                 params->device, missing);
        free(ctx);
        return ret;
    }
    ctx->device = params->device;
    if ((ret = craw_cuda_err(cudaSetDevice(ctx->device))) < 0)
        goto fail;
    if ((ret = craw_cuda_err(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount,
                                                    ctx->device))) < 0)
        goto fail;
    if (params->mem_pool) {
        ctx->pool = params->mem_pool;
    } else {
        struct cudaMemPoolProps pp;
        memset(&pp, 0, sizeof(pp));
        pp.allocType = cudaMemAllocationTypePinned;
        pp.handleTypes = cudaMemHandleTypeNone;
        pp.location.type = cudaMemLocationTypeDevice;
        pp.location.id = ctx->device;
        if ((ret = craw_cuda_err(cudaMemPoolCreate(&ctx->pool, &pp))) < 0)
            goto fail;
        ctx->own_pool = true;
    }
    if ((ret = craw_cuda_err(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking))) < 0)
        goto fail;
    craw_log(ctx, CRAW_LOG_VERBOSE, "craw context on CUDA device %d, %d SMs\n", ctx->device,
             ctx->sm_count);
    *out = ctx;
    return 0;
fail:
    craw_log(ctx, CRAW_LOG_ERROR, "CUDA context setup failed: %d\n", ret);
    if (ctx->stream)
        cudaStreamDestroy(ctx->stream);
    if (ctx->own_pool)
        cudaMemPoolDestroy(ctx->pool);
    free(ctx);
    return ret;
}

CRAW_API void craw_context_free(CRAWContext **pctx)
{
    CRAWContext *ctx;

    if (!pctx || !*pctx)
        return;
    ctx = *pctx;
    cudaSetDevice(ctx->device);
    if (ctx->stream) {
        cudaStreamSynchronize(ctx->stream);
        cudaStreamDestroy(ctx->stream);
    }
    if (ctx->own_pool)
        cudaMemPoolDestroy(ctx->pool);
    free(ctx);
    *pctx = NULL;
}

/* Allocation failure injection for the tests: the k-th allocation from now
 * (1-based) fails with ENOMEM; 0 disarms it. Not thread safe, like the
 * rest of the library. */
static int craw_fail_countdown;

int craw_forced_denoise_shape = -1;

CRAW_API int craw_debug_force_denoise_shape(int shape)
{
    if (shape < -1 || shape >= CRAW_K_DN_SHAPE_NB)
        return CRAW_ERROR(EINVAL);
    craw_forced_denoise_shape = shape;
    return 0;
}

/* The marking band of the exact denoise rounding, in units of the float
 * path's error bound, and whether its float decision stage runs. */
float craw_round_scale = 2.0f;
int craw_round_decide = 1;

CRAW_API float craw_debug_denoise_round(float scale)
{
    const float was = craw_round_scale;
    if (scale >= 0.0f)
        craw_round_scale = scale;
    return was;
}

CRAW_API int craw_debug_denoise_round_decide(int on)
{
    const int was = craw_round_decide;
    if (on >= 0)
        craw_round_decide = on ? 1 : 0;
    return was;
}

CRAW_API void craw_debug_fail_alloc(int k)
{
    craw_fail_countdown = k;
}

CRAW_API int craw_debug_rcd_tma(int on)
{
    const int was = craw_k_rcd_tma;
    craw_k_rcd_tma = on ? 1 : 0;
    return was;
}

CRAW_API int craw_debug_rcd_strips(int mode)
{
    const int was = craw_k_rcd_strips;
    if (mode >= 0 && mode <= 2)
        craw_k_rcd_strips = mode;
    return was;
}

CRAW_API int craw_debug_denoise_tma(int on)
{
    const int was = craw_k_dn_tma;
    craw_k_dn_tma = on ? 1 : 0;
    return was;
}

int craw_dev_alloc(CRAWContext *ctx, void **ptr, size_t bytes)
{
    *ptr = NULL;
    if (craw_fail_countdown > 0 && --craw_fail_countdown == 0)
        return CRAW_ERROR(ENOMEM);
    return craw_cuda_err(cudaMallocFromPoolAsync(ptr, bytes, ctx->pool, ctx->stream));
}

void craw_dev_free(CRAWContext *ctx, void *ptr)
{
    if (ptr)
        cudaFreeAsync(ptr, ctx->stream);
}

int craw_dev_sync(CRAWContext *ctx)
{
    return craw_cuda_err(cudaStreamSynchronize(ctx->stream));
}
