/*
 * Batched development of frames of uneven sizes: one persistent launch per
 * recording, captured once into a CUDA graph per set of frame shapes and
 * replayed after a copy of the per-frame constant table. See
 * include/craw/batch.h.
 */
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include <craw/batch.h>

#include "internal.h"

#define BATCH_MAX 64

struct CRAWBatch {
    CRAWContext *ctx;
    CRAWBatchParams params;
    int shape;
    bool fused, use_graph, denoise;
    uint16_t *clean[BATCH_MAX];
    size_t clean_pitch;
    CRAWKBatchTable *table;          /* host; each launch carries a copy */
    cudaStream_t cap_stream;
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    /* The shapes the captured graph was made for. */
    uint32_t sig_nb;
    uint32_t sig_w[BATCH_MAX], sig_h[BATCH_MAX];
    bool sig_dn[BATCH_MAX];
    int32_t sig_dn_items, sig_dv_items;
    uint64_t captures, replays;
    /* Frames developed by the single-frame kernels. */
    uint64_t direct_pixels;
    int direct_shape;                /* their denoise tile shape, autotuned; -1: none */
    uint64_t direct_frames;
    CRAWKBatchFrame direct[BATCH_MAX];
};

CRAW_API void craw_batch_params_init(CRAWBatchParams *p)
{
    if (!p)
        return;
    memset(p, 0, sizeof(*p));
    p->max_frames = 16;
    p->debayer = CRAW_DEBAYER_RCD;
    p->out_space = CRAW_CS_XYZ_D65;
    p->out_format = CRAW_FORMAT_RGBA32F;
}

static void batch_release(CRAWBatch *b)
{
    CRAWContext *ctx = b->ctx;
    cudaSetDevice(ctx->device);
    if (b->exec)
        cudaGraphExecDestroy(b->exec);
    if (b->graph)
        cudaGraphDestroy(b->graph);
    for (uint32_t i = 0; i < BATCH_MAX; i++)
        craw_dev_free(ctx, b->clean[i]);
    craw_dev_sync(ctx);
    free(b->table);
    if (b->cap_stream)
        cudaStreamDestroy(b->cap_stream);
    free(b);
}

/* Items of each phase for a frame list, and every frame's place in them. */
static void batch_layout(CRAWBatch *b, uint32_t nb, const uint32_t *w, const uint32_t *h,
                         const bool *dn, CRAWKBatchFrame *F, int32_t *dn_items, int32_t *dv_items)
{
    int32_t dn_n = 0, dv_n = 0;
    for (uint32_t i = 0; i < nb; i++) {
        craw_k_batch_tiles((int32_t)w[i], (int32_t)h[i], b->shape, &F[i].dn_tx, &F[i].dn_ty,
                           &F[i].dv_tx, &F[i].dv_ty);
        if (!dn[i])
            F[i].dn_tx = F[i].dn_ty = 0;
        F[i].dn_first = dn_n;
        F[i].dv_first = dv_n;
        dn_n += F[i].dn_tx * F[i].dn_ty;
        dv_n += F[i].dv_tx * F[i].dv_ty;
    }
    *dn_items = dn_n;
    *dv_items = dv_n;
}

/* Times one max-size frame through each denoise tile shape and keeps the
 * faster (the work does not depend on the data). */
static int batch_autotune(CRAWBatch *b)
{
    CRAWContext *ctx = b->ctx;
    const uint32_t w = b->params.max_width, h = b->params.max_height;
    CRAWKBatchFrame *F = &b->table->f[0];
    void *out = NULL;
    uint16_t *mosaic;
    size_t out_pitch = (((size_t)w * 16) + 255) / 256 * 256;
    cudaEvent_t e0 = NULL, e1 = NULL;
    float best = 1e30f;
    int ret = 0;

    /* The output image, then a grey mosaic to denoise. */
    if ((ret = craw_dev_alloc(ctx, &out, out_pitch * h + b->clean_pitch * h)) < 0)
        return ret;
    mosaic = (uint16_t *)((char *)out + out_pitch * h);
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        ret = CRAW_ERROR(ENOMEM);
        goto done;
    }
    /* A grey frame with plausible constants. */
    cudaMemset2DAsync(mosaic, b->clean_pitch, 0x08, (size_t)w * 2, h, ctx->stream);
    for (int shape = 0; shape < CRAW_K_BATCH_DN_NB; shape++) {
        int32_t dn_items, dv_items;
        bool dn = true;
        float t = 0.0f, ms = 1e30f;
        b->shape = shape;
        memset(F, 0, sizeof(*F));
        F->dn.pw = (int32_t)(w / 2);
        F->dn.ph = (int32_t)(h / 2);
        F->dn.gat_a = 1e-3f; F->dn.gat_c = 1e-6f; F->dn.gat_sc = 1e-3f; F->dn.gat_fwd = 2000.0f;
        F->dn.gat_inv = 2.5e-4f; F->dn.gat_off = 1e-3f; F->dn.gat_t0 = 2.0f;
        F->dn.inv_h2 = 1.0f; F->dn.guard_lo = 0.9f; F->dn.guard_inv = 10.0f;
        F->dn.mode = CRAW_K_DN_SPATIAL;
        for (int s = 0; s < 4; s++) {
            F->dn.inv_range[s] = 16.0f;
            F->dn.range[s] = 0.0625f;
            F->dv.inv_range[s] = 16.0f;
            F->dv.range[s] = 0.0625f;
            F->dv.wbs[s] = 1.0f;
        }
        F->dio.src = mosaic;
        F->dio.src_pitch = b->clean_pitch;
        F->dio.dst = b->clean[0];
        F->dio.dst_pitch = b->clean_pitch;
        F->dv.width = (int32_t)w;
        F->dv.height = (int32_t)h;
        F->dv.clip = 1.0f;
        F->dv.method = b->params.debayer;
        F->dv.color.m[0][0] = F->dv.color.m[1][1] = F->dv.color.m[2][2] = 1.0f;
        F->vio.src = b->clean[0];
        F->vio.src_pitch = b->clean_pitch;
        F->vio.dst = out;
        F->vio.dst_pitch = out_pitch;
        batch_layout(b, 1, &w, &h, &dn, F, &dn_items, &dv_items);
        for (int r = 0; r < 3; r++) {
            cudaEventRecord(e0, ctx->stream);
            if (craw_k_batch(b->table, 1, dn_items, dv_items, b->params.debayer, shape, b->fused,
                             ctx->stream) < 0) {
                ret = CRAW_ERROR(EIO);
                goto done;
            }
            cudaEventRecord(e1, ctx->stream);
            if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&t, e0, e1) != cudaSuccess) {
                ret = CRAW_ERROR(EIO);
                goto done;
            }
            if (r > 0 && t < ms)
                ms = t;
        }
        if (ms < best) {
            best = ms;
            ret = shape;
        }
    }
    b->shape = ret;
    craw_log(ctx, CRAW_LOG_VERBOSE, "batch autotune %ux%u: denoise shape %d, %.3f ms\n", w, h,
             b->shape, (double)best);
    ret = 0;
    /* The single-frame kernel's shapes, for frames developed directly. */
    b->direct_shape = -1;
    if ((uint64_t)w * h >= b->direct_pixels) {
        best = 1e30f;
        for (int shape = 0; shape < CRAW_K_DN_SHAPE_NB; shape++) {
            float t = 0.0f, ms = 1e30f;
            for (int r = 0; r < 3; r++) {
                cudaEventRecord(e0, ctx->stream);
                if (craw_k_denoise(&F->dn, &F->dio, shape, NULL, NULL, ctx->stream) < 0) {
                    ret = CRAW_ERROR(EIO);
                    goto done;
                }
                cudaEventRecord(e1, ctx->stream);
                if (cudaEventSynchronize(e1) != cudaSuccess ||
                    cudaEventElapsedTime(&t, e0, e1) != cudaSuccess) {
                    ret = CRAW_ERROR(EIO);
                    goto done;
                }
                if (r > 0 && t < ms)
                    ms = t;
            }
            if (ms < best) {
                best = ms;
                b->direct_shape = shape;
            }
        }
        craw_log(ctx, CRAW_LOG_VERBOSE, "batch autotune %ux%u: direct denoise shape %d, %.3f ms\n", w, h,
                 b->direct_shape, (double)best);
    }
done:
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    craw_dev_free(ctx, out);
    if (craw_dev_sync(ctx) < 0 && ret == 0)
        ret = CRAW_ERROR(EIO);
    return ret;
}

CRAW_API int craw_batch_create(CRAWContext *ctx, const CRAWBatchParams *params, CRAWBatch **out)
{
    CRAWBatch *b;
    int ret;

    if (!ctx || !params || !out)
        return CRAW_ERROR(EINVAL);
    *out = NULL;
    if (!params->max_frames || params->max_frames > BATCH_MAX || !params->max_width ||
        !params->max_height || (params->max_width & 1) || (params->max_height & 1) ||
        params->max_width < 12 || params->max_height < 12 || params->max_width > 32768 ||
        params->max_height > 32768 || (unsigned)params->debayer >= CRAW_DEBAYER_NB ||
        (unsigned)params->out_space >= CRAW_CS_NB ||
        !craw_is_out_format(params->out_format))
        return CRAW_ERROR(EINVAL);
    if ((params->flags & ~(uint32_t)(CRAW_PIPELINE_FLAG_DENOISE | CRAW_BATCH_FLAG_UNFUSED |
                                      CRAW_BATCH_FLAG_FUSED | CRAW_BATCH_FLAG_NO_GRAPH)) ||
        ((params->flags & CRAW_BATCH_FLAG_FUSED) && (params->flags & CRAW_BATCH_FLAG_UNFUSED))) {
        craw_log(ctx, CRAW_LOG_ERROR, "Batch flags 0x%x: only the denoise is supported in a batch\n",
                 params->flags);
        return CRAW_ERROR(ENOTSUP);
    }
    b = calloc(1, sizeof(*b));
    if (!b)
        return CRAW_ERROR(ENOMEM);
    b->ctx = ctx;
    b->params = *params;
    b->fused = (params->flags & CRAW_BATCH_FLAG_FUSED) != 0;
    b->use_graph = !(params->flags & CRAW_BATCH_FLAG_NO_GRAPH);
    b->denoise = params->flags & CRAW_PIPELINE_FLAG_DENOISE;
    b->direct_pixels = params->direct_pixels == UINT32_MAX ? UINT64_MAX :
                       (params->direct_pixels ? params->direct_pixels : CRAW_BATCH_DIRECT_PIXELS);
    b->direct_shape = -1;
    cudaSetDevice(ctx->device);

    b->clean_pitch = (((size_t)params->max_width * 2) + 255) / 256 * 256;
    for (uint32_t i = 0; i < params->max_frames; i++)
        if ((ret = craw_dev_alloc(ctx, (void **)&b->clean[i], b->clean_pitch * params->max_height)) < 0)
            goto fail;
    if (!(b->table = calloc(1, sizeof(*b->table)))) {
        ret = CRAW_ERROR(ENOMEM);
        goto fail;
    }
    if (cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking) != cudaSuccess) {
        ret = CRAW_ERROR(ENOMEM);
        goto fail;
    }
    if ((ret = craw_dev_sync(ctx)) < 0)
        goto fail;
    if (b->denoise && (ret = batch_autotune(b)) < 0)
        goto fail;
    *out = b;
    return 0;
fail:
    craw_log(ctx, CRAW_LOG_ERROR, "Batch creation failed (%d)\n", ret);
    batch_release(b);
    return ret;
}

CRAW_API void craw_batch_free(CRAWBatch **pb)
{
    if (!pb || !*pb)
        return;
    batch_release(*pb);
    *pb = NULL;
}

CRAW_API int craw_batch_get_info(CRAWBatch *b, CRAWBatchInfo *info)
{
    if (!b || !info)
        return CRAW_ERROR(EINVAL);
    memset(info, 0, sizeof(*info));
    info->denoise_shape = b->shape;
    info->fused = b->fused;
    info->graph = b->use_graph;
    info->captures = b->captures;
    info->replays = b->replays;
    info->direct_shape = b->direct_shape;
    info->direct_frames = b->direct_frames;
    return 0;
}

static int batch_capture(CRAWBatch *b, uint32_t nb, int32_t dn_items, int32_t dv_items)
{
    cudaGraph_t g = NULL;
    cudaGraphExec_t e = NULL;
    int ret;

    if (cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return CRAW_ERROR(EIO);
    ret = craw_k_batch(b->table, (int32_t)nb, dn_items, dv_items, b->params.debayer, b->shape,
                       b->fused, b->cap_stream);
    if (cudaStreamEndCapture(b->cap_stream, &g) != cudaSuccess || ret < 0) {
        if (g)
            cudaGraphDestroy(g);
        (void)cudaGetLastError();
        return CRAW_ERROR(EIO);
    }
    if (cudaGraphInstantiate(&e, g, 0) != cudaSuccess) {
        cudaGraphDestroy(g);
        (void)cudaGetLastError();
        return CRAW_ERROR(EIO);
    }
    if (b->exec)
        cudaGraphExecDestroy(b->exec);
    if (b->graph)
        cudaGraphDestroy(b->graph);
    b->graph = g;
    b->exec = e;
    b->captures++;
    return 0;
}

static int batch_persistent(CRAWBatch *b, cudaStream_t s, uint32_t nb, const uint32_t *w, const uint32_t *h,
                            const bool *dn);

CRAW_API int craw_batch_record(CRAWBatch *b, cudaStream_t s, uint32_t nb, const CRAWImage *src,
                               const CRAWImage *dst, const CRAWFrameParams *fp)
{
    CRAWContext *ctx;
    CRAWKBatchFrame *F;
    uint32_t w[BATCH_MAX], h[BATCH_MAX];
    bool dn[BATCH_MAX];
    int ret;

    if (!b || !src || !dst || !fp || !nb)
        return CRAW_ERROR(EINVAL);
    ctx = b->ctx;
    if (nb > b->params.max_frames) {
        craw_log(ctx, CRAW_LOG_ERROR, "%u frames; the batch holds %u\n", nb, b->params.max_frames);
        return CRAW_ERROR(EINVAL);
    }
    /* Each launch carries its own copy of the table (a kernel parameter),
     * so the host table is free again as soon as the launch is enqueued. */
    F = b->table->f;
    memset(F, 0, nb * sizeof(*F));
    for (uint32_t i = 0; i < nb; i++) {
        w[i] = src[i].width;
        h[i] = src[i].height;
        if (!fp[i].profile || (w[i] & 1) || (h[i] & 1) || w[i] < 12 || h[i] < 12 ||
            w[i] > b->params.max_width || h[i] > b->params.max_height) {
            craw_log(ctx, CRAW_LOG_ERROR, "Frame %u: %ux%u does not fit the batch (%ux%u, even, >= 12)\n",
                     i, w[i], h[i], b->params.max_width, b->params.max_height);
            return CRAW_ERROR(EINVAL);
        }
        if ((ret = craw_image_check(ctx, &src[i], CRAW_FORMAT_R16_UNORM, w[i], h[i], "Source")) < 0 ||
            (ret = craw_image_check(ctx, &dst[i], b->params.out_format, w[i], h[i], "Destination")) < 0)
            return ret;
        if (craw_images_overlap(&src[i], &dst[i])) {
            craw_log(ctx, CRAW_LOG_ERROR, "Frame %u: source and destination alias\n", i);
            return CRAW_ERROR(EINVAL);
        }
        for (uint32_t j = 0; j < i; j++)
            if (craw_images_overlap(&dst[i], &dst[j]) || craw_images_overlap(&dst[i], &src[j]) ||
                craw_images_overlap(&src[i], &dst[j])) {
                craw_log(ctx, CRAW_LOG_ERROR, "Frames %u and %u share memory\n", j, i);
                return CRAW_ERROR(EINVAL);
            }
        if ((ret = craw_develop_consts(ctx, w[i], h[i], b->params.debayer, false, b->params.out_space,
                                       &fp[i], &F[i].dv)) < 0)
            return ret;
        dn[i] = b->denoise && fp[i].denoise_strength > 0.0f;
        if (dn[i] && (ret = craw_denoise_consts(ctx, w[i], h[i], &fp[i], CRAW_K_DN_SPATIAL, &F[i].dn, NULL)) < 0)
            return ret;
        F[i].dio.src = src[i].data;
        F[i].dio.src_pitch = src[i].pitch;
        F[i].dio.dst = b->clean[i];
        F[i].dio.dst_pitch = b->clean_pitch;
        F[i].vio.src = dn[i] ? b->clean[i] : src[i].data;
        F[i].vio.src_pitch = dn[i] ? b->clean_pitch : src[i].pitch;
        F[i].vio.dst = dst[i].data;
        F[i].vio.dst_pitch = dst[i].pitch;
        F[i].vio.dst_fmt = craw_out_layout(dst[i].format);
    }

    /* Large frames go to the single-frame kernels; the others, in order,
     * stay in the table of the persistent launch. */
    uint32_t nd = 0, ns = 0;
    bool ddn[BATCH_MAX];
    for (uint32_t i = 0; i < nb; i++) {
        if ((uint64_t)w[i] * h[i] >= b->direct_pixels) {
            b->direct[nd] = F[i];
            ddn[nd++] = dn[i];
            continue;
        }
        if (ns != i) {
            F[ns] = F[i];
            w[ns] = w[i];
            h[ns] = h[i];
            dn[ns] = dn[i];
        }
        ns++;
    }
    if (ns > 0 && (ret = batch_persistent(b, s, ns, w, h, dn)) < 0)
        return ret;
    for (uint32_t d = 0; d < nd; d++) {
        if ((ddn[d] && craw_k_denoise(&b->direct[d].dn, &b->direct[d].dio, b->direct_shape, NULL,
                                      b->direct[d].vio.err, s) < 0) ||
            craw_k_develop(&b->direct[d].dv, &b->direct[d].vio, 0, s) < 0)
            return CRAW_ERROR(EIO);
        b->direct_frames++;
    }
    return 0;
}

/* The persistent launch of frames 0 .. nb-1 of the table: a replay of the
 * graph captured for these shapes (captured now if they are new), or a
 * launch. */
static int batch_persistent(CRAWBatch *b, cudaStream_t s, uint32_t nb, const uint32_t *w, const uint32_t *h,
                            const bool *dn)
{
    CRAWContext *ctx = b->ctx;
    CRAWKBatchFrame *F = b->table->f;
    int32_t dn_items, dv_items;
    bool same;
    int ret;

    batch_layout(b, nb, w, h, dn, F, &dn_items, &dv_items);

    same = b->exec && b->sig_nb == nb;
    for (uint32_t i = 0; same && i < nb; i++)
        same = b->sig_w[i] == w[i] && b->sig_h[i] == h[i] && b->sig_dn[i] == dn[i];
    if (b->use_graph && !same) {
        if ((ret = batch_capture(b, nb, dn_items, dv_items)) < 0) {
            craw_log(ctx, CRAW_LOG_ERROR, "Capturing the batch launch into a CUDA graph failed\n");
            return ret;
        }
        b->sig_nb = nb;
        for (uint32_t i = 0; i < nb; i++) {
            b->sig_w[i] = w[i];
            b->sig_h[i] = h[i];
            b->sig_dn[i] = dn[i];
        }
        b->sig_dn_items = dn_items;
        b->sig_dv_items = dv_items;
    }
    if (b->use_graph) {
        /* The captured nodes get this recording's table and counts. */
        if (craw_k_batch_update(b->exec, b->graph, b->table, (int32_t)nb, dn_items, dv_items) < 0 ||
            cudaGraphLaunch(b->exec, s) != cudaSuccess) {
            (void)cudaGetLastError();
            return CRAW_ERROR(EIO);
        }
        b->replays++;
    } else if (craw_k_batch(b->table, (int32_t)nb, dn_items, dv_items, b->params.debayer, b->shape,
                            b->fused, s) < 0) {
        return CRAW_ERROR(EIO);
    }
    return 0;
}
