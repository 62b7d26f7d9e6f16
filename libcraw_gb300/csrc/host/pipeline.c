/*
 * The pipeline: create, record, free, and the AWB and profiling readback
 * (reference lib/pipeline.c:543-2415, re-designed for CUDA).
 *
 * A recording evaluates the frame's constants on the host, exactly as the
 * reference does, and enqueues at most five kernels on the caller's
 * stream:
 *
 *   denoise   mosaic (+ state) -> denoised mosaic (+ next state)
 *   develop   mosaic -> dst directly (prep, debayer, colour and the AWB
 *             block records fused); with the chroma denoise, mosaic ->
 *             intermediate + quarter-resolution block means instead
 *   [blur]    quarter -> filtered quarter
 *   [up]      intermediate + quarters -> dst (+ AWB block records)
 *   awb       block records -> histogram, then a copy into the pinned
 *             host slot of this recording
 *
 * The library never synchronises the caller's stream. Intermediates come
 * from a CUDA memory pool (cudaMallocFromPoolAsync on the context's own
 * stream, which is synchronised once at the end of creation).
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include <craw/debug.h>
#include <craw/pipeline.h>

#include "internal.h"

static_assert(sizeof(CRAWPipelineParams) == 256, "CRAWPipelineParams size");
static_assert(sizeof(CRAWFrameParams) == 264, "CRAWFrameParams size");
static_assert(sizeof(CRAWContextOptions) == 1024, "CRAWContextOptions size");
static_assert(sizeof(CRAWCudaInitParams) == 64, "CRAWCudaInitParams size");

#define HIST_N (CRAW_AWB_HIST_BINS * CRAW_AWB_HIST_BINS)
#define HIST_BYTES (3 * HIST_N * sizeof(uint32_t))
#define DEFER_BYTES (CRAW_K_AWB_DEFER_MAX * sizeof(CRAWKAwbDeferred))

#define MAX_STAGES 16

enum { ST_DENOISE, ST_DEVELOP, ST_BLUR, ST_UP, ST_AWB, ST_HL, ST_ROUND, ST_NB };
static const char *const stage_names[ST_NB] = {
    "denoise_nlm", "develop", "chroma_blur", "chroma_up_color", "awb_reduce", "highlights",
    "denoise_round",
};
static const char *const plain_stage_names[ST_NB] = {
    "plain_denoise", "plain_develop", "plain_chroma", "plain_chroma", "plain_awb", "highlights",
    "denoise_round",
};

/* One AWB slot. On the host, pinned: the three histograms, the count of
 * deferred blocks and the first CRAW_K_AWB_DEFER_MAX of them, filled by
 * two async copies. On the device: the slot's whole list of deferred
 * blocks (its count, then one entry per 8x8 block of the frame at most),
 * from which a count above CRAW_K_AWB_DEFER_MAX is read on demand. */
#define SLOT_BYTES (HIST_BYTES + 16 + DEFER_BYTES)
struct awb_slot {
    uint8_t *host;            /* SLOT_BYTES */
    uint8_t *list;            /* device: the count (16 B), then room for
                               * max(nb_blocks, CRAW_K_AWB_DEFER_MAX) entries */
    bool folded;              /* deferred blocks already binned */
};

struct prof_slot {
    cudaEvent_t ev[MAX_STAGES][2];
    int stage[MAX_STAGES];
    uint32_t nb;
};

struct CRAWPipeline {
    CRAWContext *ctx;
    CRAWPipelineParams params;
    bool has_denoise, has_temporal, has_chroma, awb, profile, keep, plain, fp16;
    bool has_hl;                 /* highlight reconstruction built */
    CRAWKHighlight hl;           /* its level sizes (constants filled per frame) */
    uint16_t *hl_mosaic;         /* the rebuilt mosaic, fp16 */
    size_t hl_pitch;
    void *hl_levels;            /* the colour field's pyramid */
    int dn_shape[2], dev_shape;   /* denoise tile shape without / with a history */
    bool tune_held;              /* holds its size's autotuner cache entry */

    /* Device memory. */
    uint16_t *clean;  size_t clean_pitch;
    float *lvl[2];    size_t lvl_pitch;
    uint8_t *var[2];  size_t var_pitch;
    int tn_prev, tn_cur;
    void *inter;      size_t inter_pitch;
    void *q, *qf;     size_t q_pitch;
    int qw, qh;
    uint64_t *awb_rec;
    uint8_t *awb_dev;         /* HIST_BYTES: the histograms being built */
    uint32_t nb_blocks;
    uint32_t *kerr;           /* CRAW_K_ERR_* bits the kernels set */
    uint32_t *round_flags;    /* marks of the exact rounding, CRAW_K_ROUND_WORDS */
    uint32_t *round_stats;    /* its statistics, CRAW_K_ROUND_STATS_BYTES */
    uint32_t *round_list;     /* marked, then undecided samples, CRAW_K_ROUND_LIST entries
                               * each, then the counters */

    /* Plain-pipeline scratch. */
    float *p_v, *p_scratch, *p_t, *p_var;

    struct awb_slot slots[4];
    uint32_t nb_slots;
    uint64_t nb_recorded;
    bool last_denoised, last_hl;

    struct prof_slot prof[CRAW_PIPELINE_PROFILE_SLOTS];
    uint64_t prof_recorded;
    CRAWStageTime prof_agg[MAX_STAGES];
};

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

CRAW_API void craw_pipeline_params_init(CRAWPipelineParams *p)
{
    if (!p)
        return;
    memset(p, 0, sizeof(*p));
    p->cfa = CRAW_CFA_RGGB;
    p->debayer = CRAW_DEBAYER_RCD;
    p->out_space = CRAW_CS_XYZ_D65;
    p->out_format = CRAW_FORMAT_RGBA16F;
    p->nb_awb_slots = 1;
}

CRAW_API void craw_frame_params_init(CRAWFrameParams *fp)
{
    if (!fp)
        return;
    memset(fp, 0, sizeof(*fp));
    fp->wb_mode = CRAW_WB_AS_SHOT;
}

static int alloc_pitched(CRAWPipeline *p, void **ptr, size_t *pitch, size_t row_bytes, uint32_t rows)
{
    size_t pt = align_up(row_bytes, 256);
    if (pitch)
        *pitch = pt;
    return craw_dev_alloc(p->ctx, ptr, pt * rows);
}

static void tune_release(CRAWPipeline *p);

static void release(CRAWPipeline *p)
{
    CRAWContext *ctx = p->ctx;
    tune_release(p);
    void *bufs[] = {
        p->clean, p->lvl[0], p->lvl[1], p->var[0], p->var[1], p->inter, p->q, p->qf,
        p->awb_rec, p->awb_dev, p->kerr, p->p_v, p->p_scratch, p->p_t, p->p_var,
        p->hl_mosaic, p->hl_levels, p->round_flags, p->round_stats, p->round_list,
    };
    cudaSetDevice(ctx->device);
    for (size_t i = 0; i < CRAW_ARRAY_ELEMS(bufs); i++)
        craw_dev_free(ctx, bufs[i]);
    craw_dev_sync(ctx);
    for (uint32_t i = 0; i < 4; i++) {
        craw_dev_free(ctx, p->slots[i].list);
        if (p->slots[i].host)
            cudaFreeHost(p->slots[i].host);
    }
    for (int s = 0; s < CRAW_PIPELINE_PROFILE_SLOTS; s++)
        for (int i = 0; i < MAX_STAGES; i++)
            for (int j = 0; j < 2; j++)
                if (p->prof[s].ev[i][j])
                    cudaEventDestroy(p->prof[s].ev[i][j]);
    free(p);
}

/* The autotuner: the fastest denoise tile shape for this frame size, with
 * and without a temporal history, timed on the context's own stream over a
 * scratch mosaic (the filter's work does not depend on the data), and
 * remembered for the process (each of the two on its own) so that every
 * later pipeline of the same size starts at once with the same shapes:
 * pipelines of one size give the same results. An entry is held while a
 * pipeline of its size exists, so its shapes stay those of every live
 * pipeline of that size; when the table is full, the least recently used
 * entry that no pipeline holds makes room. */
#define TUNE_CACHE 256
static struct tune_entry {
    uint32_t w, h;
    int shape[2];
    bool known[2];
    uint32_t live;               /* pipelines of this size holding the entry */
    uint64_t used;               /* tick of the last lookup */
} tune_cache[TUNE_CACHE];
static int tune_nb;
static uint64_t tune_tick;
static pthread_mutex_t tune_lock = PTHREAD_MUTEX_INITIALIZER;

/* The cache entry of a size, created if asked and there is room (a free
 * slot, or the least recently used entry no pipeline holds); NULL
 * otherwise. Called with tune_lock held. */
static struct tune_entry *tune_entry(uint32_t w, uint32_t h, bool create)
{
    struct tune_entry *e = NULL;
    for (int i = 0; i < tune_nb; i++)
        if (tune_cache[i].w == w && tune_cache[i].h == h) {
            tune_cache[i].used = ++tune_tick;
            return &tune_cache[i];
        }
    if (!create)
        return NULL;
    if (tune_nb < TUNE_CACHE) {
        e = &tune_cache[tune_nb++];
    } else {
        for (int i = 0; i < TUNE_CACHE; i++)
            if (!tune_cache[i].live && (!e || tune_cache[i].used < e->used))
                e = &tune_cache[i];
        if (!e)
            return NULL;
    }
    memset(e, 0, sizeof(*e));
    e->w = w;
    e->h = h;
    e->used = ++tune_tick;
    return e;
}

/* Lets go of the cache entry a pipeline holds. */
static void tune_release(CRAWPipeline *p)
{
    struct tune_entry *e;
    if (!p->tune_held)
        return;
    pthread_mutex_lock(&tune_lock);
    if ((e = tune_entry(p->params.width, p->params.height, false)) && e->live)
        e->live--;
    pthread_mutex_unlock(&tune_lock);
    p->tune_held = false;
}

static int time_denoise(CRAWPipeline *p, const CRAWKDenoise *k, const CRAWKDenoiseIO *io, int shape,
                        float *ms)
{
    CRAWContext *ctx = p->ctx;
    cudaEvent_t e0, e1;
    int ret = 0;
    if (cudaEventCreate(&e0) != cudaSuccess)
        return CRAW_ERROR(ENOMEM);
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return CRAW_ERROR(ENOMEM);
    }
    /* One launch to warm up, then the best of three. */
    *ms = 1e30f;
    for (int r = 0; r < 4 && ret == 0; r++) {
        float t = 0.0f;
        cudaEventRecord(e0, ctx->stream);
        ret = craw_k_denoise(k, io, shape, NULL, NULL, ctx->stream);
        cudaEventRecord(e1, ctx->stream);
        if (ret == 0 && cudaEventSynchronize(e1) == cudaSuccess &&
            cudaEventElapsedTime(&t, e0, e1) == cudaSuccess && r > 0 && t < *ms)
            *ms = t;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ret < 0 ? CRAW_ERROR(EIO) : 0;
}

static int autotune(CRAWPipeline *p)
{
    CRAWContext *ctx = p->ctx;
    const uint32_t w = p->params.width, h = p->params.height;
    uint16_t *mosaic = NULL;
    float *lvl = NULL;
    uint8_t *var = NULL;
    size_t mp, lp, vp;
    int ret = 0;
    bool need[2] = { p->has_denoise, p->has_temporal };
    struct tune_entry *e;

    const bool want[2] = { need[0], need[1] };

    pthread_mutex_lock(&tune_lock);
    if ((e = tune_entry(w, h, false))) {
        for (int hist = 0; hist < 2; hist++)
            if (need[hist] && e->known[hist]) {
                p->dn_shape[hist] = e->shape[hist];
                need[hist] = false;
            }
        if (!need[0] && !need[1]) {
            e->live++;
            p->tune_held = true;
        }
    }
    pthread_mutex_unlock(&tune_lock);
    if (!need[0] && !need[1])
        return 0;

    if ((ret = alloc_pitched(p, (void **)&mosaic, &mp, (size_t)w * 2, h)) < 0 ||
        (ret = alloc_pitched(p, (void **)&lvl, &lp, (size_t)w * 4, h)) < 0 ||
        (ret = alloc_pitched(p, (void **)&var, &vp, (size_t)w, h)) < 0)
        goto done;
    /* A mid-grey mosaic, a state of level 0.25 and unit variance. */
    cudaMemset2DAsync(mosaic, mp, 0x08, (size_t)w * 2, h, ctx->stream);
    cudaMemset2DAsync(lvl, lp, 0, (size_t)w * 4, h, ctx->stream);
    cudaMemset2DAsync(var, vp, 0xff, (size_t)w, h, ctx->stream);
    for (int hist = 0; hist < 2; hist++) {
        CRAWKDenoise k;
        CRAWKDenoiseIO io = {
            .src = mosaic, .src_pitch = mp, .dst = p->clean, .dst_pitch = p->clean_pitch,
            .lvl_prev = hist ? lvl : NULL, .lvl_next = hist ? lvl : NULL, .lvl_pitch = lp,
            .var_prev = hist ? var : NULL, .var_next = hist ? var : NULL, .var_pitch = vp,
        };
        float best = 1e30f;
        memset(&k, 0, sizeof(k));
        k.pw = (int32_t)(w / 2);
        k.ph = (int32_t)(h / 2);
        k.gat_a = 1e-3f; k.gat_c = 1e-6f; k.gat_sc = 1e-3f; k.gat_fwd = 2000.0f;
        k.gat_inv = 2.5e-4f; k.gat_off = 1e-3f; k.gat_t0 = 2.0f;
        k.inv_h2 = 1.0f; k.t_alpha = 0.8f; k.t_inv_h2 = 1.0f;
        k.guard_lo = 0.9f; k.guard_inv = 10.0f;
        for (int s4 = 0; s4 < 4; s4++) {
            k.black[s4] = 0.0f; k.inv_range[s4] = 16.0f; k.range[s4] = 0.0625f;
        }
        k.mode = CRAW_K_DN_SPATIAL | (hist ? CRAW_K_DN_TEMPORAL | CRAW_K_DN_HISTORY : 0);
        if (!need[hist])
            continue;
        for (int shape = 0; shape < CRAW_K_DN_SHAPE_NB; shape++) {
            float ms;
            if ((ret = time_denoise(p, &k, &io, shape, &ms)) < 0)
                goto done;
            if (ms < best) {
                best = ms;
                p->dn_shape[hist] = shape;
            }
        }
        craw_log(ctx, CRAW_LOG_VERBOSE, "autotune %ux%u %s: denoise shape %d, %.3f ms\n", w, h,
                 hist ? "temporal" : "spatial", p->dn_shape[hist], (double)best);
    }
    /* Another thread may have tuned the same size meanwhile: its shapes
     * win, so that every pipeline of the size agrees. */
    pthread_mutex_lock(&tune_lock);
    if (ret == 0 && (e = tune_entry(w, h, true))) {
        for (int hist = 0; hist < 2; hist++) {
            if (!want[hist])
                continue;
            if (e->known[hist]) {
                p->dn_shape[hist] = e->shape[hist];
            } else {
                e->shape[hist] = p->dn_shape[hist];
                e->known[hist] = true;
            }
        }
        e->live++;
        p->tune_held = true;
    }
    pthread_mutex_unlock(&tune_lock);
done:
    craw_dev_free(ctx, mosaic);
    craw_dev_free(ctx, lvl);
    craw_dev_free(ctx, var);
    if (craw_dev_sync(ctx) < 0 && ret == 0)
        ret = CRAW_ERROR(EIO);
    return ret;
}

CRAW_API int craw_pipeline_get_kernel_config(CRAWPipeline *p, int *denoise_shape,
                                             int *denoise_shape_history)
{
    if (!p)
        return CRAW_ERROR(EINVAL);
    if (denoise_shape)
        *denoise_shape = p->dn_shape[0];
    if (denoise_shape_history)
        *denoise_shape_history = p->dn_shape[1];
    return 0;
}

CRAW_API int craw_debug_kernel_errors(CRAWPipeline *p)
{
    uint32_t bits = 0;
    if (!p || !p->kerr)
        return CRAW_ERROR(EINVAL);
    cudaSetDevice(p->ctx->device);
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(&bits, p->kerr, sizeof(bits), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemset(p->kerr, 0, sizeof(bits)) != cudaSuccess)
        return CRAW_ERROR(EIO);
    return (int)bits;
}

CRAW_API int craw_debug_denoise_round_stats(CRAWPipeline *p, uint32_t counts[3], float *records,
                                            uint32_t max_records)
{
    uint32_t head[4];
    if (!p || !counts || (max_records && !records))
        return CRAW_ERROR(EINVAL);
    if (!p->round_stats)
        return CRAW_ERROR(ENOTSUP);
    cudaSetDevice(p->ctx->device);
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(head, p->round_stats, sizeof(head), cudaMemcpyDeviceToHost) != cudaSuccess)
        return CRAW_ERROR(EIO);
    counts[0] = head[0];
    counts[1] = head[1];
    counts[2] = head[3];
    uint32_t nr = CRAW_MIN(CRAW_MIN(head[2], (uint32_t)CRAW_K_ROUND_RECORDS), max_records);
    if (nr && cudaMemcpy(records, p->round_stats + 4, (size_t)nr * 16, cudaMemcpyDeviceToHost) != cudaSuccess)
        return CRAW_ERROR(EIO);
    if (cudaMemset(p->round_stats, 0, CRAW_K_ROUND_STATS_BYTES) != cudaSuccess)
        return CRAW_ERROR(EIO);
    return (int)nr;
}

CRAW_API int craw_pipeline_create(CRAWContext *ctx, const CRAWPipelineParams *params,
                                  CRAWPipeline **out)
{
    const uint32_t unsupported = CRAW_PIPELINE_FLAG_LENS | CRAW_PIPELINE_FLAG_FALSE_COLOR |
                                 CRAW_PIPELINE_FLAG_DEFRINGE | CRAW_PIPELINE_FLAG_SHARPEN;
    CRAWPipeline *p;
    uint32_t w, h;
    int ret;

    if (!ctx || !params || !out)
        return CRAW_ERROR(EINVAL);
    *out = NULL;
    if (params->cfa != CRAW_CFA_RGGB) {
        craw_log(ctx, CRAW_LOG_ERROR, "Only the RGGB CFA phase is implemented\n");
        return CRAW_ERROR(ENOTSUP);
    }
    if (params->flags & unsupported) {
        craw_log(ctx, CRAW_LOG_ERROR, "Pipeline flags 0x%x name stages this library does not "
                 "build (lens, false colour, defringe, sharpening)\n",
                 params->flags & unsupported);
        return CRAW_ERROR(ENOTSUP);
    }
    if ((params->flags & CRAW_PIPELINE_FLAG_HIGHLIGHT_RECONSTRUCTION) &&
        params->impl == CRAW_IMPL_PLAIN) {
        craw_log(ctx, CRAW_LOG_ERROR, "The plain pipeline has no highlight reconstruction\n");
        return CRAW_ERROR(ENOTSUP);
    }
    w = params->width;
    h = params->height;
    if (!w || !h || (w & 1) || (h & 1) || w < 8 || h < 8) {
        craw_log(ctx, CRAW_LOG_ERROR, "Invalid frame size %ux%u: both must be even and at least 8\n", w, h);
        return CRAW_ERROR(EINVAL);
    }
    if (w > 32768 || h > 32768) {
        craw_log(ctx, CRAW_LOG_ERROR, "Frame size %ux%u is larger than 32768 on a side\n", w, h);
        return CRAW_ERROR(EINVAL);
    }
    if (!craw_is_out_format(params->out_format)) {
        craw_log(ctx, CRAW_LOG_ERROR, "Output format must be RGBA16F, RGBA32F or RGB32F\n");
        return CRAW_ERROR(EINVAL);
    }
    if ((unsigned)params->debayer >= CRAW_DEBAYER_NB || (unsigned)params->out_space >= CRAW_CS_NB ||
        (unsigned)params->storage > CRAW_STORAGE_FP16 || (unsigned)params->impl > CRAW_IMPL_PLAIN ||
        params->nb_awb_slots > 4)
        return CRAW_ERROR(EINVAL);

    p = calloc(1, sizeof(*p));
    if (!p)
        return CRAW_ERROR(ENOMEM);
    p->ctx = ctx;
    p->params = *params;
    p->awb = params->flags & CRAW_PIPELINE_FLAG_AWB_HISTOGRAM;
    p->has_denoise = params->flags & CRAW_PIPELINE_FLAG_DENOISE;
    p->has_temporal = params->flags & CRAW_PIPELINE_FLAG_TEMPORAL_DENOISE;
    p->has_chroma = params->flags & CRAW_PIPELINE_FLAG_CHROMA_DENOISE;
    p->has_hl = params->flags & CRAW_PIPELINE_FLAG_HIGHLIGHT_RECONSTRUCTION;
    p->profile = params->flags & CRAW_PIPELINE_FLAG_PROFILE;
    p->keep = params->flags & CRAW_PIPELINE_FLAG_KEEP_INTERMEDIATE;
    p->plain = params->impl == CRAW_IMPL_PLAIN;
    p->fp16 = params->storage == CRAW_STORAGE_FP16 && !p->plain;
    p->tn_prev = p->tn_cur = -1;
    p->nb_slots = params->nb_awb_slots ? params->nb_awb_slots : 1;
    p->qw = (int)((w + 3) / 4);
    p->qh = (int)((h + 3) / 4);
    p->dn_shape[0] = p->dn_shape[1] = CRAW_K_DN_SHAPE_2x8;

    if ((p->has_denoise || p->has_temporal)) {
        /* The plane mirror holds for one reflection of the search + patch
         * radius (+1 for the temporal 3x3), reference pipeline.c:809-826. */
        uint32_t dn_min = 2 * (3 + 1 + 1 + (p->has_temporal ? 1 : 0));
        if (w < dn_min || h < dn_min) {
            craw_log(ctx, CRAW_LOG_ERROR, "Denoising needs a frame of at least %ux%u, got %ux%u\n",
                     dn_min, dn_min, w, h);
            free(p);
            return CRAW_ERROR(EINVAL);
        }
    }
    if (p->has_chroma && (w < 20 || h < 20)) {
        craw_log(ctx, CRAW_LOG_ERROR, "The chroma denoise needs a frame of at least 20x20\n");
        free(p);
        return CRAW_ERROR(EINVAL);
    }

    if ((ret = cudaSetDevice(ctx->device)) != cudaSuccess) {
        free(p);
        return CRAW_ERROR(EIO);
    }

    if (p->has_denoise || p->has_temporal)
        if ((ret = alloc_pitched(p, (void **)&p->clean, &p->clean_pitch, (size_t)w * 2, h)) < 0)
            goto fail;
    if (p->has_temporal) {
        for (int i = 0; i < 2; i++) {
            if ((ret = alloc_pitched(p, (void **)&p->lvl[i], &p->lvl_pitch, (size_t)w * 4, h)) < 0 ||
                (ret = alloc_pitched(p, (void **)&p->var[i], &p->var_pitch, (size_t)w, h)) < 0)
                goto fail;
        }
    }
    if (p->has_chroma || p->keep || p->plain) {
        size_t bpp = p->fp16 ? 8 : 16;
        if ((ret = alloc_pitched(p, &p->inter, &p->inter_pitch, (size_t)w * bpp, h)) < 0)
            goto fail;
    }
    if (p->has_hl) {
        /* The rebuilt mosaic (fp16) and the colour field's pyramid: 62 MB
         * at 5760x3240. */
        int64_t texels = craw_k_highlight_levels((int32_t)w, (int32_t)h, &p->hl);
        if (texels < 0) {
            ret = CRAW_ERROR(EINVAL);
            goto fail;
        }
        if ((ret = alloc_pitched(p, (void **)&p->hl_mosaic, &p->hl_pitch, (size_t)w * 2, h)) < 0 ||
            (ret = craw_dev_alloc(ctx, &p->hl_levels, (size_t)texels * 16)) < 0)
            goto fail;
    }
    if (p->has_chroma) {
        size_t bpp = p->fp16 ? 8 : 16;
        if (p->plain)
            bpp = 16;
        if ((ret = alloc_pitched(p, &p->q, &p->q_pitch, (size_t)p->qw * bpp, (uint32_t)p->qh)) < 0 ||
            (ret = alloc_pitched(p, &p->qf, NULL, (size_t)p->qw * bpp, (uint32_t)p->qh)) < 0)
            goto fail;
        if (p->plain)
            p->q_pitch = (size_t)p->qw * 16;   /* the plain kernels index densely */
    }
    if (p->awb) {
        p->nb_blocks = ((w + 7) / 8) * ((h + 7) / 8);
        if ((ret = craw_dev_alloc(ctx, (void **)&p->awb_rec, (size_t)p->nb_blocks * 8)) < 0 ||
            (ret = craw_dev_alloc(ctx, (void **)&p->awb_dev, HIST_BYTES)) < 0)
            goto fail;
        for (uint32_t i = 0; i < p->nb_slots; i++) {
            /* Room for every block, and at least for the part the slot's
             * async copy reads. */
            const size_t entries = CRAW_MAX((size_t)p->nb_blocks, (size_t)CRAW_K_AWB_DEFER_MAX);
            if ((ret = craw_dev_alloc(ctx, (void **)&p->slots[i].list,
                                      16 + entries * sizeof(CRAWKAwbDeferred))) < 0)
                goto fail;
            if (cudaHostAlloc((void **)&p->slots[i].host, SLOT_BYTES, cudaHostAllocDefault) != cudaSuccess) {
                ret = CRAW_ERROR(ENOMEM);
                goto fail;
            }
            memset(p->slots[i].host, 0, SLOT_BYTES);
        }
    }
    if ((ret = craw_dev_alloc(ctx, (void **)&p->kerr, 16)) < 0)
        goto fail;
    if (p->has_denoise && !p->plain && (params->flags & CRAW_PIPELINE_FLAG_EXACT_ROUNDING)) {
        /* The exact rounding: its marks (a bit per sample, 2.3 MB at
         * 5760x3240), its lists of the marked samples and of those its
         * float stage cannot settle (a sixteenth of the samples each: 9.8
         * MB), their counters and its statistics. */
        if ((ret = craw_dev_alloc(ctx, (void **)&p->round_flags,
                                  CRAW_K_ROUND_WORDS(w / 2, h / 2) * sizeof(uint32_t))) < 0 ||
            (ret = craw_dev_alloc(ctx, (void **)&p->round_stats, CRAW_K_ROUND_STATS_BYTES)) < 0 ||
            (ret = craw_dev_alloc(ctx, (void **)&p->round_list,
                                  (2 * CRAW_K_ROUND_LIST(w / 2, h / 2) + 4) * sizeof(uint32_t))) < 0)
            goto fail;
        if (cudaMemsetAsync(p->round_stats, 0, CRAW_K_ROUND_STATS_BYTES, ctx->stream) != cudaSuccess) {
            ret = CRAW_ERROR(EIO);
            goto fail;
        }
    }
    if (cudaMemsetAsync(p->kerr, 0, 16, ctx->stream) != cudaSuccess) {
        ret = CRAW_ERROR(EIO);
        goto fail;
    }
    if (p->plain) {
        size_t n = (size_t)w * h;
        if ((ret = craw_dev_alloc(ctx, (void **)&p->p_v, n * 4)) < 0)
            goto fail;
        if (params->debayer == CRAW_DEBAYER_RCD &&
            (ret = craw_dev_alloc(ctx, (void **)&p->p_scratch, 7 * n * 4)) < 0)
            goto fail;
        if (p->has_denoise || p->has_temporal) {
            if ((ret = craw_dev_alloc(ctx, (void **)&p->p_t, n * 4)) < 0 ||
                (ret = craw_dev_alloc(ctx, (void **)&p->p_var, 3 * n * 4)) < 0)
                goto fail;
        }
    }
    if (p->profile) {
        for (int s = 0; s < CRAW_PIPELINE_PROFILE_SLOTS; s++)
            for (int i = 0; i < MAX_STAGES; i++)
                for (int j = 0; j < 2; j++)
                    if (cudaEventCreate(&p->prof[s].ev[i][j]) != cudaSuccess) {
                        ret = CRAW_ERROR(ENOMEM);
                        goto fail;
                    }
    }
    if ((ret = craw_dev_sync(ctx)) < 0)
        goto fail;
    if (!p->plain && craw_k_develop_prepare(params->debayer) < 0) {
        ret = CRAW_ERROR(EIO);
        goto fail;
    }
    if (craw_forced_denoise_shape >= 0) {
        p->dn_shape[0] = p->dn_shape[1] = craw_forced_denoise_shape;
    } else if ((p->has_denoise || p->has_temporal) && !p->plain &&
               !(params->flags & CRAW_PIPELINE_FLAG_NO_AUTOTUNE) && (ret = autotune(p)) < 0) {
        goto fail;
    }
    craw_log(ctx, CRAW_LOG_VERBOSE, "pipeline %ux%u debayer %d flags 0x%x storage %s impl %s\n",
             w, h, params->debayer, params->flags, p->fp16 ? "fp16" : "fp32",
             p->plain ? "plain" : "fused");
    *out = p;
    return 0;
fail:
    craw_log(ctx, CRAW_LOG_ERROR, "Pipeline allocation failed (%d)\n", ret);
    release(p);
    return ret < 0 ? ret : CRAW_ERROR(ENOMEM);
}

CRAW_API void craw_pipeline_free(CRAWPipeline **pp)
{
    if (!pp || !*pp)
        return;
    release(*pp);
    *pp = NULL;
}

struct prof_ctx {
    CRAWPipeline *p;
    cudaStream_t s;
    struct prof_slot *slot;
};

static void prof_begin(struct prof_ctx *pc, int stage)
{
    if (!pc->slot || pc->slot->nb >= MAX_STAGES)
        return;
    pc->slot->stage[pc->slot->nb] = stage;
    cudaEventRecord(pc->slot->ev[pc->slot->nb][0], pc->s);
}

static void prof_end(struct prof_ctx *pc)
{
    if (!pc->slot || pc->slot->nb >= MAX_STAGES)
        return;
    cudaEventRecord(pc->slot->ev[pc->slot->nb][1], pc->s);
    pc->slot->nb++;
}

CRAW_API int craw_pipeline_record(CRAWPipeline *p, cudaStream_t s, const CRAWImage *src,
                                  const CRAWImage *dst, const CRAWFrameParams *fp)
{
    CRAWContext *ctx;
    CRAWKDevelop dk;
    CRAWKDevelopIO dio;
    CRAWKDenoise dnk;
    CRAWKDenoiseExact dnx;
    CRAWKRound rd = { 0 };
    bool exact = false;
    CRAWKChroma ck;
    struct prof_ctx pc = { 0 };
    bool spatial, temporal, replay, denoise, chroma;
    int t_read, t_write, dn_mode = 0, ret;
    const uint16_t *mosaic;
    size_t mosaic_pitch;
    uint32_t w, h;

    if (!p || !src || !dst || !fp || !fp->profile)
        return CRAW_ERROR(EINVAL);
    ctx = p->ctx;
    w = p->params.width;
    h = p->params.height;
    if ((ret = craw_image_check(ctx, src, CRAW_FORMAT_R16_UNORM, w, h, "Source")) < 0 ||
        (ret = craw_image_check(ctx, dst, p->params.out_format, w, h, "Destination")) < 0)
        return ret;
    if (craw_images_overlap(src, dst)) {
        craw_log(ctx, CRAW_LOG_ERROR, "Source and destination must not alias\n");
        return CRAW_ERROR(EINVAL);
    }
    if ((ret = craw_develop_consts(ctx, w, h, p->params.debayer, p->fp16, p->params.out_space, fp,
                                   &dk)) < 0)
        return ret;

    /* Filters on or off for this frame, and the temporal sets (reference
     * pipeline.c:1785-1818): a replay reads what the last recording read
     * and rewrites what it wrote; a reset reads nothing. */
    spatial = p->has_denoise && fp->denoise_strength > 0.0f;
    temporal = p->has_temporal && fp->denoise_temporal_strength > 0.0f;
    if (temporal && !(fp->denoise_temporal_strength <= 1.0f)) {
        craw_log(ctx, CRAW_LOG_ERROR, "denoise_temporal_strength = %g; at most 1.0\n",
                 (double)fp->denoise_temporal_strength);
        return CRAW_ERROR(EINVAL);
    }
    replay = fp->denoise_temporal_replay;
    t_read = replay ? p->tn_prev : p->tn_cur;
    if (fp->flags & CRAW_FRAME_FLAG_TEMPORAL_RESET)
        t_read = -1;
    t_write = -1;
    if (temporal)
        t_write = replay && p->tn_cur >= 0 ? p->tn_cur : (t_read == 0 ? 1 : 0);
    denoise = spatial || temporal;
    if (denoise) {
        dn_mode = (spatial ? CRAW_K_DN_SPATIAL : 0) | (temporal ? CRAW_K_DN_TEMPORAL : 0) |
                  (temporal && t_read >= 0 ? CRAW_K_DN_HISTORY : 0);
        /* The exact rounding of the codes: the spatial filter without a
         * temporal history (the other modes round as the float path does). */
        exact = !p->plain && p->round_flags && dn_mode == CRAW_K_DN_SPATIAL && craw_round_scale > 0.0f;
        if ((ret = craw_denoise_consts(ctx, w, h, fp, dn_mode, &dnk, exact ? &dnx : NULL)) < 0)
            return ret;
        if (exact) {
            craw_denoise_round_band(&dnk, craw_round_scale, &rd);
            rd.flags = p->round_flags;
            rd.count2 = p->round_list + 2 * CRAW_K_ROUND_LIST(w / 2, h / 2);
        }
    }

    chroma = p->has_chroma && fp->denoise_chroma_strength > 0.0f;
    if (chroma && !(fp->denoise_chroma_strength <= 1.0f)) {
        craw_log(ctx, CRAW_LOG_ERROR, "denoise_chroma_strength = %g; at most 1.0\n",
                 (double)fp->denoise_chroma_strength);
        return CRAW_ERROR(EINVAL);
    }

    /* Nothing can fail on the host from here on. */
    if (p->profile) {
        pc.p = p;
        pc.s = s;
        pc.slot = &p->prof[p->prof_recorded % CRAW_PIPELINE_PROFILE_SLOTS];
        pc.slot->nb = 0;
    }

    uint8_t *awb_hist = NULL;
    CRAWKAwbOut awb = { 0 };
    if (p->awb) {
        uint8_t *list = p->slots[p->nb_recorded % p->nb_slots].list;
        awb_hist = p->awb_dev;
        awb.rec = p->plain ? NULL : p->awb_rec;
        awb.deferred = (CRAWKAwbDeferred *)(list + 16);
        awb.nb_deferred = (uint32_t *)list;
        if (cudaMemsetAsync(awb_hist, 0, HIST_BYTES, s) != cudaSuccess ||
            cudaMemsetAsync(awb.nb_deferred, 0, 4, s) != cudaSuccess)
            return CRAW_ERROR(EIO);
    }

    mosaic = src->data;
    mosaic_pitch = src->pitch;
    if (denoise) {
        CRAWKDenoiseIO io = {
            .src = src->data, .src_pitch = src->pitch,
            .dst = p->clean, .dst_pitch = p->clean_pitch,
            .lvl_pitch = p->lvl_pitch, .var_pitch = p->var_pitch,
        };
        if (temporal) {
            if (t_read >= 0) {
                io.lvl_prev = p->lvl[t_read];
                io.var_prev = p->var[t_read];
            }
            io.lvl_next = p->lvl[t_write];
            io.var_next = p->var[t_write];
        }
        prof_begin(&pc, ST_DENOISE);
        ret = p->plain ? craw_k_plain_denoise(&dnk, &io, p->p_t, p->p_var, s)
                       : craw_k_denoise(&dnk, &io, p->dn_shape[(dn_mode & CRAW_K_DN_HISTORY) != 0],
                                        exact ? &rd : NULL, p->kerr, s);
        prof_end(&pc);
        if (ret < 0)
            goto launch_fail;
        if (exact) {
            prof_begin(&pc, ST_ROUND);
            ret = craw_k_denoise_round(&dnk, &dnx, &io, &rd, p->round_list, p->round_stats, ctx->sm_count, s);
            prof_end(&pc);
            if (ret < 0)
                goto launch_fail;
        }
        mosaic = p->clean;
        mosaic_pitch = p->clean_pitch;
    }

    memset(&dio, 0, sizeof(dio));
    dio.src = mosaic;
    dio.src_pitch = mosaic_pitch;
    dio.awb = awb;
    dio.err = p->kerr;

    /* Highlight reconstruction (reference pipeline.c:2047-2062): the
     * rebuilt, balanced fp16 mosaic replaces the one the debayer reads, and
     * the debayer's prep becomes the identity with no clip. */
    if (p->has_hl && (fp->flags & CRAW_FRAME_FLAG_HIGHLIGHT_RECONSTRUCTION)) {
        CRAWKHighlight hk = p->hl;
        CRAWKHighlightIO hio = {
            .src = mosaic, .src_pitch = mosaic_pitch,
            .dst = p->hl_mosaic, .dst_pitch = p->hl_pitch,
            .levels = p->hl_levels, .err = p->kerr,
        };
        hk.width = (int32_t)w;
        hk.height = (int32_t)h;
        for (int i = 0; i < 4; i++) {
            hk.black[i] = dk.black[i];
            hk.inv_range[i] = dk.inv_range[i];
        }
        hk.wb[0] = dk.wbs[0];
        hk.wb[1] = dk.wbs[1];
        hk.wb[2] = dk.wbs[3];
        prof_begin(&pc, ST_HL);
        ret = craw_k_highlights(&hk, &hio, s);
        prof_end(&pc);
        if (ret < 0)
            goto launch_fail;
        dio.src = p->hl_mosaic;
        dio.src_pitch = p->hl_pitch;
        dio.src_f16 = 1;
        for (int i = 0; i < 4; i++) {
            dk.black[i] = 0.0f;
            dk.inv_range[i] = 1.0f;
            dk.wbs[i] = 1.0f;
        }
        dk.clip = FLT_MAX;
    }
    memset(&ck, 0, sizeof(ck));
    ck.width = (int32_t)w;
    ck.height = (int32_t)h;
    ck.qw = p->qw;
    ck.qh = p->qh;
    ck.strength = fp->denoise_chroma_strength;
    ck.fp16 = p->fp16;
    ck.err = p->kerr;

    if (p->plain) {
        dio.dst = dst->data;
        dio.dst_pitch = dst->pitch;
        dio.dst_fmt = craw_out_layout(dst->format);
        prof_begin(&pc, ST_DEVELOP);
        ret = craw_k_plain_develop(&dk, &dio, chroma ? &ck : NULL, p->p_v, p->inter, p->inter_pitch,
                                   p->p_scratch, p->q, p->qf, p->awb ? (uint32_t *)awb_hist : NULL, s);
        prof_end(&pc);
        if (ret < 0)
            goto launch_fail;
    } else if (!chroma) {
        dio.dst = dst->data;
        dio.dst_pitch = dst->pitch;
        dio.dst_fmt = craw_out_layout(dst->format);
        if (p->keep) {
            dio.inter = p->inter;
            dio.inter_pitch = p->inter_pitch;
        }
        prof_begin(&pc, ST_DEVELOP);
        ret = craw_k_develop(&dk, &dio, p->dev_shape, s);
        prof_end(&pc);
        if (ret < 0)
            goto launch_fail;
    } else {
        CRAWKAwbOut none = { 0 };
        dio.inter = p->inter;
        dio.inter_pitch = p->inter_pitch;
        dio.quarter = p->q;
        dio.quarter_pitch = p->q_pitch;
        dio.awb = none;
        prof_begin(&pc, ST_DEVELOP);
        ret = craw_k_develop(&dk, &dio, p->dev_shape, s);
        prof_end(&pc);
        if (ret < 0)
            goto launch_fail;
        prof_begin(&pc, ST_BLUR);
        ret = craw_k_chroma_blur(&ck, p->q, p->q_pitch, p->qf, p->q_pitch, s);
        prof_end(&pc);
        if (ret < 0)
            goto launch_fail;
        prof_begin(&pc, ST_UP);
        ret = craw_k_chroma_up_color(&dk, &ck, p->inter, p->inter_pitch, p->q, p->qf, p->q_pitch,
                                     dst->data, dst->pitch, craw_out_layout(dst->format),
                                     p->keep ? p->inter : NULL, &awb, s);
        prof_end(&pc);
        if (ret < 0)
            goto launch_fail;
    }

    if (p->awb) {
        struct awb_slot *slot = &p->slots[p->nb_recorded % p->nb_slots];
        if (!p->plain) {
            prof_begin(&pc, ST_AWB);
            ret = craw_k_awb_reduce(p->awb_rec, p->nb_blocks, (uint32_t *)awb_hist, s);
            prof_end(&pc);
            if (ret < 0)
                goto launch_fail;
        }
        if (cudaMemcpyAsync(slot->host, p->awb_dev, HIST_BYTES, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaMemcpyAsync(slot->host + HIST_BYTES, slot->list, 16 + DEFER_BYTES, cudaMemcpyDeviceToHost,
                            s) != cudaSuccess) {
            ret = CRAW_ERROR(EIO);
            goto launch_fail;
        }
        slot->folded = false;
        p->nb_recorded++;
    }
    if (p->profile)
        p->prof_recorded++;
    p->last_denoised = denoise;
    p->last_hl = dio.src_f16;

    /* Only now does the temporal state move (reference pipeline.c:2303-2313). */
    if (p->has_temporal) {
        p->tn_prev = t_read;
        if (temporal)
            p->tn_cur = t_write;
        else if (!replay)
            p->tn_cur = -1;
    }
    return 0;

launch_fail:
    /* A launch CUDA refused: the stream may hold part of this recording,
     * so the temporal state is forgotten rather than trusted. */
    craw_log(ctx, CRAW_LOG_ERROR, "Kernel launch failed (%s)\n", cudaGetErrorString(cudaPeekAtLastError()));
    p->tn_prev = p->tn_cur = -1;
    return CRAW_ERROR(EIO);
}

CRAW_API int craw_pipeline_get_awb_histogram_n(CRAWPipeline *p, uint32_t frames_back,
                                               CRAWAwbHistogram *out)
{
    struct awb_slot *slot;
    uint32_t *hist;

    if (!p || !out)
        return CRAW_ERROR(EINVAL);
    if (!p->awb) {
        craw_log(p->ctx, CRAW_LOG_ERROR, "Pipeline was created without CRAW_PIPELINE_FLAG_AWB_HISTOGRAM\n");
        return CRAW_ERROR(EINVAL);
    }
    if (frames_back >= p->nb_slots || frames_back >= p->nb_recorded)
        return CRAW_ERROR(EINVAL);
    slot = &p->slots[(p->nb_recorded - 1 - frames_back) % p->nb_slots];
    hist = (uint32_t *)slot->host;
    if (!slot->folded) {
        /* Bin the blocks the device deferred, with this host's logf: the
         * first CRAW_K_AWB_DEFER_MAX came with the slot, the rest (a frame
         * with that many blocks on bin edges) are read from the slot's
         * device list now. */
        const CRAWKAwbDeferred *d = (const CRAWKAwbDeferred *)(slot->host + HIST_BYTES + 16);
        const uint32_t nd = *(const uint32_t *)(slot->host + HIST_BYTES);
        const uint32_t nd0 = CRAW_MIN(nd, (uint32_t)CRAW_K_AWB_DEFER_MAX);
        for (uint32_t i = 0; i < nd0; i++)
            craw_awb_bin_host(d[i].rr, d[i].bb, d[i].g, hist, hist + HIST_N, hist + 2 * HIST_N);
        if (nd > nd0) {
            CRAWKAwbDeferred *rest = malloc((size_t)(nd - nd0) * sizeof(*rest));
            if (!rest)
                return CRAW_ERROR(ENOMEM);
            cudaSetDevice(p->ctx->device);
            if (cudaMemcpy(rest, slot->list + 16 + (size_t)nd0 * sizeof(*rest), (size_t)(nd - nd0) * sizeof(*rest),
                           cudaMemcpyDeviceToHost) != cudaSuccess) {
                free(rest);
                return CRAW_ERROR(EIO);
            }
            for (uint32_t i = 0; i < nd - nd0; i++)
                craw_awb_bin_host(rest[i].rr, rest[i].bb, rest[i].g, hist, hist + HIST_N, hist + 2 * HIST_N);
            free(rest);
        }
        slot->folded = true;
    }
    out->bins = CRAW_AWB_HIST_BINS;
    out->log_min = CRAW_AWB_HIST_LOG_MIN;
    out->log_max = CRAW_AWB_HIST_LOG_MAX;
    out->count = hist;
    out->weight = hist + HIST_N;
    out->weight_bright = hist + 2 * HIST_N;
    return 0;
}

CRAW_API int craw_pipeline_get_awb_histogram(CRAWPipeline *p, CRAWAwbHistogram *out)
{
    return craw_pipeline_get_awb_histogram_n(p, 0, out);
}

CRAW_API int craw_pipeline_get_stage_times_n(CRAWPipeline *p, uint32_t frames_back,
                                             CRAWStageTime *out, uint32_t max)
{
    struct prof_slot *slot;
    uint32_t nb_agg = 0;

    if (!p || (max && !out))
        return CRAW_ERROR(EINVAL);
    if (!p->profile) {
        craw_log(p->ctx, CRAW_LOG_ERROR, "Pipeline was created without CRAW_PIPELINE_FLAG_PROFILE\n");
        return CRAW_ERROR(EINVAL);
    }
    if (frames_back >= CRAW_PIPELINE_PROFILE_SLOTS || frames_back >= p->prof_recorded)
        return CRAW_ERROR(EINVAL);
    slot = &p->prof[(p->prof_recorded - 1 - frames_back) % CRAW_PIPELINE_PROFILE_SLOTS];
    if (!slot->nb)
        return 0;
    /* Never blocks: a recording still in flight is EAGAIN. */
    for (uint32_t i = 0; i < slot->nb; i++) {
        cudaError_t e = cudaEventQuery(slot->ev[i][1]);
        if (e == cudaErrorNotReady)
            return CRAW_ERROR(EAGAIN);
        if (e != cudaSuccess)
            return CRAW_ERROR(EIO);
    }
    for (uint32_t i = 0; i < slot->nb; i++) {
        const char *name = (p->plain ? plain_stage_names : stage_names)[slot->stage[i]];
        float ms = 0.0f;
        uint32_t j;
        cudaEventElapsedTime(&ms, slot->ev[i][0], slot->ev[i][1]);
        for (j = 0; j < nb_agg; j++)
            if (!strcmp(p->prof_agg[j].name, name))
                break;
        if (j == nb_agg)
            p->prof_agg[nb_agg++] = (CRAWStageTime) { .name = name };
        p->prof_agg[j].count++;
        p->prof_agg[j].ms += ms;
    }
    if (max)
        memcpy(out, p->prof_agg, CRAW_MIN(max, nb_agg) * sizeof(*out));
    return (int)nb_agg;
}

CRAW_API int craw_pipeline_get_stage_times(CRAWPipeline *p, CRAWStageTime *out, uint32_t max)
{
    return craw_pipeline_get_stage_times_n(p, 0, out, max);
}

CRAW_API int craw_pipeline_get_intermediate(CRAWPipeline *p, CRAWImage *rgb, CRAWImage *mosaic)
{
    if (!p || !p->keep)
        return CRAW_ERROR(EINVAL);
    if (rgb) {
        rgb->data = p->inter;
        rgb->pitch = p->inter_pitch;
        rgb->format = p->fp16 ? CRAW_FORMAT_RGBA16F : CRAW_FORMAT_RGBA32F;
        rgb->width = p->params.width;
        rgb->height = p->params.height;
    }
    if (mosaic) {
        mosaic->data = p->last_hl ? (void *)p->hl_mosaic : (p->last_denoised ? p->clean : NULL);
        mosaic->pitch = p->last_hl ? p->hl_pitch : p->clean_pitch;
        mosaic->format = p->last_hl ? CRAW_FORMAT_R16F : CRAW_FORMAT_R16_UNORM;
        mosaic->width = p->params.width;
        mosaic->height = p->params.height;
    }
    return 0;
}

CRAW_API int craw_pipeline_get_temporal_state(CRAWPipeline *p, CRAWImage *level, CRAWImage *sqrt_var)
{
    if (!p || !p->has_temporal)
        return CRAW_ERROR(EINVAL);
    if (p->tn_cur < 0)
        return CRAW_ERROR(EAGAIN);
    if (level) {
        level->data = p->lvl[p->tn_cur];
        level->pitch = p->lvl_pitch;
        level->format = (CRAWFormat)0;
        level->width = p->params.width;
        level->height = p->params.height;
    }
    if (sqrt_var) {
        sqrt_var->data = p->var[p->tn_cur];
        sqrt_var->pitch = p->var_pitch;
        sqrt_var->format = (CRAWFormat)0;
        sqrt_var->width = p->params.width;
        sqrt_var->height = p->params.height;
    }
    return 0;
}
