/*
 * craw-gb300: batched development (extension, no counterpart in the
 * reference, which develops one frame per recording).
 *
 * A batch develops up to max_frames independent frames of different sizes
 * in persistent launches: every denoise tile of every frame, then every
 * develop tile of every frame. The launches are captured into a CUDA
 * graph the first time a set of frame shapes is seen and replayed for
 * every later recording with the same shapes; each replay gets the
 * recording's per-frame constants as new parameters of the captured
 * kernel nodes (the table travels with the launch). Frames of at least
 * direct_pixels pixels run the single-frame kernels instead, after them.
 * Frames of a batch have no temporal history and no AWB histogram.
 */
#ifndef CRAW_BATCH_H
#define CRAW_BATCH_H

#include <craw/pipeline.h>

typedef struct CRAWBatch CRAWBatch;

/* The persistent part runs as two launches (every denoise tile, then every
 * develop tile) by default: measured faster than one launch with a
 * grid-wide barrier, which carries the denoise phase's registers into the
 * develop phase and halves its occupancy. CRAW_BATCH_FLAG_FUSED asks for the
 * one launch; CRAW_BATCH_FLAG_UNFUSED names the default. */
#define CRAW_BATCH_FLAG_UNFUSED  (1u << 20)
#define CRAW_BATCH_FLAG_FUSED    (1u << 22)
/* Launch directly on every recording instead of replaying a CUDA graph. */
#define CRAW_BATCH_FLAG_NO_GRAPH (1u << 21)

typedef struct CRAWBatchParams {
    uint32_t max_frames;             /* frames one recording may carry, 1..64 */
    uint32_t max_width, max_height;  /* the largest frame (even) */
    enum CRAWDebayer debayer;        /* all frames of a batch */
    enum CRAWColorSpace out_space;   /* default; a frame may override it */
    CRAWFormat out_format;           /* CRAW_FORMAT_RGBA16F, CRAW_FORMAT_RGBA32F or RGB32F */
    uint32_t flags;                  /* CRAW_PIPELINE_FLAG_DENOISE, CRAW_BATCH_FLAG_* */
    /* Frames of at least this many pixels are developed by the single-frame
     * kernels, launched one frame after another on the recording's stream
     * after the persistent launch of the others: on frames that large the
     * persistent kernel's per-tile cost is higher and its saved launches
     * worth nothing. 0: CRAW_BATCH_DIRECT_PIXELS; UINT32_MAX: every frame in
     * the persistent launch. */
    uint32_t direct_pixels;
    uint8_t padding[64 - 8 * 4];
} CRAWBatchParams;

#define CRAW_BATCH_DIRECT_PIXELS 4000000u

typedef struct CRAWBatchInfo {
    int denoise_shape;               /* the autotuned tile shape: 0 = 2x4, 1 = 2x8 */
    int fused;                       /* one launch with a grid barrier */
    int graph;                       /* recordings replay a captured graph */
    uint64_t captures, replays;      /* graphs captured, replays launched */
    int direct_shape;                /* the single-frame denoise shape of direct frames
                                      * (craw_pipeline_get_kernel_config's numbering), -1: none */
    uint64_t direct_frames;          /* frames developed by the single-frame kernels */
} CRAWBatchInfo;

CRAW_API void craw_batch_params_init(CRAWBatchParams *p);

/* Allocates a denoised-mosaic buffer per frame slot, the constant table,
 * and times the denoise tile shapes on a max_width x max_height scratch
 * frame to pick the faster. */
CRAW_API int craw_batch_create(CRAWContext *ctx, const CRAWBatchParams *params, CRAWBatch **out);

/* Enqueues the development of `nb_frames` frames on `stream`: src[i]
 * (R16_UNORM) -> dst[i] (out_format) with the settings fp[i] (the denoise
 * strength and noise model, white balance, exposure, output space and
 * their flags; temporal and chroma settings are ignored). Every frame is
 * checked as craw_pipeline_record() checks it; a failed recording
 * enqueues nothing. Recordings of one batch must be ordered (one stream,
 * or events). */
CRAW_API int craw_batch_record(CRAWBatch *b, cudaStream_t stream, uint32_t nb_frames,
                               const CRAWImage *src, const CRAWImage *dst,
                               const CRAWFrameParams *fp);

CRAW_API int craw_batch_get_info(CRAWBatch *b, CRAWBatchInfo *info);

CRAW_API void craw_batch_free(CRAWBatch **b);

#endif /* CRAW_BATCH_H */
