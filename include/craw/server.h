/*
 * craw-gb300: a frame server (extension, no counterpart in the reference,
 * whose callers drive one pipeline per clip themselves).
 *
 * A server develops frames of many streams - clips and stills of different
 * sizes - as they arrive. Each stream owns a pipeline (its temporal
 * denoise state stays resident on the device between frames), a CUDA
 * stream, and a few device staging slots for its input mosaic and output
 * image; it may also keep an AWB illuminant track. Streams are admitted
 * against a device-memory budget: opening one that does not fit next to
 * the streams already open fails with CRAW_ERROR(EAGAIN) (or ENOSPC when
 * it would not fit in an empty server) and nothing of it stays allocated.
 *
 * Frames are submitted from host memory (pinned memory lets the copies
 * overlap the kernels) and queued. A worker thread launches every queued
 * frame whose stream has a free slot while fewer than max_inflight frames
 * are on the device: copy in, craw_pipeline_record(), copy out, all on
 * the stream's CUDA stream. Frames of different streams run concurrently
 * on the GPU, and a frame that arrives while others are in flight starts
 * as soon as a slot frees up. A stream's frames start and finish in
 * submission order. Results (latency, device time, status, AWB track) are
 * collected with craw_server_poll().
 *
 * All functions are thread safe. A stream whose producer stops submitting
 * for longer than idle_timeout_ms with nothing in flight is closed by the
 * server and its memory returned to the budget (a dead producer cannot
 * hold device memory forever).
 */
#ifndef CRAW_SERVER_H
#define CRAW_SERVER_H

#include <craw/awb.h>
#include <craw/pipeline.h>

typedef struct CRAWServer CRAWServer;

typedef struct CRAWServerParams {
    uint64_t hbm_budget;           /* bytes the open streams may hold on the device */
    uint32_t max_inflight;         /* frames on the device at once; 0: 32 */
    uint32_t slots_per_stream;     /* staging slots (frames in flight) per stream; 0: 2 */
    uint32_t idle_timeout_ms;      /* 0: streams are only closed by their owner */
    uint32_t max_queued;           /* frames a stream may have waiting for the device;
                                    * a submit beyond it returns EAGAIN at once (the
                                    * producer polls and submits again); 0: no limit */
    uint8_t padding[64 - 24];
} CRAWServerParams;

/* Stream flags. */
/* Keep an AWB illuminant track: after each frame the worker reads the
 * frame's histogram, estimates its illuminant with the frame's profile
 * (craw_awb_estimate), pushes it into the stream's smoother at the frame's
 * pts, and develops the stream's next frame with CRAW_WB_REBALANCE at the
 * track. Needs CRAW_PIPELINE_FLAG_AWB_HISTOGRAM and a profile with a white
 * balance table; the stream's frames then run one at a time. */
#define CRAW_SERVER_STREAM_AUTO_WB (1u << 0)
/* A stream without a noise model: its first frame's model is measured on
 * the device (craw_noise_estimate_cuda on the staged mosaic, default
 * options, before the frame develops) and is the noise override of every
 * frame of the stream that carries none (noise_override.a <= 0). The
 * first frame's result carries the estimate (noise_valid). A frame whose
 * estimate fails (too few levels) fails with that error and the next frame
 * tries again. The estimate's scratch (6 bytes a sample, freed at once)
 * comes from the device's default memory pool, outside the budget. Needs
 * CRAW_PIPELINE_FLAG_DENOISE or CRAW_PIPELINE_FLAG_TEMPORAL_DENOISE. */
#define CRAW_SERVER_STREAM_ESTIMATE_NOISE (1u << 1)

typedef struct CRAWServerStreamParams {
    CRAWPipelineParams pipeline;   /* frame size, debayer, output, stages */
    uint32_t flags;                /* CRAW_SERVER_STREAM_* */
    CRAWAwbParams awb;             /* estimator, with AUTO_WB */
    CRAWAwbSmootherParams smoother;
    float deadline_ms;             /* the latency a frame of the stream should meet (its
                                    * frame interval, say): waiting frames launch earliest
                                    * deadline first; 0: none (best effort, after every
                                    * stream with one) */
    uint8_t padding[60];
} CRAWServerStreamParams;

typedef struct CRAWServerResult {
    uint64_t user;                 /* as submitted */
    uint32_t stream;
    int status;                    /* 0, or the negative errno of the failed step */
    double queue_ms;               /* submission to launch (host clock) */
    double latency_ms;             /* submission to the result being ready in dst */
    double device_ms;              /* copy in + develop + copy out on the device */
    bool awb_valid;                /* AUTO_WB: the track after this frame */
    CRAWIlluminant awb;
    CRAWAwbEstimate estimate;      /* AUTO_WB: this frame's own reading */
    bool noise_valid;              /* ESTIMATE_NOISE: measured on this frame */
    CRAWNoiseEstimate noise;
} CRAWServerResult;

typedef struct CRAWServerStats {
    uint64_t hbm_budget, hbm_resident;   /* bytes */
    uint32_t streams, queued, inflight;
    uint64_t submitted, completed, failed;
    uint64_t streams_admitted, streams_refused, streams_reclaimed;
    uint64_t submits_refused;            /* EAGAIN: the stream's queue was full */
} CRAWServerStats;

CRAW_API void craw_server_params_init(CRAWServerParams *p);
CRAW_API void craw_server_stream_params_init(CRAWServerStreamParams *p);

/* Creates a server on `ctx`'s device with its own context (so that its
 * memory accounting sees only its streams) and starts its worker. */
CRAW_API int craw_server_create(CRAWContext *ctx, const CRAWServerParams *params, CRAWServer **out);

/* Stops the worker after every submitted frame has finished, closes every
 * stream and frees the server. Results not polled are dropped. */
CRAW_API void craw_server_free(CRAWServer **s);

/* Admits a stream: creates its pipeline, CUDA stream and staging slots and
 * charges their device memory to the budget. CRAW_ERROR(EAGAIN) when the
 * stream does not fit beside the open ones, CRAW_ERROR(ENOSPC) when it
 * would not fit alone; pipeline creation errors as craw_pipeline_create(). */
CRAW_API int craw_server_stream_open(CRAWServer *s, const CRAWServerStreamParams *params,
                                     uint32_t *stream_id);

/* Closes a stream once its submitted frames are done (their results are
 * still delivered) and returns its memory to the budget. */
CRAW_API int craw_server_stream_close(CRAWServer *s, uint32_t stream_id);

/* Queues one frame of a stream: `src` is the R16 mosaic in host memory
 * (pitch in bytes), `dst` receives the developed image in the stream's
 * output format; both must stay valid until the frame's result is polled.
 * `fp` is copied (its profile must outlive the frame). `pts` is the
 * presentation time in seconds (AWB track). Returns at once;
 * CRAW_ERROR(ENOENT) for a stream that is not open, CRAW_ERROR(EAGAIN)
 * when the stream already has max_queued frames waiting (nothing is
 * queued: poll for results and submit again). */
CRAW_API int craw_server_submit(CRAWServer *s, uint32_t stream_id, const void *src,
                                size_t src_pitch, void *dst, size_t dst_pitch,
                                const CRAWFrameParams *fp, double pts, uint64_t user);

/* Up to `max` finished frames, oldest first; waits up to timeout_ms (0:
 * not at all, negative: until one arrives) when none is ready. Returns
 * their number. */
CRAW_API int craw_server_poll(CRAWServer *s, CRAWServerResult *out, uint32_t max, int timeout_ms);

/* Blocks until nothing is queued or in flight. */
CRAW_API int craw_server_drain(CRAWServer *s);

CRAW_API int craw_server_get_stats(CRAWServer *s, CRAWServerStats *out);

#endif /* CRAW_SERVER_H */
