/*
 * craw-gb300: auto white balance histogram and its CPU builder
 * (reference include/craw/awb.h).
 *
 * The GPU reduces each frame to a 2D histogram of raw chromaticity with
 * three counters per bin; the host reads it back, estimates the frame's
 * illuminant from it (craw_awb_estimate) and smooths the estimates of a
 * stream into a track (craw_awb_smoother_*).
 */
#ifndef CRAW_AWB_H
#define CRAW_AWB_H

#include <stdint.h>
#include <stdbool.h>

#include <cuda_runtime_api.h>

#include <craw/profile.h>

/* Histogram geometry, as the reference's (awb.h:38-40). */
#define CRAW_AWB_HIST_BINS     128
#define CRAW_AWB_HIST_LOG_MIN -2.5f
#define CRAW_AWB_HIST_LOG_MAX  1.0f

/* Histogram over ln(R/G) (x) and ln(B/G) (y) of the raw response (the
 * applied white balance divided back out), one sample per 8x8 block mean,
 * clipped (max >= 0.98) and near-black (g < 0.002) blocks left out;
 * index = iy * bins + ix. Reference awb.h:45-56. */
typedef struct CRAWAwbHistogram {
    uint32_t bins;
    float log_min, log_max;
    const uint32_t *count;          /* samples per bin */
    const uint32_t *weight;         /* sum of min(g, 0.5), 16.16 fixed point */
    const uint32_t *weight_bright;  /* sum of g^4, 16.16 fixed point */
} CRAWAwbHistogram;

/* CPU builder with the GPU pass's semantics: `rgb` is interleaved float
 * camera RGB after the prep (white balance `wb_applied`, clip at 1.0),
 * `stride` floats between rows, `channels` 3 or 4. The three arrays hold
 * CRAW_AWB_HIST_BINS^2 entries each and are zeroed first. Blocks hanging
 * over the right or bottom edge average the pixels that exist. Reference
 * awb.h:135-139 (lib/awb.c:213-296). */
CRAW_API int craw_awb_histogram_from_rgb(const float *rgb, uint32_t width,
                                         uint32_t height, size_t stride,
                                         int channels, const float wb_applied[3],
                                         uint32_t *count, uint32_t *weight,
                                         uint32_t *weight_bright);

/* ----------------------------------------------------------- estimator */

/* Parameters of craw_awb_estimate(), the reference's (awb.h:62-89). */
typedef struct CRAWAwbParams {
    float band;                     /* neutral band around the locus, ln-ratio units; 0.08 */
    float sigma;                    /* Gaussian falloff of a bin's weight with its distance; 0.05 */
    float min_zone_fraction;        /* share of the mass inside the band below which the
                                     * reading is invalid; 0.02 */
    float ambience;                 /* 0: correct fully; 1: keep the warmth below the knee */
    float ambience_knee_cct;        /* 4000 */
    float cct_min, cct_max;         /* clamps of the reported cct; 0: the table's range */
    bool prefer_bright;             /* take the g^4 reading when it is valid; true */
    float bright_max_spread_mired;  /* the g^4 reading's spread limit along the locus; 60 */
} CRAWAwbParams;

CRAW_API void craw_awb_params_init(CRAWAwbParams *p);

/* One reading of the histogram under one weighting. */
typedef struct CRAWAwbCandidate {
    bool valid;
    CRAWIlluminant illuminant;      /* before ambience and clamping */
    float in_zone_fraction;         /* share of the weighting's mass inside the band */
    float spread_mired;             /* weighted standard deviation along the locus */
} CRAWAwbCandidate;

enum CRAWAwbSource {
    CRAW_AWB_SOURCE_NONE = 0,
    CRAW_AWB_SOURCE_ZONE,           /* the min(g, 0.5) weighted neutral bins */
    CRAW_AWB_SOURCE_BRIGHT,         /* the g^4 weighted ones */
};

typedef struct CRAWAwbEstimate {
    bool valid;
    CRAWIlluminant illuminant;      /* the chosen reading after ambience and clamping */
    float confidence;               /* 0..1, from the in-band share and the spread */
    float in_zone_fraction;
    float spread_mired;
    enum CRAWAwbSource source;
    CRAWAwbCandidate zone, bright;
} CRAWAwbEstimate;

/* The illuminant of one frame from its histogram (a pipeline's
 * craw_pipeline_get_awb_histogram()): every occupied bin centre is taken as
 * a neutral, placed on the profile's locus, and weighted by its two
 * counters and a Gaussian of its distance from the locus; the in-band
 * weighted means give two readings, of which the bright one wins when it
 * is valid and preferred. `params` NULL means the defaults. Needs a white
 * balance table of two knots or more. Reference awb.h:115-123
 * (lib/awb.c:86-211). */
CRAW_API int craw_awb_estimate(const CRAWProfile *p, const CRAWAwbHistogram *hist,
                               const CRAWAwbParams *params, CRAWAwbEstimate *out);

/* ------------------------------------------------------------ smoother */

/* A per-stream illuminant track kept in mired (reference awb.h:141-180,
 * lib/awb_smoother.c): exponential smoothing with a time constant, a
 * hysteresis dead band and a slew limit; estimates below min_confidence
 * hold the track; a scene cut with a confident estimate restarts it. */
typedef struct CRAWAwbSmoother CRAWAwbSmoother;

typedef struct CRAWAwbSmootherParams {
    float time_constant;            /* seconds; 1.0 */
    float hysteresis_mired;         /* 3.0 */
    float max_slew_mired_per_s;     /* 30.0 */
    float min_confidence;           /* 0.2 */
} CRAWAwbSmootherParams;

CRAW_API void craw_awb_smoother_params_init(CRAWAwbSmootherParams *p);
/* `params` NULL means the defaults; non-finite or non-positive time
 * constant or slew, or a negative hysteresis, is CRAW_ERROR(EINVAL). */
CRAW_API int craw_awb_smoother_create(const CRAWAwbSmootherParams *params,
                                      CRAWAwbSmoother **sm);
CRAW_API void craw_awb_smoother_free(CRAWAwbSmoother **sm);
/* Forgets the track: the next push starts one. */
CRAW_API void craw_awb_smoother_reset(CRAWAwbSmoother *sm);
/* Puts the track at `illum` as of `pts_s` (a seed, e.g. the camera's own
 * balance); an illuminant that is not finite and positive is ignored. */
CRAW_API void craw_awb_smoother_set(CRAWAwbSmoother *sm, double pts_s,
                                    const CRAWIlluminant *illum);
/* Feeds the estimate of the frame at `pts_s` and returns the illuminant to
 * apply to it. The first usable estimate starts the track whatever its
 * confidence; with no track and no usable estimate the call returns
 * CRAW_ERROR(EAGAIN) and leaves `out` as it was. The step is clamped to
 * [0, 1] s of presentation time. */
CRAW_API int craw_awb_smoother_push(CRAWAwbSmoother *sm, double pts_s,
                                    const CRAWAwbEstimate *est, bool scene_cut,
                                    CRAWIlluminant *out);

/* ------------------------------------------------------------ no-alloc */

/* The most 8x8 blocks craw_awb_histogram_from_rgb_cuda_noalloc() takes:
 * a 4096 x 4096 image, or any other whose ceil(w/8) * ceil(h/8) fits. */
#define CRAW_AWB_NOALLOC_MAX_BLOCKS (1u << 18)

/* The same histogram as craw_awb_histogram_from_rgb(), bit for bit, of an
 * image in device memory, built on the GPU without allocating anything.
 * This entry point has no counterpart in the reference.
 *
 * Who needs it: a caller that must not allocate device memory at the
 * moment it wants the statistic. A serving loop that has handed its whole
 * device-memory budget to the streams it admitted; a latency-bound thread
 * that cannot afford the device-wide synchronisation a fresh allocation
 * may cause; code that runs under an allocator it does not own, which may
 * refuse or reorder a request made at that moment. The pipeline's own AWB pass gets its scratch from memory it
 * allocates at creation; this one uses a fixed array in the library's
 * device image instead (3.3 MB per device, present once the library's
 * module is loaded there).
 *
 * Arguments as craw_awb_histogram_from_rgb(), except that `rgb` is a device
 * pointer; count, weight and weight_bright are host arrays of
 * CRAW_AWB_HIST_BINS^2 entries, overwritten. The work is enqueued on
 * `stream` and the call returns once the histogram is in those arrays (it
 * waits for `stream`). The few blocks whose bin lies within rounding of a
 * bin edge are binned on the host with its logf, as the CPU builder does.
 *
 * Limits and rules:
 *  - an image of more than CRAW_AWB_NOALLOC_MAX_BLOCKS blocks is refused
 *    with CRAW_ERROR(EINVAL) and a log line, before any device work;
 *  - the first call on each device does the set-up: it looks up the device
 *    address of the scratch array (cudaGetSymbolAddress, with that device
 *    current) and registers a 200 KB host staging area with
 *    cudaHostRegister, and keeps both for the process (a failed set-up is
 *    retried on the next call). Make that first call before any stream
 *    capture begins. A cudaDeviceReset() (or any other teardown of the
 *    device's primary context) leaves the kept address stale: do not call
 *    this entry point on a device after resetting it;
 *  - after the set-up a call makes only asynchronous copies (into the
 *    staging area) and waits on `stream` alone, with the calling thread's
 *    capture interaction relaxed for the call
 *    (cudaThreadExchangeStreamCaptureMode, restored before it returns).
 *    So it may run while another thread holds a global-mode stream
 *    capture, given a `stream` created with cudaStreamNonBlocking that is
 *    not itself capturing (the legacy default stream would synchronise
 *    with the capturing one);
 *  - a CUDA error that an earlier call left pending on the calling thread
 *    is reported (CRAW_ERROR(EIO)), not cleared;
 *  - the histograms and the counter in the scratch must be zero when the
 *    kernel starts; each call clears them on `stream` itself first;
 *  - all calls on one device share the one scratch array: two calls that
 *    overlap in time (two threads, or two streams) race on it and both
 *    results are garbage. Serialise the calls on a device.
 * Errors: CRAW_ERROR(EINVAL) for arguments, CRAW_ERROR(ENODEV) without a
 * current device, CRAW_ERROR(EIO) when a CUDA call fails. */
CRAW_API int craw_awb_histogram_from_rgb_cuda_noalloc(const float *rgb, uint32_t width,
                                                      uint32_t height, size_t stride,
                                                      int channels, const float wb_applied[3],
                                                      uint32_t *count, uint32_t *weight,
                                                      uint32_t *weight_bright,
                                                      cudaStream_t stream);

#endif /* CRAW_AWB_H */
