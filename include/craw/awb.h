/*
 * craw-gb300: auto white balance histogram and its CPU builder
 * (reference include/craw/awb.h).
 *
 * The GPU reduces each frame to a 2D histogram of raw chromaticity with
 * three counters per bin; the host reads it back. The estimator that
 * searches it is not part of this library's path.
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

/* The most 8x8 blocks craw_awb_histogram_from_rgb_cuda_noalloc() takes:
 * a 4096 x 4096 image, or any other whose ceil(w/8) * ceil(h/8) fits. */
#define CRAW_AWB_NOALLOC_MAX_BLOCKS (1u << 18)

/* The same histogram as craw_awb_histogram_from_rgb(), bit for bit, of an
 * image in device memory, built on the GPU without allocating anything.
 * This entry point has no counterpart in the reference.
 *
 * Who needs it: a caller that must not allocate device memory at the
 * moment it wants the statistic. A thread that runs while another thread
 * of the process captures a CUDA graph in global mode, where a cudaMalloc
 * would invalidate that capture; a serving loop that has handed its whole
 * device-memory budget to the streams it admitted; a latency-bound thread
 * that cannot afford the device-wide synchronisation a fresh allocation
 * may cause. The pipeline's own AWB pass gets its scratch from memory it
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
 *    current). Make that first call before any stream capture begins;
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
