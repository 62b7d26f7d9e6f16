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

#endif /* CRAW_AWB_H */
