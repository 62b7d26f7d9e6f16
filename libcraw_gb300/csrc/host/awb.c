/*
 * The CPU AWB histogram builder (reference lib/awb.c:213-296), also used
 * by the pipeline to bin the few blocks the device defers because their
 * bin sits within rounding of an edge: both go through awb_bin() below,
 * so the device histogram is the builder's bit for bit.
 */
#include <math.h>
#include <string.h>

#include <craw/awb.h>

#include "internal.h"

static void awb_bin(float rr, float bb, float g, uint32_t *count, uint32_t *weight,
                    uint32_t *weight_bright)
{
    const uint32_t bins = CRAW_AWB_HIST_BINS;
    const float lmin = CRAW_AWB_HIST_LOG_MIN, lmax = CRAW_AWB_HIST_LOG_MAX;
    const float span = lmax - lmin;
    float x = logf(rr), y = logf(bb), w;
    int ix, iy;

    /* A NaN from a negative overshoot lands in the first bin. */
    x = x > lmin ? (x < lmax ? x : lmax) : lmin;
    y = y > lmin ? (y < lmax ? y : lmax) : lmin;
    ix = (int)floorf((x - lmin) / span * bins);
    iy = (int)floorf((y - lmin) / span * bins);
    ix = CRAW_CLAMP(ix, 0, (int)bins - 1);
    iy = CRAW_CLAMP(iy, 0, (int)bins - 1);
    w = CRAW_MIN(g, 0.5f);
    count[iy * bins + ix] += 1;
    weight[iy * bins + ix] += (uint32_t)roundf(w * 65536.0f);
    weight_bright[iy * bins + ix] += (uint32_t)roundf(g * g * g * g * 65536.0f);
}

void craw_awb_bin_host(float rr, float bb, float g, uint32_t *count, uint32_t *weight,
                       uint32_t *weight_bright)
{
    awb_bin(rr, bb, g, count, weight, weight_bright);
}

CRAW_API int craw_awb_histogram_from_rgb(const float *rgb, uint32_t width, uint32_t height,
                                         size_t stride, int channels, const float wb[3],
                                         uint32_t *count, uint32_t *weight,
                                         uint32_t *weight_bright)
{
    const size_t n = (size_t)CRAW_AWB_HIST_BINS * CRAW_AWB_HIST_BINS;

    if (!rgb || !wb || !count || !weight || !weight_bright)
        return CRAW_ERROR(EINVAL);
    if ((channels != 3 && channels != 4) || stride < (size_t)width * (size_t)channels)
        return CRAW_ERROR(EINVAL);
    if (!(wb[0] > 0.0f) || !(wb[2] > 0.0f))
        return CRAW_ERROR(EINVAL);
    memset(count, 0, n * sizeof(*count));
    memset(weight, 0, n * sizeof(*weight));
    memset(weight_bright, 0, n * sizeof(*weight_bright));

    for (uint32_t by = 0; by < height; by += 8) {
        uint32_t y1 = CRAW_MIN(by + 8, height);
        for (uint32_t bx = 0; bx < width; bx += 8) {
            uint32_t x1 = CRAW_MIN(bx + 8, width);
            float s[3] = { 0.0f, 0.0f, 0.0f }, n_px = (float)((y1 - by) * (x1 - bx));
            float r, g, b;
            /* Row by row, left to right, over the pixels that exist. */
            for (uint32_t y = by; y < y1; y++) {
                const float *row = rgb + (size_t)y * stride;
                for (uint32_t x = bx; x < x1; x++)
                    for (int c = 0; c < 3; c++)
                        s[c] += row[(size_t)x * channels + c];
            }
            r = s[0] / n_px;
            g = s[1] / n_px;
            b = s[2] / n_px;
            /* Clipped blocks have lost their colour, dark ones never had it. */
            if (CRAW_MAX(CRAW_MAX(r, g), b) >= 0.98f || g < 0.002f)
                continue;
            awb_bin((r / wb[0]) / g, (b / wb[2]) / g, g, count, weight, weight_bright);
        }
    }
    return 0;
}
