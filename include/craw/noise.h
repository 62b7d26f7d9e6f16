/*
 * craw-gb300: sensor noise model (reference include/craw/noise.h).
 *
 * var(u) = a * u + b, with u the signal above black normalised so that
 * black is 0 and white 1, before any white balance. One (a, b) pair holds
 * for all four CFA planes.
 */
#ifndef CRAW_NOISE_H
#define CRAW_NOISE_H

#include <stdint.h>
#include <stdbool.h>

#include <craw/utils.h>

struct CRAWProfile;

typedef struct CRAWNoiseModel {
    float a;   /* shot term */
    float b;   /* read term */
} CRAWNoiseModel;

/* The model measured at one exposure index; tables ascend in iso. */
typedef struct CRAWNoiseKnot {
    float iso;
    float a, b;
} CRAWNoiseKnot;

#define CRAW_PROFILE_MAX_NOISE_KNOTS 16

/* Evaluates a knot table at `iso`: a power law between knots (linear in
 * log iso of log a and log b, or linear where a term is zero), a ~ iso on
 * both sides outside the table, b ~ iso^2 above it and b constant below
 * it; a non-positive or non-finite iso gets the first knot.
 * CRAW_ERROR(EINVAL) on an empty table. Same contract as reference
 * noise.h:65-66 (lib/noise.c:37-110). */
CRAW_API int craw_noise_model_eval(const CRAWNoiseKnot *knots, uint32_t nb_knots,
                                   float iso, CRAWNoiseModel *out);

/* ------------------------------------------------------------ estimation */

/* Options of craw_noise_estimate() (reference noise.h:86-104, same layout).
 * Zero-initialise and call craw_noise_estimate_params_init() for the
 * defaults. */
typedef struct CRAWNoiseEstimateParams {
    /* Intensity bins, 8 to CRAW_NOISE_MAX_BINS (0: 128), equally spaced in
     * the square root of the local mean. */
    uint32_t nb_bins;

    /* Bins with fewer samples are dropped (0: 20000). */
    uint32_t min_bin_samples;

    /* Samples whose local mean is above this are ignored (0: 0.98). */
    float max_level;

    /* Reserved, must be zero. */
    uint8_t padding[64 - 4 * 3];
} CRAWNoiseEstimateParams;

#define CRAW_NOISE_MAX_BINS 512

/* What craw_noise_estimate() found (reference noise.h:107-129, same
 * layout): the model and the evidence for it. */
typedef struct CRAWNoiseEstimate {
    CRAWNoiseModel model;

    uint32_t nb_bins;       /* bins that had enough samples */
    uint32_t nb_inliers;    /* of those, bins the fit explains (|ln error| < 0.35) */

    /* RMS of ln(measured variance) - ln(modelled variance) over the
     * inliers: the fit's relative error. */
    float fit_rms;

    /* sqrt(b) in 16-bit code values of site 0's range. */
    float read_noise_lsb;

    /* Reserved. */
    uint8_t padding[64 - 4 * 6];
} CRAWNoiseEstimate;

CRAW_API void craw_noise_estimate_params_init(CRAWNoiseEstimateParams *p);

/* Fits var = a * u + b to one Bayer frame (reference noise.h:131-161,
 * lib/noise.c:338-504), measured on the GPU.
 *
 * `bayer` is width x height 16-bit UNORM samples in host memory with
 * `stride` samples per row; `profile` gives the per-site black and white
 * levels and the CFA phase. Both dimensions must be even and at least 32.
 * Each CFA plane is high-pass filtered with [1 -2 1; -2 4 -2; 1 -2 1] / 6,
 * every interior sample is binned by its 9x9 plane mean (bins equally
 * spaced in sqrt(mean)), each bin's noise is the median |residual| /
 * 0.6745, and the line through the bins is fitted robustly (least trimmed
 * squares over bin pairs, then Tukey-weighted Gauss-Newton on ln variance).
 *
 * The frame is copied to the calling thread's current CUDA device and
 * binned there; the call returns when the estimate is ready. Fails with
 * CRAW_ERROR(EINVAL) on bad arguments, CRAW_ERROR(ENOTSUP) for a
 * non-RGGB phase, CRAW_ERROR(ENODATA) when fewer than three bins survive
 * or no physical line fits them, CRAW_ERROR(ENOMEM) / CRAW_ERROR(EIO) on
 * device failures. craw_noise_estimate_cuda() (craw/cuda.h) takes a frame
 * already on the device. */
CRAW_API int craw_noise_estimate(const uint16_t *bayer, uint32_t width, uint32_t height,
                                 size_t stride, const struct CRAWProfile *profile,
                                 const CRAWNoiseEstimateParams *params,
                                 CRAWNoiseEstimate *out);

#endif /* CRAW_NOISE_H */
