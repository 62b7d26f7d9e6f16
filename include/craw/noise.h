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

#endif /* CRAW_NOISE_H */
