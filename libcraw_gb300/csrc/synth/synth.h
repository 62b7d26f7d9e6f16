/*
 * Seeded synthetic Bayer frames for the benchmark and the tests: a linear
 * RGB scene (two-axis colour gradient, random axis-aligned rectangles of
 * uniform reflectance, zone plates, optional moving rectangles), divided
 * by the inverse white balance, mosaicked RGGB and given Poisson-Gaussian
 * noise in 12-bit code values, var = a_dn * signal + b_dn, then clipped.
 * Every pixel's noise comes from a counter-based hash of (seed, frame,
 * position), so a frame is the same however many threads make it.
 */
#ifndef CRAW_SYNTH_H
#define CRAW_SYNTH_H

#include <stddef.h>
#include <stdint.h>

#define CRAW_SYNTH_MAX_MOVERS 4

typedef struct CRAWSynthParams {
    uint32_t width, height;       /* even */
    uint64_t seed;                /* scene layout and noise */
    uint32_t frame;               /* frame index: noise and mover positions */
    uint32_t nb_rects;            /* random rectangles */
    uint32_t nb_zone_plates;      /* 256 x 256 zone plates */
    float noise_a_dn;             /* shot term, DN per DN of signal */
    float noise_b_dn;             /* read term, DN^2 */
    float wb[3];                  /* the camera's gains; the scene is divided by them */
    uint32_t black_dn, white_dn;  /* e.g. 256 and 4095 */

    /* Moving rectangles over a static background: speed in px/frame along
     * x, and level above the background in units of the local noise
     * sigma. nb_movers 0 for none. */
    uint32_t nb_movers;
    float mover_speed[CRAW_SYNTH_MAX_MOVERS];
    float mover_contrast[CRAW_SYNTH_MAX_MOVERS];
} CRAWSynthParams;

/* Fills `out` (stride in samples) with one frame; 0 or -EINVAL. Uses the
 * host's OpenMP threads. */
int craw_synth_frame(const CRAWSynthParams *p, uint16_t *out, size_t stride);

#endif /* CRAW_SYNTH_H */
