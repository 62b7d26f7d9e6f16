/*
 * craw-gb300: the lens-correction record (reference include/craw/lens.h).
 *
 * The lens warp is not part of this library's path; the struct is kept
 * only because CRAWFrameParams carries it by value (reference
 * pipeline.h:320), so that the frame parameters stay byte compatible.
 */
#ifndef CRAW_LENS_H
#define CRAW_LENS_H

#include <stdint.h>
#include <stdbool.h>

#include <craw/utils.h>

typedef struct CRAWLensCorrection {
    float k[3][4];      /* per channel R, G, B radial terms */
    float centre[2];    /* optical centre, normalised frame coordinates */
    bool valid;         /* false: no correction for this frame */
    uint8_t reserved[64 - 3*4*4 - 2*4 - 1];
} CRAWLensCorrection;

/* The largest turn a frame may ask for, either way, in degrees. */
#define CRAW_LENS_MAX_ROTATION 45.0f

#endif /* CRAW_LENS_H */
