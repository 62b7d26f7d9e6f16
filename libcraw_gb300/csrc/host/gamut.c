/*
 * ACES 1.3 Reference Gamut Compression constants (reference
 * lib/gamut.c:21-59): the Academy CTL's per-channel distance limits and
 * thresholds, power 1.2, and the scale that puts a distance of exactly
 * the limit on the AP1 hull, solved in double.
 */
#include <math.h>

#include "internal.h"

void craw_gamut_compress_params(CRAWGamutCompress *g)
{
    /* cyan, magenta, yellow */
    static const double lim[3] = { 1.147, 1.264, 1.312 };
    static const double thr[3] = { 0.815, 0.803, 0.880 };
    const double pwr = 1.2;

    for (int i = 0; i < 3; i++) {
        double r = pow((1.0 - thr[i]) / (lim[i] - thr[i]), -pwr) - 1.0;
        g->thr[i] = (float)thr[i];
        g->scl[i] = (float)((lim[i] - thr[i]) / pow(r, 1.0 / pwr));
    }
    g->pwr = (float)pwr;
    g->inv_pwr = (float)(1.0 / pwr);
}
