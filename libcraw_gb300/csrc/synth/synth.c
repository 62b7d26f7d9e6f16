/*
 * Seeded synthetic Bayer frames; see synth.h. Host code, shared by the
 * benchmark and the tests; not part of the development path.
 */
#include <errno.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "synth.h"

#define SYN_API __attribute__((visibility("default")))

/* splitmix64: the seed sequence for the layout and the per-pixel hash. */
static uint64_t syn_mix(uint64_t z)
{
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

typedef struct { uint64_t s; } syn_rng;

static double syn_uniform(syn_rng *r)
{
    r->s = syn_mix(r->s);
    return (double)(r->s >> 11) * (1.0 / 9007199254740992.0);
}

static inline int syn_chan(uint32_t x, uint32_t y)
{
    int s = (int)((y & 1) * 2 + (x & 1));
    return s == 0 ? 0 : (s == 3 ? 2 : 1);
}

/* The background at one pixel: a smooth gradient in both axes, different
 * per channel, within [0.08, 0.62]. */
static inline float syn_gradient(const CRAWSynthParams *p, uint32_t x, uint32_t y, int c)
{
    double fx = (double)x / (double)(p->width - 1), fy = (double)y / (double)(p->height - 1);
    switch (c) {
    case 0:  return (float)(0.10 + 0.45 * fx + 0.05 * fy);
    case 1:  return (float)(0.12 + 0.10 * fx + 0.40 * fy);
    default: return (float)(0.08 + 0.30 * (1.0 - fx) + 0.24 * fy);
    }
}

struct syn_rect { int x0, y0, x1, y1; float refl[3]; };

static void syn_fill_rect(float *s, const CRAWSynthParams *p, const struct syn_rect *r)
{
    int x0 = r->x0 < 0 ? 0 : r->x0, y0 = r->y0 < 0 ? 0 : r->y0;
    int x1 = r->x1 > (int)p->width ? (int)p->width : r->x1;
    int y1 = r->y1 > (int)p->height ? (int)p->height : r->y1;
    #pragma omp parallel for schedule(static)
    for (int y = y0; y < y1; y++)
        for (int x = x0; x < x1; x++)
            s[(size_t)y * p->width + x] = r->refl[syn_chan((uint32_t)x, (uint32_t)y)];
}

/* A 256 x 256 zone plate: cos(pi r^2 / 256), whose local frequency runs
 * from 0 at the centre to the Nyquist rate at r = 128, tinted per
 * channel, between 0.05 and 0.85 of the tint. */
static void syn_fill_zone(float *s, const CRAWSynthParams *p, int cx, int cy, const float tint[3])
{
    int x0 = cx - 128, y0 = cy - 128;
    #pragma omp parallel for schedule(static)
    for (int j = 0; j < 256; j++) {
        int y = y0 + j;
        if (y < 0 || y >= (int)p->height)
            continue;
        for (int i = 0; i < 256; i++) {
            int x = x0 + i;
            double dx = (double)i - 127.5, dy = (double)j - 127.5;
            double v;
            if (x < 0 || x >= (int)p->width)
                continue;
            v = 0.45 + 0.40 * cos(3.14159265358979323846 * (dx * dx + dy * dy) / 256.0);
            s[(size_t)y * p->width + x] = (float)v * tint[syn_chan((uint32_t)x, (uint32_t)y)];
        }
    }
}

SYN_API int craw_synth_frame(const CRAWSynthParams *p, uint16_t *out, size_t stride)
{
    float *s;
    syn_rng rng;
    double range;

    if (!p || !out || p->width < 2 || p->height < 2 || (p->width & 1) || (p->height & 1) ||
        stride < p->width || !(p->wb[0] > 0) || !(p->wb[1] > 0) || !(p->wb[2] > 0) ||
        p->white_dn <= p->black_dn || p->nb_movers > CRAW_SYNTH_MAX_MOVERS)
        return -EINVAL;
    s = malloc((size_t)p->width * p->height * sizeof(float));
    if (!s)
        return -ENOMEM;
    range = (double)(p->white_dn - p->black_dn);

    #pragma omp parallel for schedule(static)
    for (uint32_t y = 0; y < p->height; y++)
        for (uint32_t x = 0; x < p->width; x++)
            s[(size_t)y * p->width + x] = syn_gradient(p, x, y, syn_chan(x, y));

    rng.s = syn_mix(p->seed ^ 0x5eedull);
    for (uint32_t i = 0; i < p->nb_rects; i++) {
        struct syn_rect r;
        int rw = 8 + (int)(syn_uniform(&rng) * (double)p->width / 8.0);
        int rh = 8 + (int)(syn_uniform(&rng) * (double)p->height / 8.0);
        r.x0 = (int)(syn_uniform(&rng) * (double)p->width) - rw / 2;
        r.y0 = (int)(syn_uniform(&rng) * (double)p->height) - rh / 2;
        r.x1 = r.x0 + rw;
        r.y1 = r.y0 + rh;
        for (int c = 0; c < 3; c++)
            r.refl[c] = (float)(0.05 + 0.85 * syn_uniform(&rng));
        syn_fill_rect(s, p, &r);
    }
    for (uint32_t i = 0; i < p->nb_zone_plates; i++) {
        float tint[3];
        int cx = (int)(syn_uniform(&rng) * (double)p->width);
        int cy = (int)(syn_uniform(&rng) * (double)p->height);
        for (int c = 0; c < 3; c++)
            tint[c] = (float)(0.6 + 0.4 * syn_uniform(&rng));
        syn_fill_zone(s, p, cx, cy, tint);
    }
    /* Movers: 96 x 64 grey patches in their own rows, entering from the
     * left and wrapping around, at background + k sigma, where sigma is
     * the noise at that background level in the scene's units. */
    for (uint32_t i = 0; i < p->nb_movers; i++) {
        struct syn_rect r;
        double base = 0.30, sig_dn, k = p->mover_contrast[i];
        int span = (int)p->width + 96;
        int x = (int)fmod((double)p->mover_speed[i] * (double)p->frame, (double)span) - 96;
        r.x0 = x;
        r.x1 = x + 96;
        r.y0 = (int)(((double)i + 0.5) * (double)p->height / (double)(p->nb_movers + 1)) & ~1;
        r.y1 = r.y0 + 64;
        for (int c = 0; c < 3; c++) {
            double sig = base / p->wb[c] * range;
            sig_dn = sqrt(p->noise_a_dn * sig + p->noise_b_dn);
            r.refl[c] = (float)(base + k * sig_dn / range * p->wb[c]);
        }
        syn_fill_rect(s, p, &r);
    }

    #pragma omp parallel for schedule(static)
    for (uint32_t y = 0; y < p->height; y++) {
        for (uint32_t x = 0; x < p->width; x++) {
            int c = syn_chan(x, y);
            double sig = (double)s[(size_t)y * p->width + x] / p->wb[c] * range;
            double var = p->noise_a_dn * (sig > 0 ? sig : 0) + p->noise_b_dn;
            uint64_t h = syn_mix(p->seed * 0x100000001b3ull ^ syn_mix(((uint64_t)p->frame << 40) ^
                                 ((uint64_t)y << 20) ^ x));
            double u1 = ((double)(h >> 40) + 0.5) * (1.0 / 16777216.0);
            double u2 = (double)((h >> 16) & 0xffffff) * (1.0 / 16777216.0);
            double g = sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
            double v = (double)p->black_dn + sig + sqrt(var) * g;
            long iv = lrint(v);
            iv = iv < 0 ? 0 : (iv > (long)p->white_dn ? (long)p->white_dn : iv);
            out[(size_t)y * stride + x] = (uint16_t)iv;
        }
    }
    free(s);
    return 0;
}
