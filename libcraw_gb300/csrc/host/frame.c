/*
 * Per-frame constants shared by the pipeline and the batch: image checks,
 * the prep and colour constants of the develop kernels (reference
 * lib/pipeline.c:1360-1383, 1899-1931) and the denoise constants
 * (reference lib/pipeline.c:1385-1467).
 */
#include <math.h>
#include <string.h>

#include <craw/pipeline.h>

#include "internal.h"

/* Denoise highlight guard, reference lib/pipeline.c:291-292. */
#define DN_GUARD_LO 0.90f
#define DN_GUARD_HI 1.00f

size_t craw_format_bpp(CRAWFormat fmt)
{
    switch (fmt) {
    case CRAW_FORMAT_R16_UNORM:
    case CRAW_FORMAT_R16F:    return 2;
    case CRAW_FORMAT_RGBA16F: return 8;
    case CRAW_FORMAT_RGB32F:  return 12;
    default:                  return 16;
    }
}

bool craw_is_out_format(CRAWFormat fmt)
{
    return fmt == CRAW_FORMAT_RGBA16F || fmt == CRAW_FORMAT_RGBA32F || fmt == CRAW_FORMAT_RGB32F;
}

int craw_out_layout(CRAWFormat fmt)
{
    return fmt == CRAW_FORMAT_RGBA16F ? CRAW_K_OUT_RGBA16F
         : fmt == CRAW_FORMAT_RGB32F  ? CRAW_K_OUT_RGB32F : CRAW_K_OUT_RGBA32F;
}

int craw_image_check(CRAWContext *ctx, const CRAWImage *img, CRAWFormat fmt, uint32_t w, uint32_t h,
                     const char *what)
{
    size_t bpp = craw_format_bpp(fmt);
    if (img->format != fmt) {
        craw_log(ctx, CRAW_LOG_ERROR, "%s format %d, expected %d\n", what, (int)img->format, (int)fmt);
        return CRAW_ERROR(EINVAL);
    }
    if (img->width != w || img->height != h) {
        craw_log(ctx, CRAW_LOG_ERROR, "%s is %ux%u, expected %ux%u\n", what, img->width, img->height,
                 w, h);
        return CRAW_ERROR(EINVAL);
    }
    if (!img->data || ((uintptr_t)img->data & 15) || (img->pitch & 15) ||
        img->pitch < (size_t)img->width * bpp) {
        craw_log(ctx, CRAW_LOG_ERROR, "%s needs 16-byte aligned data and pitch >= width * %zu\n",
                 what, bpp);
        return CRAW_ERROR(EINVAL);
    }
    return 0;
}

bool craw_images_overlap(const CRAWImage *a, const CRAWImage *b)
{
    uintptr_t a0 = (uintptr_t)a->data, a1 = a0 + a->pitch * a->height;
    uintptr_t b0 = (uintptr_t)b->data, b1 = b0 + b->pitch * b->height;
    return a0 < b1 && b0 < a1;
}

static void mat3_mul_f(float out[3][3], const float a[3][3], const float b[3][3])
{
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            out[i][j] = a[i][0] * b[0][j] + a[i][1] * b[1][j] + a[i][2] * b[2][j];
}

int craw_develop_consts(CRAWContext *ctx, uint32_t w, uint32_t h, int debayer, bool fp16,
                        enum CRAWColorSpace default_space, const CRAWFrameParams *fp, CRAWKDevelop *dk)
{
    static const int chan[4] = { 0, 1, 1, 2 };
    CRAWColorParams frame;
    CRAWGamutCompress gc;
    enum CRAWColorSpace out_space;
    float m_out[3][3], scale;
    int ret;

    /* The prep applies the frame's own gains, so that the clip at 1.0
     * keeps blown highlights neutral under whatever illuminant is chosen. */
    if ((ret = craw_profile_eval(fp->profile, fp->wb_mode, &fp->illuminant, &frame)) < 0)
        return ret;
    memset(dk, 0, sizeof(*dk));
    dk->width = (int32_t)w;
    dk->height = (int32_t)h;
    dk->clip = 1.0f;
    dk->method = debayer;
    dk->fp16 = fp16;
    for (int s = 0; s < 4; s++) {
        float range = fp->profile->white_level[s] - fp->profile->black_level[s];
        if (!(range > 0.0f)) {
            craw_log(ctx, CRAW_LOG_ERROR, "Profile site %d has white level %f <= black level %f\n",
                     s, fp->profile->white_level[s], fp->profile->black_level[s]);
            return CRAW_ERROR(EINVAL);
        }
        dk->black[s] = fp->profile->black_level[s];
        dk->range[s] = range;
        dk->inv_range[s] = 1.0f / range;
        dk->wbs[s] = frame.wb[chan[s]];
    }
    for (int c = 0; c < 3; c++)
        dk->awb_wb[c] = frame.wb[c];

    /* M_out * cam_to_xyz * gain * 2^stops, composed in float; the RGC for
     * ACEScg unless the frame vetoes it. */
    out_space = fp->out_space_set ? fp->out_space : default_space;
    if ((ret = craw_colorspace_from_xyz_d65(out_space, m_out)) < 0) {
        craw_log(ctx, CRAW_LOG_ERROR, "Unknown output colour space %d\n", (int)out_space);
        return ret;
    }
    craw_gamut_compress_params(&gc);
    mat3_mul_f(dk->color.m, m_out, frame.cam_to_xyz);
    scale = frame.gain * exp2f(fp->exposure_stops);
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++)
            dk->color.m[i][j] *= scale;
        dk->color.gc_thr[i] = gc.thr[i];
        dk->color.gc_scl[i] = gc.scl[i];
    }
    dk->color.gc_pwr = gc.pwr;
    dk->color.gc_inv_pwr = gc.inv_pwr;
    dk->color.flags = (fp->flags & CRAW_FRAME_FLAG_CLAMP_NEGATIVE) ? CRAW_K_COLOR_CLAMP : 0;
    if (out_space == CRAW_CS_ACES_AP1_LINEAR && !(fp->flags & CRAW_FRAME_FLAG_NO_GAMUT_COMPRESSION))
        dk->color.flags |= CRAW_K_COLOR_RGC;
    return 0;
}

int craw_denoise_consts(CRAWContext *ctx, uint32_t w, uint32_t h, const CRAWFrameParams *fp, int mode,
                        CRAWKDenoise *k, CRAWKDenoiseExact *ex)
{
    CRAWNoiseModel nm;
    float a, b, c, hs;
    int ret;

    /* The override when it carries a positive a, else the profile's table
     * at its as-shot exposure index. */
    if (fp->noise_override.a > 0.0f) {
        nm = fp->noise_override;
    } else if ((ret = craw_profile_noise_eval(fp->profile, fp->profile->as_shot_ei, &nm)) < 0) {
        craw_log(ctx, CRAW_LOG_ERROR, "Denoising needs a noise model: the profile `%s` has no "
                 "table and CRAWFrameParams.noise_override was not set\n",
                 fp->profile->name[0] ? fp->profile->name : "(unnamed)");
        return ret;
    }
    a = nm.a;
    b = CRAW_MAX(nm.b, 0.0f);
    if (!(a > 0.0f)) {
        craw_log(ctx, CRAW_LOG_ERROR, "Noise model a = %g is not positive\n", (double)a);
        return CRAW_ERROR(EINVAL);
    }
    c = 3.0f * a * a / 8.0f + b;
    /* One threshold for both filters: the spatial strength when that one
     * runs, the modelled noise level when it does not. */
    hs = (mode & CRAW_K_DN_SPATIAL) ? fp->denoise_strength : 1.0f;
    memset(k, 0, sizeof(*k));
    k->pw = (int32_t)(w / 2);
    k->ph = (int32_t)(h / 2);
    k->gat_a = a;
    k->gat_c = c;
    k->gat_sc = sqrtf(c);
    k->gat_fwd = 2.0f / a;
    k->gat_inv = a / 4.0f;
    k->gat_off = c / a;
    k->gat_t0 = k->gat_fwd * k->gat_sc;
    k->inv_h2 = 1.0f / (hs * hs);
    k->t_alpha = (mode & CRAW_K_DN_TEMPORAL) ? fp->denoise_temporal_strength : 0.0f;
    k->t_inv_h2 = 1.0f / (hs * hs);
    k->guard_lo = DN_GUARD_LO;
    k->guard_inv = 1.0f / (DN_GUARD_HI - DN_GUARD_LO);
    k->mode = mode;
    for (int s = 0; s < 4; s++) {
        float range = fp->profile->white_level[s] - fp->profile->black_level[s];
        k->black[s] = fp->profile->black_level[s];
        k->inv_range[s] = 1.0f / range;
        k->range[s] = range;
    }
    if (ex)
        craw_denoise_exact_consts(k, fp->profile, nm.a, b, hs, ex);
    return 0;
}

/* A double split into two floats: hi the nearest float, lo the nearest
 * float to the rest (together within 2^-48 relative of v). */
static void split(double v, float out[2])
{
    out[0] = (float)v;
    out[1] = (float)(v - (double)out[0]);
}

void craw_denoise_exact_consts(const CRAWKDenoise *k, const CRAWProfile *prof, float a, float b, float strength,
                               CRAWKDenoiseExact *ex)
{
    /* The reference's arithmetic in double (lib/ref/ref_denoise.c:25-58,
     * 173-336 with R = double): the noise model, the levels and the
     * strength are floats and enter exactly. */
    const double ad = a, cd = 3.0 * ad * ad / 8.0 + (double)b, h = strength > 0.0f ? strength : 1.0;
    const double sc = sqrt(cd), fwd = 2.0 / ad;
    double bmax = 0.0;
    memset(ex, 0, sizeof(*ex));
    ex->pw = k->pw;
    ex->ph = k->ph;
    ex->mode = k->mode;
    for (int s = 0; s < 4; s++) {
        const double blk = (double)prof->black_level[s], rng = (double)prof->white_level[s] - blk;
        split(blk, ex->black[s]);
        split(rng, ex->range[s]);
        split(1.0 / rng, ex->inv_range[s]);
        /* The float decision stage. */
        ex->k1[s] = (float)(1.0 / (65535.0 * rng));
        ex->k0[s] = (float)(blk / rng);
        ex->q[s] = (float)(4.0 / (65535.0 * rng * ad));
        ex->k2[s] = (float)(65535.0 * rng * ad / 4.0);
        split(4.0 / (65535.0 * rng * ad), ex->qq[s]);
        split(4.0 * cd / (ad * ad) - 4.0 * blk / (ad * rng), ex->beta[s]);
        bmax = fmax(bmax, blk);
    }
    split(1.0 / 65535.0, ex->inv65535);
    ex->gat_a = a;
    split(cd, ex->gat_c);
    split(sc, ex->gat_sc);
    split(1.0 / sc, ex->gat_isc);
    split(fwd, ex->gat_fwd);
    split(ad / 4.0, ex->gat_inv);
    split(cd / ad, ex->gat_off);
    split(fwd * sc, ex->gat_t0);
    split((1.0 / 9.0) * (1.0 / (h * h)), ex->k_nlm);
    split((double)DN_GUARD_LO, ex->guard_lo);
    split(1.0 / ((double)DN_GUARD_HI - (double)DN_GUARD_LO), ex->guard_inv);
    ex->kn = (float)((1.0 / 9.0) / (h * h));
    ex->c1 = (float)(-1.4426950408889634 * (1.0 / 9.0) / (h * h));
    ex->c0 = (float)(2.0 * 1.4426950408889634);
    ex->dark_code = (uint32_t)ceil(bmax * 65535.0) + 1u;
    ex->decide = craw_round_decide;
}

void craw_denoise_round_band(const CRAWKDenoise *k, float scale, CRAWKRound *rd)
{
    /* The float path's error in codes, about B ulps of t carried through
     * dx/dt = 65535 range (a/2) t (the inverse transform), plus a few ulps
     * of x itself (x <= 65535 black + 65535 range a/4 t^2) and of t near
     * the transform's linear branch. With the weighted sums centred (the
     * marking kernel sums w (q - c), c a neighbour's value), B = 6 makes the
     * band at scale 1 about twice the largest error seen in the float
     * evaluation; `scale` multiplies the whole band (2 by default). */
    const double B = 6.0 * 0x1p-24, X = 2.0 * 0x1p-24;
    double rmax = 0.0, bmax = 0.0;
    for (int s = 0; s < 4; s++) {
        rmax = fmax(rmax, (double)k->range[s]);
        bmax = fmax(bmax, (double)k->black[s]);
    }
    const double a = k->gat_a;
    rd->c2 = (float)(scale * (B * 65535.0 * rmax * a / 2.0 + X * 65535.0 * rmax * a / 4.0));
    rd->c0 = (float)(scale * (B * 65535.0 * rmax * ((double)k->gat_sc + a / 2.0 * (double)k->gat_t0) *
                              ((double)k->gat_t0 + 1.0) + X * 65535.0 * bmax));
    if (scale >= 1e6f) {
        /* Every sample. */
        rd->c0 = 1.0f;
        rd->c2 = 0.0f;
    }
}
