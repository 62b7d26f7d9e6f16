/*
 * The AWB estimator over a frame's 128^2 histogram and the per-stream
 * illuminant track that smooths its readings (reference lib/awb.c:15-211
 * and lib/awb_smoother.c). Host code: the histogram is 64 KB per counter
 * and the search walks the white balance locus once per occupied bin. The
 * arithmetic is the reference's, in double, so that both give the same
 * illuminant for the same histogram.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <craw/awb.h>

/* The in-band share at which a reading is fully trusted, and the spread
 * along the locus at which it is not trusted at all (reference
 * lib/awb.c:12-13). */
#define CONF_FULL_ZONE_FRACTION 0.3
#define CONF_ZERO_SPREAD_MIRED  60.0

CRAW_API void craw_awb_params_init(CRAWAwbParams *p)
{
    if (!p)
        return;
    memset(p, 0, sizeof(*p));
    p->band = 0.08f;
    p->sigma = 0.05f;
    p->min_zone_fraction = 0.02f;
    p->ambience = 0.0f;
    p->ambience_knee_cct = 4000.0f;
    p->prefer_bright = true;
    p->bright_max_spread_mired = 60.0f;
}

/* Running sums of one weighting: its whole mass, the mass inside the band,
 * and the falloff-weighted moments of mired and tint inside it. */
struct reading {
    double total, zone;
    double w, w_mired, w_mired2, w_tint;
};

static void reading_add(struct reading *r, double mass, bool in_band, double falloff,
                        double mired, double tint)
{
    double w;
    r->total += mass;
    if (!in_band)
        return;
    r->zone += mass;
    w = mass * falloff;
    if (!(w > 0.0))
        return;
    r->w += w;
    r->w_mired += w * mired;
    r->w_mired2 += w * mired * mired;
    r->w_tint += w * tint;
}

/* A reading becomes a candidate: weighted mean mired and tint, the share
 * inside the band, and the standard deviation along the locus (the
 * variance clamped at zero, since all mass in one bin makes it a rounding
 * residue). `max_spread` 0 means no spread limit. */
static void reading_result(const struct reading *r, double min_zone_fraction, double max_spread,
                           CRAWAwbCandidate *c)
{
    double in_band, mired, var, spread;

    memset(c, 0, sizeof(*c));
    if (!(r->total > 0.0) || !(r->w > 0.0))
        return;
    in_band = r->zone / r->total;
    mired = r->w_mired / r->w;
    var = r->w_mired2 / r->w - mired * mired;
    spread = var > 0.0 ? sqrt(var) : 0.0;
    c->valid = in_band >= min_zone_fraction && (max_spread <= 0.0 || spread <= max_spread);
    c->illuminant.cct = (float)(1e6 / mired);
    c->illuminant.tint = (float)(r->w_tint / r->w);
    c->in_zone_fraction = (float)in_band;
    c->spread_mired = (float)spread;
}

static double clampd(double v, double lo, double hi)
{
    return v < lo ? lo : (v > hi ? hi : v);
}

CRAW_API int craw_awb_estimate(const CRAWProfile *p, const CRAWAwbHistogram *hist,
                               const CRAWAwbParams *params, CRAWAwbEstimate *out)
{
    CRAWAwbParams def;
    struct reading zone, bright;
    const CRAWAwbCandidate *pick;
    double span, cct, conf, lo, hi;
    int ret;

    if (!p || !hist || !out || !hist->count || !hist->weight || hist->bins < 2 ||
        !(hist->log_max > hist->log_min))
        return CRAW_ERROR(EINVAL);
    if (p->nb_wb_knots < 2)
        return CRAW_ERROR(ENOTSUP);
    if (!params) {
        craw_awb_params_init(&def);
        params = &def;
    }
    if (!(params->band > 0.0f) || !(params->sigma > 0.0f))
        return CRAW_ERROR(EINVAL);

    memset(out, 0, sizeof(*out));
    memset(&zone, 0, sizeof(zone));
    memset(&bright, 0, sizeof(bright));
    span = (double)hist->log_max - hist->log_min;

    for (uint32_t iy = 0; iy < hist->bins; iy++) {
        const double y = hist->log_min + span * (iy + 0.5) / hist->bins;
        for (uint32_t ix = 0; ix < hist->bins; ix++) {
            const uint32_t i = iy * hist->bins + ix;
            const CRAWIlluminant *at;
            CRAWIlluminant il;
            float n_rg, n_bg;
            double x, dx, dy, d, q;

            if (!hist->count[i])
                continue;
            x = hist->log_min + span * (ix + 0.5) / hist->bins;
            /* The bin centre as a neutral: its locus point and how far
             * from the locus it sits (distance to the tint-free neutral of
             * that point). */
            if ((ret = craw_profile_neutral_to_illuminant(p, (float)exp(x), (float)exp(y), &il)) < 0)
                return ret;
            at = &(CRAWIlluminant){ .cct = il.cct, .tint = 0.0f };
            if ((ret = craw_profile_illuminant_to_neutral(p, at, &n_rg, &n_bg)) < 0)
                return ret;
            dx = x - log((double)n_rg);
            dy = y - log((double)n_bg);
            d = sqrt(dx * dx + dy * dy);
            q = d / params->sigma;
            reading_add(&zone, hist->weight[i] / 65536.0, d < params->band, exp(-q * q),
                        1e6 / il.cct, il.tint);
            if (hist->weight_bright)
                reading_add(&bright, hist->weight_bright[i] / 65536.0, d < params->band,
                            exp(-q * q), 1e6 / il.cct, il.tint);
        }
    }
    reading_result(&zone, params->min_zone_fraction, 0.0, &out->zone);
    reading_result(&bright, params->min_zone_fraction, params->bright_max_spread_mired,
                   &out->bright);

    /* A light source (or its glare) in frame is the illuminant itself. */
    if (params->prefer_bright && out->bright.valid) {
        pick = &out->bright;
        out->source = CRAW_AWB_SOURCE_BRIGHT;
    } else if (out->zone.in_zone_fraction > 0.0f || out->zone.valid) {
        pick = &out->zone;
        out->source = CRAW_AWB_SOURCE_ZONE;
    } else {
        return 0;
    }
    if (!(pick->illuminant.cct > 0.0f))
        return 0;

    conf = clampd(pick->in_zone_fraction / CONF_FULL_ZONE_FRACTION, 0.0, 1.0) *
           clampd(1.0 - pick->spread_mired / CONF_ZERO_SPREAD_MIRED, 0.0, 1.0);
    cct = pick->illuminant.cct;
    /* Ambience keeps part of a warm light's warmth instead of correcting
     * it fully to neutral. */
    if (params->ambience > 0.0f && cct < params->ambience_knee_cct)
        cct += (double)params->ambience * (params->ambience_knee_cct - cct);
    lo = params->cct_min > 0.0f ? params->cct_min : p->wb_knots[0].cct;
    hi = params->cct_max > 0.0f ? params->cct_max : p->wb_knots[p->nb_wb_knots - 1].cct;
    if (hi < lo)
        hi = lo;
    cct = clampd(cct, lo, hi);

    out->valid = pick->valid;
    out->illuminant.cct = (float)cct;
    out->illuminant.tint = pick->illuminant.tint;
    out->confidence = (float)conf;
    out->in_zone_fraction = pick->in_zone_fraction;
    out->spread_mired = pick->spread_mired;
    return 0;
}

/* ------------------------------------------------------------ smoother */

/* The track in mired, where a fixed step is a roughly constant visual
 * change at any colour temperature. */
struct CRAWAwbSmoother {
    CRAWAwbSmootherParams params;
    bool tracking;
    double mired, tint, last_pts;
};

CRAW_API void craw_awb_smoother_params_init(CRAWAwbSmootherParams *p)
{
    if (!p)
        return;
    p->time_constant = 1.0f;
    p->hysteresis_mired = 3.0f;
    p->max_slew_mired_per_s = 30.0f;
    p->min_confidence = 0.2f;
}

CRAW_API int craw_awb_smoother_create(const CRAWAwbSmootherParams *params, CRAWAwbSmoother **sm)
{
    CRAWAwbSmoother *s;
    const CRAWAwbSmootherParams *q;

    if (!sm)
        return CRAW_ERROR(EINVAL);
    *sm = NULL;
    if (!(s = calloc(1, sizeof(*s))))
        return CRAW_ERROR(ENOMEM);
    if (params)
        s->params = *params;
    else
        craw_awb_smoother_params_init(&s->params);
    q = &s->params;
    if (!(q->time_constant > 0.0f) || !(q->max_slew_mired_per_s > 0.0f) ||
        !(q->hysteresis_mired >= 0.0f) || !isfinite(q->hysteresis_mired) ||
        !isfinite(q->time_constant) || !isfinite(q->max_slew_mired_per_s) ||
        !isfinite(q->min_confidence)) {
        free(s);
        return CRAW_ERROR(EINVAL);
    }
    *sm = s;
    return 0;
}

CRAW_API void craw_awb_smoother_free(CRAWAwbSmoother **sm)
{
    if (!sm || !*sm)
        return;
    free(*sm);
    *sm = NULL;
}

CRAW_API void craw_awb_smoother_reset(CRAWAwbSmoother *sm)
{
    if (!sm)
        return;
    sm->tracking = false;
    sm->mired = sm->tint = sm->last_pts = 0.0;
}

CRAW_API void craw_awb_smoother_set(CRAWAwbSmoother *sm, double pts_s, const CRAWIlluminant *illum)
{
    if (!sm || !illum || !isfinite(illum->cct) || !(illum->cct > 0.0f) || !isfinite(illum->tint))
        return;
    sm->mired = 1e6 / (double)illum->cct;
    sm->tint = illum->tint;
    sm->tracking = true;
    sm->last_pts = pts_s;
}

CRAW_API int craw_awb_smoother_push(CRAWAwbSmoother *sm, double pts_s, const CRAWAwbEstimate *est,
                                    bool scene_cut, CRAWIlluminant *out)
{
    double dt, goal_mired = 0.0, goal_tint = 0.0;
    bool usable, confident;

    if (!sm || !est || !out)
        return CRAW_ERROR(EINVAL);
    usable = est->valid && isfinite(est->illuminant.cct) && est->illuminant.cct > 0.0f &&
             isfinite(est->illuminant.tint);
    if (usable) {
        goal_mired = 1e6 / (double)est->illuminant.cct;
        goal_tint = est->illuminant.tint;
    }
    confident = est->confidence >= sm->params.min_confidence;
    /* Presentation time since the last push, in [0, 1] s: a seek or a gap
     * is no licence for a jump, a step backwards no reason to undo one. */
    dt = sm->tracking ? pts_s - sm->last_pts : 0.0;
    if (!(dt > 0.0))
        dt = 0.0;
    if (dt > 1.0)
        dt = 1.0;

    if (usable && (!sm->tracking || (scene_cut && confident))) {
        /* Start (or, at a confident cut, restart) the track here. */
        sm->mired = goal_mired;
        sm->tint = goal_tint;
        sm->tracking = true;
    } else if (!sm->tracking) {
        return CRAW_ERROR(EAGAIN);
    } else if (usable && confident) {
        const double delta = goal_mired - sm->mired;
        if (fabs(delta) >= (double)sm->params.hysteresis_mired) {
            double frac = 1.0 - exp(-dt / (double)sm->params.time_constant);
            const double limit = (double)sm->params.max_slew_mired_per_s * dt;
            const double step = delta * frac;
            /* The slew limit scales the fraction, so the tint closes the
             * same share of its error as the temperature. */
            if (fabs(step) > limit)
                frac *= limit / fabs(step);
            sm->mired += delta * frac;
            sm->tint += (goal_tint - sm->tint) * frac;
        }
    }
    sm->last_pts = pts_s;
    out->cct = (float)(1e6 / sm->mired);
    out->tint = (float)sm->tint;
    return 0;
}
