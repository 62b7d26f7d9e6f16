/*
 * CPU oracle for the frame-development path: a restatement of the
 * reference's CPU implementation (lib/ref, and the host colour/noise/AWB
 * code it calls), in float and in double.
 *
 * TEST INFRASTRUCTURE ONLY -- the oracle, never the product. Only the
 * tests, the smoke check and bench.py's CPU-baseline leg load it. The
 * float instantiation is pinned against the reference's own build
 * (oracle/_ref, tests/golden) by the CPU test suite.
 *
 * Compiled by __graft_entry__.build() with
 *   gcc -std=c2x -O2 -fPIC -ffp-contract=off -fopenmp
 * -ffp-contract=off keeps a*b+c unfused on every host (aarch64 gcc would
 * otherwise contract to fma and drift from the x86 results).
 */
#include <errno.h>
#include <math.h>
#include <stdbool.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <craw/pipeline.h>

#include "craw_oracle.h"

#define ORC_API __attribute__((visibility("default")))

/* ---------------------------------------------------- host constants */

/* Profile evaluation, reference lib/profile.c:198-253 (knot intervals
 * 160-196, computed in double and stored as float). */
static void orc_knot_frac(double ca, double cb, double cct, double *frac)
{
    double f = 0.0;
    if (cb > ca)
        f = (cct - ca) / (cb - ca);
    *frac = f < 0.0 ? 0.0 : (f > 1.0 ? 1.0 : f);
}

ORC_API int orc_profile_eval(const CRAWProfile *p, int mode, const CRAWIlluminant *illum,
                             CRAWColorParams *out)
{
    if (!p || !out)
        return -EINVAL;
    if (mode == CRAW_WB_AS_SHOT) {
        memcpy(out->wb, p->as_shot_wb, sizeof(out->wb));
        memcpy(out->cam_to_xyz, p->as_shot_matrix, sizeof(out->cam_to_xyz));
    } else if (mode == CRAW_WB_REBALANCE) {
        double wb[3], cct, tg, f;
        uint32_t i = 0, nb = p->nb_wb_knots;
        if (!illum)
            return -EINVAL;
        if (!nb)
            return -ENOTSUP;
        if (!isfinite(illum->cct) || !isfinite(illum->tint))
            return -EINVAL;
        cct = (double)illum->cct;
        cct = cct < p->wb_knots[0].cct ? p->wb_knots[0].cct :
              (cct > p->wb_knots[nb - 1].cct ? p->wb_knots[nb - 1].cct : cct);
        if (nb == 1) {
            for (int c = 0; c < 3; c++)
                wb[c] = p->wb_knots[0].wb[c];
        } else {
            while (i + 2 < nb && cct >= p->wb_knots[i + 1].cct)
                i++;
            orc_knot_frac(p->wb_knots[i].cct, p->wb_knots[i + 1].cct, cct, &f);
            for (int c = 0; c < 3; c++) {
                double a = p->wb_knots[i].wb[c], b = p->wb_knots[i + 1].wb[c];
                wb[c] = a + (b - a) * f;
            }
        }
        tg = exp((double)illum->tint * 0.70710678118654752440);
        wb[0] *= tg;
        wb[2] *= tg;
        for (int c = 0; c < 3; c++)
            out->wb[c] = (float)wb[c];
        if (p->nb_matrix_knots) {
            uint32_t nm = p->nb_matrix_knots, k = 0;
            double mc = cct < p->matrix_knots[0].cct ? p->matrix_knots[0].cct :
                        (cct > p->matrix_knots[nm - 1].cct ? p->matrix_knots[nm - 1].cct : cct);
            if (nm == 1) {
                memcpy(out->cam_to_xyz, p->matrix_knots[0].m, sizeof(float) * 9);
            } else {
                while (k + 2 < nm && mc >= p->matrix_knots[k + 1].cct)
                    k++;
                orc_knot_frac(p->matrix_knots[k].cct, p->matrix_knots[k + 1].cct, mc, &f);
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++) {
                        double a = p->matrix_knots[k].m[r][c], b = p->matrix_knots[k + 1].m[r][c];
                        out->cam_to_xyz[r][c] = (float)(a + (b - a) * f);
                    }
            }
        } else {
            memcpy(out->cam_to_xyz, p->as_shot_matrix, sizeof(out->cam_to_xyz));
        }
    } else {
        return -EINVAL;
    }
    out->gain = p->gain;
    if (p->as_shot_ei > 0.0f && p->exposure_index > 0.0f)
        out->gain *= p->exposure_index / p->as_shot_ei;
    return 0;
}

/* Colour-space matrices in double, reference lib/colorspace.c:20-270:
 * published primaries, D65 (0.3127, 0.3290), the ACES white
 * (0.32168, 0.33767) and the Bradford cone matrix. */
static const double orc_prim[CRAW_CS_NB][3][2] = {
    [CRAW_CS_BT709_LINEAR]    = { { 0.64, 0.33 }, { 0.30, 0.60 }, { 0.15, 0.06 } },
    [CRAW_CS_BT2020_LINEAR]   = { { 0.708, 0.292 }, { 0.170, 0.797 }, { 0.131, 0.046 } },
    [CRAW_CS_P3D65_LINEAR]    = { { 0.680, 0.320 }, { 0.265, 0.690 }, { 0.150, 0.060 } },
    [CRAW_CS_V_GAMUT_LINEAR]  = { { 0.730, 0.280 }, { 0.165, 0.840 }, { 0.100, -0.030 } },
    [CRAW_CS_ACES_AP0_LINEAR] = { { 0.7347, 0.2653 }, { 0.0, 1.0 }, { 0.0001, -0.0770 } },
    [CRAW_CS_ACES_AP1_LINEAR] = { { 0.713, 0.293 }, { 0.165, 0.830 }, { 0.128, 0.044 } },
};

static void orc_xyz(double x, double y, double o[3])
{
    o[0] = x / y;
    o[1] = 1.0;
    o[2] = (1.0 - x - y) / y;
}

static void orc_mul(const double a[3][3], const double b[3][3], double o[3][3])
{
    double t[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            t[i][j] = a[i][0] * b[0][j] + a[i][1] * b[1][j] + a[i][2] * b[2][j];
    memcpy(o, t, sizeof(t));
}

static void orc_mulv(const double m[3][3], const double v[3], double o[3])
{
    double t[3];
    for (int i = 0; i < 3; i++)
        t[i] = m[i][0] * v[0] + m[i][1] * v[1] + m[i][2] * v[2];
    memcpy(o, t, sizeof(t));
}

static int orc_inv(const double m[3][3], double o[3][3])
{
    double det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1])
               - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0])
               + m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    double t[3][3];
    if (!(fabs(det) > 1e-12))
        return -EINVAL;
    t[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]) / det;
    t[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) / det;
    t[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) / det;
    t[1][0] = (m[1][2] * m[2][0] - m[1][0] * m[2][2]) / det;
    t[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) / det;
    t[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) / det;
    t[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]) / det;
    t[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) / det;
    t[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) / det;
    memcpy(o, t, sizeof(t));
    return 0;
}

static int orc_rgb_to_xyz(const double prim[3][2], const double white[2], double o[3][3])
{
    double p[3][3], inv[3][3], w[3], s[3];
    for (int c = 0; c < 3; c++) {
        double col[3];
        orc_xyz(prim[c][0], prim[c][1], col);
        for (int i = 0; i < 3; i++)
            p[i][c] = col[i];
    }
    orc_xyz(white[0], white[1], w);
    if (orc_inv(p, inv) < 0)
        return -EINVAL;
    orc_mulv(inv, w, s);
    for (int i = 0; i < 3; i++)
        for (int c = 0; c < 3; c++)
            o[i][c] = p[i][c] * s[c];
    return 0;
}

static int orc_bradford(const double src[2], const double dst[2], double o[3][3])
{
    static const double bfd[3][3] = {
        {  0.8951,  0.2664, -0.1614 },
        { -0.7502,  1.7135,  0.0367 },
        {  0.0389, -0.0685,  1.0296 },
    };
    double bi[3][3], sc[3][3] = { { 0 } }, t[3][3], ws[3], wd[3], cs[3], cd[3];
    orc_xyz(src[0], src[1], ws);
    orc_xyz(dst[0], dst[1], wd);
    orc_mulv(bfd, ws, cs);
    orc_mulv(bfd, wd, cd);
    for (int i = 0; i < 3; i++) {
        if (!(fabs(cs[i]) > 1e-12))
            return -EINVAL;
        sc[i][i] = cd[i] / cs[i];
    }
    if (orc_inv(bfd, bi) < 0)
        return -EINVAL;
    orc_mul(sc, bfd, t);
    orc_mul(bi, t, o);
    return 0;
}

static int orc_colorspace_to_xyz_d(int cs, double o[3][3])
{
    static const double d65[2] = { 0.3127, 0.3290 }, aces[2] = { 0.32168, 0.33767 };
    bool aw;
    double m[3][3];

    if (cs < 0 || cs >= CRAW_CS_NB)
        return -EINVAL;
    if (cs == CRAW_CS_XYZ_D65) {
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                o[i][j] = i == j;
        return 0;
    }
    aw = cs == CRAW_CS_ACES_AP0_LINEAR || cs == CRAW_CS_ACES_AP1_LINEAR;
    if (orc_rgb_to_xyz(orc_prim[cs], aw ? aces : d65, m) < 0)
        return -EINVAL;
    if (aw) {
        double cat[3][3];
        if (orc_bradford(aces, d65, cat) < 0)
            return -EINVAL;
        orc_mul(cat, m, m);
    }
    memcpy(o, m, sizeof(m));
    return 0;
}

ORC_API int orc_colorspace_from_xyz_d(int cs, double o[3][3])
{
    double to[3][3];
    int ret = orc_colorspace_to_xyz_d(cs, to);
    if (ret < 0)
        return ret;
    return orc_inv(to, o);
}

ORC_API int orc_colorspace_from_xyz_f(int cs, float o[3][3])
{
    double m[3][3];
    int ret = orc_colorspace_from_xyz_d(cs, m);
    if (ret < 0)
        return ret;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            o[i][j] = (float)m[i][j];
    return 0;
}

/* ACES 1.3 RGC constants from the Academy's CTL, scales solved in double,
 * reference lib/gamut.c:21-59. */
ORC_API void orc_gamut_params(struct orc_gamut *g)
{
    static const double lim[3] = { 1.147, 1.264, 1.312 };
    static const double thr[3] = { 0.815, 0.803, 0.880 };
    const double pwr = 1.2;
    for (int i = 0; i < 3; i++) {
        g->thr[i] = (float)thr[i];
        g->scl[i] = (float)((lim[i] - thr[i]) /
                            pow(pow((1.0 - thr[i]) / (lim[i] - thr[i]), -pwr) - 1.0, 1.0 / pwr));
    }
    g->pwr = (float)pwr;
    g->inv_pwr = (float)(1.0 / pwr);
}

/* Noise table evaluation, reference lib/noise.c:37-110. */
ORC_API int orc_noise_model_eval(const CRAWNoiseKnot *k, uint32_t n, float iso, CRAWNoiseModel *out)
{
    uint32_t i;
    float t;
    if (!k || !n || !out)
        return -EINVAL;
    if (!(iso > 0.0f) || !isfinite(iso)) {
        out->a = k[0].a;
        out->b = k[0].b;
        return 0;
    }
    if (iso <= k[0].iso) {
        out->a = k[0].a * (iso / k[0].iso);
        out->b = k[0].b;
        return 0;
    }
    if (iso >= k[n - 1].iso) {
        float g = iso / k[n - 1].iso;
        out->a = k[n - 1].a * g;
        out->b = k[n - 1].b * g * g;
        return 0;
    }
    for (i = 0; i + 1 < n; i++)
        if (iso <= k[i + 1].iso)
            break;
    if (!(k[i + 1].iso > k[i].iso)) {
        out->a = k[i].a;
        out->b = k[i].b;
        return 0;
    }
    t = (logf(iso) - logf(k[i].iso)) / (logf(k[i + 1].iso) - logf(k[i].iso));
    if (k[i].a > 0.0f && k[i + 1].a > 0.0f)
        out->a = expf(logf(k[i].a) + t * (logf(k[i + 1].a) - logf(k[i].a)));
    else
        out->a = k[i].a + t * (k[i + 1].a - k[i].a);
    if (k[i].b > 0.0f && k[i + 1].b > 0.0f)
        out->b = expf(logf(k[i].b) + t * (logf(k[i + 1].b) - logf(k[i].b)));
    else
        out->b = k[i].b + t * (k[i + 1].b - k[i].b);
    return 0;
}

/* The frame's noise model: the override when a > 0, else the profile's
 * table at as_shot_ei; reference lib/ref/ref_color.c:78-89,
 * lib/noise.c:112-123. */
ORC_API int orc_noise_model(const CRAWFrameParams *fp, CRAWNoiseModel *out)
{
    const CRAWProfile *p;
    float iso;
    if (!fp || !fp->profile || !out)
        return -EINVAL;
    if (fp->noise_override.a > 0.0f) {
        *out = fp->noise_override;
        return 0;
    }
    p = fp->profile;
    if (!p->nb_noise_knots)
        return -ENOTSUP;
    iso = p->as_shot_ei;
    return orc_noise_model_eval(p->noise_knots, p->nb_noise_knots, iso, out);
}

/* ------------------------------------------------ noise-model estimation */

/* Constants of reference lib/noise.c:14-27 and 145: the MAD of a unit
 * Gaussian, the Tukey cut, the floor on the residual scale, the radius of
 * the box mean. */
#define ORC_NE_MAD 0.674489750196081746f
#define ORC_NE_TUKEY 4.685
#define ORC_NE_FLOOR 0.02
#define ORC_NE_R 4

static int orc_cmp_f(const void *a, const void *b)
{
    float x = *(const float *)a, y = *(const float *)b;
    return (x > y) - (x < y);
}

static int orc_cmp_d(const void *a, const void *b)
{
    double x = *(const double *)a, y = *(const double *)b;
    return (x > y) - (x < y);
}

/* Sum of the `keep` smallest of v[0..n) (sorted in place, ascending). */
static double orc_ne_trimmed(double *v, int n, int keep)
{
    double s = 0.0;
    qsort(v, (size_t)n, sizeof(*v), orc_cmp_d);
    for (int k = 0; k < keep; k++)
        s += v[k];
    return s;
}

/* Median |x| of x[0..n) times 1.4826 (the Gaussian sigma), floored. */
static double orc_ne_scale(const double *x, int n, double *work)
{
    double s;
    for (int k = 0; k < n; k++)
        work[k] = fabs(x[k]);
    qsort(work, (size_t)n, sizeof(*work), orc_cmp_d);
    s = 1.4826 * work[n / 2];
    return s < ORC_NE_FLOOR ? ORC_NE_FLOOR : s;
}

/* Estimate of var = a u + b from one RGGB frame: reference
 * lib/noise.c:338-504 (binning 396-450, bin statistics 452-467), the
 * least-trimmed-squares seed 187-250 and the reweighted Gauss-Newton
 * 252-336. Bin sums follow the reference's sample order (plane, row,
 * column) so that the bin means are its doubles bit for bit. */
ORC_API int orc_noise_estimate(const uint16_t *bayer, uint32_t width, uint32_t height,
                               size_t stride, const CRAWProfile *pr,
                               const CRAWNoiseEstimateParams *params, CRAWNoiseEstimate *out)
{
    uint32_t nbins, min_n;
    float maxl;
    int w2, h2, ret = 0, nb = 0, nin = 0;
    float *plane = NULL, *res = NULL;
    uint16_t *lab = NULL;
    size_t *cnt = NULL, *start = NULL, ns = 0;
    double *msum = NULL, *m = NULL, *v = NULL, *c = NULL, *work = NULL, *rr = NULL;
    double a = 0.0, b = 0.0, best = INFINITY, scale, la, lb, rms = 0.0, range0;

    if (!bayer || !pr || !out)
        return -EINVAL;
    if (pr->cfa != CRAW_CFA_RGGB)
        return -ENOTSUP;
    if ((width & 1) || (height & 1) || width < 32 || height < 32 || stride < width)
        return -EINVAL;
    nbins = params && params->nb_bins ? params->nb_bins : 128;
    min_n = params && params->min_bin_samples ? params->min_bin_samples : 20000;
    maxl = params && params->max_level > 0.0f ? params->max_level : 0.98f;
    if (nbins < 8 || nbins > CRAW_NOISE_MAX_BINS)
        return -EINVAL;
    for (int s = 0; s < 4; s++)
        if (!(pr->white_level[s] > pr->black_level[s]))
            return -EINVAL;
    w2 = (int)width / 2;
    h2 = (int)height / 2;
    if (w2 < 2 * ORC_NE_R + 1 || h2 < 2 * ORC_NE_R + 1)
        return -EINVAL;

    ns = (size_t)4 * (size_t)(w2 - 2 * ORC_NE_R) * (size_t)(h2 - 2 * ORC_NE_R);
    plane = malloc((size_t)w2 * h2 * sizeof(*plane));
    res = malloc(ns * sizeof(*res));
    lab = malloc(ns * sizeof(*lab));
    cnt = calloc(nbins, sizeof(*cnt));
    start = calloc(nbins + 1, sizeof(*start));
    msum = calloc(nbins, sizeof(*msum));
    m = malloc(nbins * sizeof(*m));
    v = malloc(nbins * sizeof(*v));
    c = malloc(nbins * sizeof(*c));
    work = malloc(nbins * sizeof(*work));
    rr = malloc(nbins * sizeof(*rr));
    if (!plane || !res || !lab || !cnt || !start || !msum || !m || !v || !c || !work || !rr) {
        ret = -ENOMEM;
        goto done;
    }

    /* Every interior sample of every plane: its |high-pass| and its bin
     * (0xffff: not binned). */
    ns = 0;
    for (int s = 0; s < 4; s++) {
        const int px = s & 1, py = s >> 1;
        const double black = pr->black_level[s];
        const double range = pr->white_level[s] - pr->black_level[s];
        for (int k = 0; k < h2; k++)
            for (int i = 0; i < w2; i++) {
                const double raw = bayer[(size_t)(2 * k + py) * stride + 2 * i + px] * (1.0 / 65535.0);
                plane[(size_t)k * w2 + i] = (float)((raw - black) / range);
            }
        for (int k = ORC_NE_R; k < h2 - ORC_NE_R; k++)
            for (int i = ORC_NE_R; i < w2 - ORC_NE_R; i++, ns++) {
                const float *p = plane + (size_t)k * w2 + i;
                float hp, mean = 0.0f;
                int bi;
                hp = (p[-w2 - 1] + p[-w2 + 1] + p[w2 - 1] + p[w2 + 1] -
                      2.0f * (p[-w2] + p[w2] + p[-1] + p[1]) + 4.0f * p[0]) * (1.0f / 6.0f);
                for (int dy = -ORC_NE_R; dy <= ORC_NE_R; dy++)
                    for (int dx = -ORC_NE_R; dx <= ORC_NE_R; dx++)
                        mean += p[dy * w2 + dx];
                mean *= 1.0f / 81;
                lab[ns] = 0xffff;
                if (!(mean > 0.0f) || mean > maxl)
                    continue;
                bi = (int)(sqrtf(mean) * (float)nbins);
                bi = bi < 0 ? 0 : (bi > (int)nbins - 1 ? (int)nbins - 1 : bi);
                lab[ns] = (uint16_t)bi;
                res[ns] = fabsf(hp);
                cnt[bi]++;
                msum[bi] += mean;
            }
    }

    /* Group the residuals by bin (counting sort), then each bin's median. */
    for (uint32_t i = 0; i < nbins; i++)
        start[i + 1] = start[i] + cnt[i];
    {
        float *grp = malloc((start[nbins] ? start[nbins] : 1) * sizeof(*grp));
        size_t *fill = calloc(nbins, sizeof(*fill));
        if (!grp || !fill) {
            free(grp);
            free(fill);
            ret = -ENOMEM;
            goto done;
        }
        for (size_t j = 0; j < ns; j++)
            if (lab[j] != 0xffff)
                grp[start[lab[j]] + fill[lab[j]]++] = res[j];
        for (uint32_t i = 0; i < nbins; i++) {
            double sigma;
            if (cnt[i] < min_n)
                continue;
            qsort(grp + start[i], cnt[i], sizeof(*grp), orc_cmp_f);
            sigma = grp[start[i] + cnt[i] / 2] / ORC_NE_MAD;
            if (!(sigma > 0.0))
                continue;
            m[nb] = msum[i] / (double)cnt[i];
            v[nb] = sigma * sigma;
            c[nb] = (double)cnt[i];
            nb++;
        }
        free(grp);
        free(fill);
    }
    if (nb < 3) {
        ret = -ENODATA;
        goto done;
    }

    /* Seed: the physical line through two bins whose two-thirds smallest
     * squared log residuals sum least (first found on a tie). */
    {
        const int keep = nb * 2 / 3 + 1;
        for (int i = 0; i < nb; i++)
            for (int j = i + 1; j < nb; j++) {
                double sa, sb, cost;
                if (m[j] - m[i] < 1e-5)
                    continue;
                sa = (v[j] - v[i]) / (m[j] - m[i]);
                sb = v[i] - sa * m[i];
                if (!(sa > 0.0) || sb < 0.0)
                    continue;
                for (int k = 0; k < nb; k++) {
                    const double d = log(v[k]) - log(sa * m[k] + sb);
                    work[k] = d * d;
                }
                cost = orc_ne_trimmed(work, nb, keep);
                if (cost < best) {
                    best = cost;
                    a = sa;
                    b = sb;
                }
            }
        if (!(a > 0.0)) {
            ret = -ENODATA;
            goto done;
        }
        scale = sqrt(best / keep);
    }

    /* Refinement in (ln a, ln b): 40 damped Gauss-Newton steps at most,
     * Tukey weights times ln(1 + count), the scale re-measured every 8. */
    la = log(a);
    lb = log(b > 1e-16 ? b : 1e-16);
    if (scale < ORC_NE_FLOOR)
        scale = ORC_NE_FLOOR;
    for (int it = 0; it < 40; it++) {
        const double ea = exp(la), eb = exp(lb);
        double saa = 0.0, sab = 0.0, sbb = 0.0, ra = 0.0, rb = 0.0, det, d0, d1, cut;
        for (int k = 0; k < nb; k++)
            rr[k] = log(v[k]) - log(ea * m[k] + eb);
        if ((it & 7) == 0)
            scale = orc_ne_scale(rr, nb, work);
        cut = ORC_NE_TUKEY * scale;
        for (int k = 0; k < nb; k++) {
            const double den = ea * m[k] + eb, ja = ea * m[k] / den, jb = eb / den;
            const double u = rr[k] / cut;
            double w = fabs(u) < 1.0 ? (1.0 - u * u) * (1.0 - u * u) : 0.0;
            w *= log(1.0 + c[k]);
            saa += w * ja * ja;
            sab += w * ja * jb;
            sbb += w * jb * jb;
            ra += w * ja * rr[k];
            rb += w * jb * rr[k];
        }
        det = (saa + 1e-9) * (sbb + 1e-9) - sab * sab;
        if (!(fabs(det) > 1e-30))
            break;
        d0 = ((sbb + 1e-9) * ra - sab * rb) / det;
        d1 = (-sab * ra + (saa + 1e-9) * rb) / det;
        d0 = d0 < -0.5 ? -0.5 : (d0 > 0.5 ? 0.5 : d0);
        d1 = d1 < -0.5 ? -0.5 : (d1 > 0.5 ? 0.5 : d1);
        la += d0;
        lb += d1;
        if (lb < -40.0)
            lb = -40.0;
        if (fabs(d0) < 1e-9 && fabs(d1) < 1e-9)
            break;
    }
    a = exp(la);
    b = lb <= -40.0 ? 0.0 : exp(lb);

    for (int k = 0; k < nb; k++) {
        const double d = log(v[k]) - log(a * m[k] + b);
        if (fabs(d) < 0.35) {
            rms += d * d;
            nin++;
        }
    }
    rms = sqrt(rms / (nin ? nin : 1));
    range0 = pr->white_level[0] - pr->black_level[0];
    memset(out, 0, sizeof(*out));
    out->model.a = (float)a;
    out->model.b = (float)b;
    out->nb_bins = (uint32_t)nb;
    out->nb_inliers = (uint32_t)nin;
    out->fit_rms = (float)rms;
    out->read_noise_lsb = (float)(sqrt(b) * range0 * 65535.0);
done:
    free(plane);
    free(res);
    free(lab);
    free(cnt);
    free(start);
    free(msum);
    free(m);
    free(v);
    free(c);
    free(work);
    free(rr);
    return ret;
}

/* AWB histogram of 8x8 block means, reference lib/awb.c:213-296. */
ORC_API int orc_awb_histogram(const float *rgb, uint32_t width, uint32_t height, size_t stride,
                              int channels, const float wb[3], uint32_t *count,
                              uint32_t *weight, uint32_t *weight_bright)
{
    const uint32_t bins = 128;
    const float lmin = -2.5f, lmax = 1.0f;

    if (!rgb || !wb || !count || !weight || !weight_bright)
        return -EINVAL;
    if (channels != 3 && channels != 4)
        return -EINVAL;
    if (stride < (size_t)width * (size_t)channels)
        return -EINVAL;
    if (!(wb[0] > 0.0f) || !(wb[2] > 0.0f))
        return -EINVAL;
    memset(count, 0, (size_t)bins * bins * 4);
    memset(weight, 0, (size_t)bins * bins * 4);
    memset(weight_bright, 0, (size_t)bins * bins * 4);
    for (uint32_t by = 0; by < height; by += 8) {
        uint32_t y1 = by + 8 < height ? by + 8 : height;
        for (uint32_t bx = 0; bx < width; bx += 8) {
            uint32_t x1 = bx + 8 < width ? bx + 8 : width;
            float acc[3] = { 0.0f, 0.0f, 0.0f };
            float n = (float)((y1 - by) * (x1 - bx));
            float r, g, b, rr, bb, x, y, w, span = lmax - lmin;
            int ix, iy;
            for (uint32_t py = by; py < y1; py++) {
                const float *row = rgb + (size_t)py * stride;
                for (uint32_t px = bx; px < x1; px++) {
                    acc[0] += row[(size_t)px * channels + 0];
                    acc[1] += row[(size_t)px * channels + 1];
                    acc[2] += row[(size_t)px * channels + 2];
                }
            }
            r = acc[0] / n;
            g = acc[1] / n;
            b = acc[2] / n;
            if (fmaxf(fmaxf(r, g), b) >= 0.98f || g < 0.002f)
                continue;
            rr = (r / wb[0]) / g;
            bb = (b / wb[2]) / g;
            x = logf(rr);
            y = logf(bb);
            x = x > lmin ? (x < lmax ? x : lmax) : lmin;
            y = y > lmin ? (y < lmax ? y : lmax) : lmin;
            ix = (int)floorf((x - lmin) / span * bins);
            iy = (int)floorf((y - lmin) / span * bins);
            ix = ix < 0 ? 0 : (ix > (int)bins - 1 ? (int)bins - 1 : ix);
            iy = iy < 0 ? 0 : (iy > (int)bins - 1 ? (int)bins - 1 : iy);
            w = g < 0.5f ? g : 0.5f;
            count[iy * bins + ix] += 1;
            weight[iy * bins + ix] += (uint32_t)roundf(w * 65536.0f);
            weight_bright[iy * bins + ix] += (uint32_t)roundf(g * g * g * g * 65536.0f);
        }
    }
    return 0;
}

/* Rounds a float to the nearest binary16 value, ties to even, returned as a
 * float: the storage format of the rebuilt highlight mosaic (reference
 * lib/ref/ref.h:20-57 rounds the same way; magnitudes beyond the half range
 * do not occur there). */
static inline float orc_to_half(float f)
{
    uint32_t b, sign, mag, keep, rem;

    memcpy(&b, &f, sizeof(b));
    sign = b & 0x80000000u;
    mag = b & 0x7FFFFFFFu;
    if (mag == 0 || mag >= 0x7F800000u)
        return f;
    if ((int)(mag >> 23) - 127 < -14) {
        /* A half subnormal: a multiple of 2^-24. */
        float q = rintf(fabsf(f) * 16777216.0f) / 16777216.0f;
        return sign ? -q : q;
    }
    /* Ten mantissa bits kept, the other thirteen rounded to nearest even;
     * a carry out of the mantissa moves into the exponent. */
    keep = mag >> 13;
    rem = mag & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (keep & 1u)))
        keep++;
    b = sign | (keep << 13);
    memcpy(&f, &b, sizeof(f));
    return f;
}

/* ------------------------------------------------- the two instantiations */

static inline float orc_mstore_f32(double x) { return (float)x; }
static inline double orc_mstore_f64(double x) { return x; }

#define R float
#define SFX(n) ORC_API_F32(n)
#define ORC_API_F32(n) n##_f32
#define R_SQRT sqrtf
#define R_EXP expf
#define R_EXP2 exp2f
#define R_LOG logf
#define R_POW powf
#define R_RINT rintf
#define R_FABS fabsf
#define R_FLOOR floorf
#include "oracle_impl.h"
#undef R
#undef SFX
#undef R_SQRT
#undef R_EXP
#undef R_EXP2
#undef R_LOG
#undef R_POW
#undef R_RINT
#undef R_FABS
#undef R_FLOOR
#undef ORC_DN_S
#undef ORC_DN_P
#undef ORC_DN_GUARD_LO
#undef ORC_DN_GUARD_HI
#undef ORC_DN_VAR_MIN
#undef ORC_RCD_EPS
#undef ORC_CD_RADIUS
#undef ORC_CD_INV_2S2
#undef ORC_CD_RANGE_K
#undef ORC_CD_CHROMA_K
#undef ORC_CD_RANGE_EPS
#undef ORC_HL_U_LO
#undef ORC_HL_U_HI
#undef ORC_HL_EPS
#undef ORC_HL_LOG_MAX
#undef ORC_HL_W_SAT
#undef ORC_HL_DILATE
#undef ORC_HL_LEVELS

#define R double
#define SFX(n) ORC_API_F64(n)
#define ORC_API_F64(n) n##_f64
#define R_SQRT sqrt
#define R_EXP exp
#define R_EXP2 exp2
#define R_LOG log
#define R_POW pow
#define R_RINT rint
#define R_FABS fabs
#define R_FLOOR floor
#include "oracle_impl.h"
