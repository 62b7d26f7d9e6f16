/*
 * Camera profile evaluation (reference lib/profile.c:19-253): identity
 * initialisation, validation, and the frame's white balance, camera
 * matrix and gain, either as shot or re-balanced at an illuminant from
 * the per-CCT tables (linear in Kelvin, in double, stored as float).
 */
#include <math.h>
#include <string.h>

#include <craw/profile.h>

#define CRAW_INV_SQRT2 0.70710678118654752440

CRAW_API void craw_profile_init(CRAWProfile *p)
{
    if (!p)
        return;
    memset(p, 0, sizeof(*p));
    p->cfa = CRAW_CFA_RGGB;
    for (int s = 0; s < 4; s++)
        p->white_level[s] = 1.0f;
    for (int c = 0; c < 3; c++) {
        p->as_shot_wb[c] = 1.0f;
        p->as_shot_matrix[c][c] = 1.0f;
    }
    p->gain = 1.0f;
}

static bool finite_all(const float *v, size_t n)
{
    for (size_t i = 0; i < n; i++)
        if (!isfinite(v[i]))
            return false;
    return true;
}

CRAW_API int craw_profile_validate(const CRAWProfile *p)
{
    if (!p || (unsigned)p->cfa > CRAW_CFA_GBRG)
        return CRAW_ERROR(EINVAL);
    for (int s = 0; s < 4; s++) {
        float b = p->black_level[s], w = p->white_level[s];
        if (!isfinite(b) || !isfinite(w) || b < 0.0f || w > 1.0f || !(w > b))
            return CRAW_ERROR(EINVAL);
    }
    if (!finite_all(p->as_shot_wb, 3) || !finite_all(&p->as_shot_matrix[0][0], 9))
        return CRAW_ERROR(EINVAL);
    for (int c = 0; c < 3; c++)
        if (!(p->as_shot_wb[c] > 0.0f))
            return CRAW_ERROR(EINVAL);
    {
        /* A singular camera matrix is always a filling mistake. */
        const float (*m)[3] = p->as_shot_matrix;
        double det = (double)m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1])
                   - (double)m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0])
                   + (double)m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
        if (!(fabs(det) > 1e-9))
            return CRAW_ERROR(EINVAL);
    }
    if (!isfinite(p->gain) || !(p->gain > 0.0f) ||
        !isfinite(p->as_shot_cct) || p->as_shot_cct < 0.0f ||
        !isfinite(p->as_shot_ei) || p->as_shot_ei < 0.0f ||
        !isfinite(p->exposure_index) || p->exposure_index < 0.0f)
        return CRAW_ERROR(EINVAL);
    if (p->nb_wb_knots > CRAW_PROFILE_MAX_KNOTS || p->nb_matrix_knots > CRAW_PROFILE_MAX_KNOTS)
        return CRAW_ERROR(EINVAL);
    for (uint32_t i = 0; i < p->nb_wb_knots; i++) {
        const CRAWWbKnot *k = &p->wb_knots[i];
        if (!isfinite(k->cct) || !(k->cct > 0.0f) || (i && !(k->cct > k[-1].cct)) ||
            !finite_all(k->wb, 3))
            return CRAW_ERROR(EINVAL);
        for (int c = 0; c < 3; c++)
            if (!(k->wb[c] > 0.0f))
                return CRAW_ERROR(EINVAL);
    }
    for (uint32_t i = 0; i < p->nb_matrix_knots; i++) {
        const CRAWMatrixKnot *k = &p->matrix_knots[i];
        if (!isfinite(k->cct) || !(k->cct > 0.0f) || (i && !(k->cct > k[-1].cct)) ||
            !finite_all(&k->m[0][0], 9))
            return CRAW_ERROR(EINVAL);
    }
    if (p->name[sizeof(p->name) - 1] != '\0')
        return CRAW_ERROR(EINVAL);
    return 0;
}

/* Index of the knot interval holding `cct` (clamped to the table) and the
 * position inside it. */
static uint32_t knot_interval(const float *cct_of, size_t stride, uint32_t nb, double cct,
                              double *frac)
{
#define CCT(i) (*(const float *)((const char *)cct_of + (size_t)(i) * stride))
    uint32_t i = 0;
    double a, b, f = 0.0;
    while (i + 2 < nb && cct >= CCT(i + 1))
        i++;
    a = CCT(i);
    b = CCT(i + 1);
    if (b > a)
        f = (cct - a) / (b - a);
    *frac = f < 0.0 ? 0.0 : (f > 1.0 ? 1.0 : f);
    return i;
#undef CCT
}

CRAW_API int craw_profile_eval(const CRAWProfile *p, enum CRAWWbMode mode,
                               const CRAWIlluminant *illum, CRAWColorParams *out)
{
    if (!p || !out)
        return CRAW_ERROR(EINVAL);
    if (mode == CRAW_WB_AS_SHOT) {
        memcpy(out->wb, p->as_shot_wb, sizeof(out->wb));
        memcpy(out->cam_to_xyz, p->as_shot_matrix, sizeof(out->cam_to_xyz));
    } else if (mode == CRAW_WB_REBALANCE) {
        uint32_t nb = p->nb_wb_knots;
        double cct, wb[3], f, tint;
        if (!illum)
            return CRAW_ERROR(EINVAL);
        if (!nb)
            return CRAW_ERROR(ENOTSUP);
        if (!isfinite(illum->cct) || !isfinite(illum->tint))
            return CRAW_ERROR(EINVAL);
        cct = fmin(fmax((double)illum->cct, (double)p->wb_knots[0].cct),
                   (double)p->wb_knots[nb - 1].cct);
        if (nb == 1) {
            for (int c = 0; c < 3; c++)
                wb[c] = p->wb_knots[0].wb[c];
        } else {
            uint32_t i = knot_interval(&p->wb_knots[0].cct, sizeof(CRAWWbKnot), nb, cct, &f);
            for (int c = 0; c < 3; c++) {
                double a = p->wb_knots[i].wb[c], b = p->wb_knots[i + 1].wb[c];
                wb[c] = a + (b - a) * f;
            }
        }
        tint = exp((double)illum->tint * CRAW_INV_SQRT2);
        wb[0] *= tint;
        wb[2] *= tint;
        for (int c = 0; c < 3; c++)
            out->wb[c] = (float)wb[c];
        if (p->nb_matrix_knots) {
            uint32_t nm = p->nb_matrix_knots;
            double mc = fmin(fmax(cct, (double)p->matrix_knots[0].cct),
                             (double)p->matrix_knots[nm - 1].cct);
            if (nm == 1) {
                memcpy(out->cam_to_xyz, p->matrix_knots[0].m, sizeof(out->cam_to_xyz));
            } else {
                uint32_t i = knot_interval(&p->matrix_knots[0].cct, sizeof(CRAWMatrixKnot), nm,
                                           mc, &f);
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++) {
                        double a = p->matrix_knots[i].m[r][c], b = p->matrix_knots[i + 1].m[r][c];
                        out->cam_to_xyz[r][c] = (float)(a + (b - a) * f);
                    }
            }
        } else {
            memcpy(out->cam_to_xyz, p->as_shot_matrix, sizeof(out->cam_to_xyz));
        }
    } else {
        return CRAW_ERROR(EINVAL);
    }
    out->gain = p->gain;
    if (p->as_shot_ei > 0.0f && p->exposure_index > 0.0f)
        out->gain *= p->exposure_index / p->as_shot_ei;
    return 0;
}

CRAW_API int craw_profile_noise_eval(const CRAWProfile *p, float iso, CRAWNoiseModel *out)
{
    if (!p || !out)
        return CRAW_ERROR(EINVAL);
    if (!p->nb_noise_knots)
        return CRAW_ERROR(ENOTSUP);
    if (!(iso > 0.0f))
        iso = p->as_shot_ei;
    return craw_noise_model_eval(p->noise_knots, p->nb_noise_knots, iso, out);
}

/* ------------------------------------------------------- white balance locus */

/* Spacing of the locus samples between two knots, in mired. */
#define LOCUS_STEP_MIRED 5.0

/* The white balance gains of the table at `cct`, linear in Kelvin between
 * knots, held at the ends. */
static void wb_gains_at(const CRAWProfile *p, double cct, double wb[3])
{
    double f;
    uint32_t i;

    if (p->nb_wb_knots == 1) {
        for (int c = 0; c < 3; c++)
            wb[c] = p->wb_knots[0].wb[c];
        return;
    }
    i = knot_interval(&p->wb_knots[0].cct, sizeof(CRAWWbKnot), p->nb_wb_knots, cct, &f);
    for (int c = 0; c < 3; c++) {
        double a = p->wb_knots[i].wb[c], b = p->wb_knots[i + 1].wb[c];
        wb[c] = a + (b - a) * f;
    }
}

/* Residual (ln R/G, ln B/G) of the neutral (lx, ly) from the locus point at
 * `cct` - the point being the inverse of the gains there - and its
 * component across the green direction, res[0] - res[1]. */
static double across_green(const CRAWProfile *p, double lx, double ly, double cct, double res[2])
{
    double wb[3];
    wb_gains_at(p, cct, wb);
    res[0] = lx + log(wb[0]);
    res[1] = ly + log(wb[2]);
    return res[0] - res[1];
}

/* The locus point that (lx, ly) lies from along the green direction: the
 * locus is sampled from the warm end to the cool one, at every knot and at
 * most LOCUS_STEP_MIRED apart in between, until the across-green residual
 * changes sign; the crossing is then bisected in mired (60 halvings, past
 * double resolution). Without a crossing the point goes to the end with
 * the smaller residual. Reference lib/profile.c:254-365. */
static int locus_along_green(const CRAWProfile *p, double lx, double ly, double *cct_out,
                             double res[2])
{
    const uint32_t nk = p->nb_wb_knots;
    double lo_cct = 0.0, lo_g = 0.0, hi_cct = 0.0;
    bool have_lo = false, crossed = false;

    for (uint32_t k = 0; k < nk && !crossed; k++) {
        const double m0 = 1e6 / p->wb_knots[k].cct;
        const double span = k + 1 < nk ? m0 - 1e6 / p->wb_knots[k + 1].cct : 0.0;
        int n = k + 1 < nk ? (int)ceil(span / LOCUS_STEP_MIRED) : 1;
        if (n < 1)
            n = 1;
        for (int j = 0; j < n; j++) {
            const double cct = 1e6 / (m0 - span * ((double)j / n));
            const double g = across_green(p, lx, ly, cct, res);
            if (g == 0.0) {
                *cct_out = cct;
                return 0;
            }
            if (have_lo && (g > 0.0) != (lo_g > 0.0)) {
                hi_cct = cct;
                crossed = true;
                break;
            }
            lo_cct = cct;
            lo_g = g;
            have_lo = true;
        }
    }
    if (!crossed) {
        double rw[2], rc[2];
        const double warm = p->wb_knots[0].cct, cool = p->wb_knots[nk - 1].cct;
        const bool take_warm = fabs(across_green(p, lx, ly, warm, rw)) <=
                               fabs(across_green(p, lx, ly, cool, rc));
        *cct_out = take_warm ? warm : cool;
        res[0] = take_warm ? rw[0] : rc[0];
        res[1] = take_warm ? rw[1] : rc[1];
        return 0;
    }
    {
        double ma = 1e6 / lo_cct, mb = 1e6 / hi_cct;
        for (int it = 0; it < 60; it++) {
            const double m = 0.5 * (ma + mb);
            const double g = across_green(p, lx, ly, 1e6 / m, res);
            if (g == 0.0) {
                ma = mb = m;
                break;
            }
            if ((g > 0.0) == (lo_g > 0.0)) {
                ma = m;
                lo_g = g;
            } else {
                mb = m;
            }
        }
        *cct_out = 1e6 / (0.5 * (ma + mb));
    }
    across_green(p, lx, ly, *cct_out, res);
    return 0;
}

CRAW_API int craw_profile_neutral_to_illuminant(const CRAWProfile *p, float raw_rg, float raw_bg,
                                                CRAWIlluminant *out)
{
    double cct, res[2];
    int ret;

    if (!out || !p)
        return CRAW_ERROR(EINVAL);
    if (!(raw_rg > 0.0f) || !(raw_bg > 0.0f) || !isfinite(raw_rg) || !isfinite(raw_bg))
        return CRAW_ERROR(EINVAL);
    if (p->nb_wb_knots < 2)
        return CRAW_ERROR(ENOTSUP);
    if ((ret = locus_along_green(p, log((double)raw_rg), log((double)raw_bg), &cct, res)) < 0)
        return ret;
    out->cct = (float)cct;
    out->tint = (float)(-(res[0] + res[1]) * CRAW_INV_SQRT2);
    return 0;
}

CRAW_API int craw_profile_illuminant_to_neutral(const CRAWProfile *p, const CRAWIlluminant *illum,
                                                float *raw_rg, float *raw_bg)
{
    double wb[3], cct, g;
    uint32_t nk;

    if (!p || !illum || !raw_rg || !raw_bg)
        return CRAW_ERROR(EINVAL);
    if (!(nk = p->nb_wb_knots))
        return CRAW_ERROR(ENOTSUP);
    if (!isfinite(illum->cct) || !isfinite(illum->tint))
        return CRAW_ERROR(EINVAL);
    cct = fmin(fmax((double)illum->cct, (double)p->wb_knots[0].cct), (double)p->wb_knots[nk - 1].cct);
    wb_gains_at(p, cct, wb);
    g = exp(-(double)illum->tint * CRAW_INV_SQRT2);
    *raw_rg = (float)(g / wb[0]);
    *raw_bg = (float)(g / wb[2]);
    return 0;
}
