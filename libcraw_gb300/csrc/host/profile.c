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
