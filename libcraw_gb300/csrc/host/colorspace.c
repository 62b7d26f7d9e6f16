/*
 * Output colour spaces (reference lib/colorspace.c:20-319): each space's
 * RGB -> XYZ matrix built in double from its published primaries and
 * white, the ACES spaces adapted from their own white to D65 with the
 * Bradford transform, and the inverse taken for XYZ -> RGB.
 */
#include <math.h>
#include <string.h>

#include <craw/profile.h>

typedef double mat3[3][3];

/* CIE 1931 xy of the primaries R, G, B of each space. */
static const double cs_prim[CRAW_CS_NB][3][2] = {
    [CRAW_CS_BT709_LINEAR]    = { { 0.64, 0.33 }, { 0.30, 0.60 }, { 0.15, 0.06 } },
    [CRAW_CS_BT2020_LINEAR]   = { { 0.708, 0.292 }, { 0.170, 0.797 }, { 0.131, 0.046 } },
    [CRAW_CS_P3D65_LINEAR]    = { { 0.680, 0.320 }, { 0.265, 0.690 }, { 0.150, 0.060 } },
    [CRAW_CS_V_GAMUT_LINEAR]  = { { 0.730, 0.280 }, { 0.165, 0.840 }, { 0.100, -0.030 } },
    [CRAW_CS_ACES_AP0_LINEAR] = { { 0.7347, 0.2653 }, { 0.0, 1.0 }, { 0.0001, -0.0770 } },
    [CRAW_CS_ACES_AP1_LINEAR] = { { 0.713, 0.293 }, { 0.165, 0.830 }, { 0.128, 0.044 } },
};
static const double white_d65[2] = { 0.3127, 0.3290 };
static const double white_aces[2] = { 0.32168, 0.33767 };

static void xy_to_xyz(const double xy[2], double o[3])
{
    o[0] = xy[0] / xy[1];
    o[1] = 1.0;
    o[2] = (1.0 - xy[0] - xy[1]) / xy[1];
}

static void mat_mul(const mat3 a, const mat3 b, mat3 o)
{
    mat3 t;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            t[i][j] = a[i][0] * b[0][j] + a[i][1] * b[1][j] + a[i][2] * b[2][j];
    memcpy(o, t, sizeof(t));
}

static void mat_vec(const mat3 m, const double v[3], double o[3])
{
    double t[3];
    for (int i = 0; i < 3; i++)
        t[i] = m[i][0] * v[0] + m[i][1] * v[1] + m[i][2] * v[2];
    memcpy(o, t, sizeof(t));
}

/* Inverse by the adjugate; EINVAL for a (near) singular matrix. */
static int mat_inv(const mat3 m, mat3 o)
{
    double c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
    double c01 = m[1][0] * m[2][2] - m[1][2] * m[2][0];
    double c02 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
    double det = m[0][0] * c00 - m[0][1] * c01 + m[0][2] * c02;
    mat3 t;
    if (!(fabs(det) > 1e-12))
        return CRAW_ERROR(EINVAL);
    t[0][0] = c00 / det;
    t[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) / det;
    t[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) / det;
    t[1][0] = -c01 / det;
    t[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) / det;
    t[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) / det;
    t[2][0] = c02 / det;
    t[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) / det;
    t[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) / det;
    memcpy(o, t, sizeof(t));
    return 0;
}

/* Columns along the primaries, scaled so that they sum to the white. */
static int rgb_to_xyz(const double prim[3][2], const double white[2], mat3 o)
{
    mat3 p, inv;
    double w[3], s[3];
    for (int c = 0; c < 3; c++) {
        double col[3];
        xy_to_xyz(prim[c], col);
        for (int i = 0; i < 3; i++)
            p[i][c] = col[i];
    }
    xy_to_xyz(white, w);
    if (mat_inv(p, inv) < 0)
        return CRAW_ERROR(EINVAL);
    mat_vec(inv, w, s);
    for (int i = 0; i < 3; i++)
        for (int c = 0; c < 3; c++)
            o[i][c] = p[i][c] * s[c];
    return 0;
}

/* von Kries scaling in the Bradford cone space. */
static int bradford(const double src[2], const double dst[2], mat3 o)
{
    static const mat3 cone = {
        {  0.8951,  0.2664, -0.1614 },
        { -0.7502,  1.7135,  0.0367 },
        {  0.0389, -0.0685,  1.0296 },
    };
    mat3 cone_inv, scale = { { 0 } }, t;
    double ws[3], wd[3], ls[3], ld[3];
    xy_to_xyz(src, ws);
    xy_to_xyz(dst, wd);
    mat_vec(cone, ws, ls);
    mat_vec(cone, wd, ld);
    for (int i = 0; i < 3; i++) {
        if (!(fabs(ls[i]) > 1e-12))
            return CRAW_ERROR(EINVAL);
        scale[i][i] = ld[i] / ls[i];
    }
    if (mat_inv(cone, cone_inv) < 0)
        return CRAW_ERROR(EINVAL);
    mat_mul(scale, cone, t);
    mat_mul(cone_inv, t, o);
    return 0;
}

static int to_xyz_d65(enum CRAWColorSpace cs, mat3 o)
{
    bool aces;
    mat3 m;
    if ((unsigned)cs >= CRAW_CS_NB)
        return CRAW_ERROR(EINVAL);
    if (cs == CRAW_CS_XYZ_D65) {
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                o[i][j] = i == j ? 1.0 : 0.0;
        return 0;
    }
    aces = cs == CRAW_CS_ACES_AP0_LINEAR || cs == CRAW_CS_ACES_AP1_LINEAR;
    if (rgb_to_xyz(cs_prim[cs], aces ? white_aces : white_d65, m) < 0)
        return CRAW_ERROR(EINVAL);
    if (aces) {
        mat3 cat;
        if (bradford(white_aces, white_d65, cat) < 0)
            return CRAW_ERROR(EINVAL);
        mat_mul(cat, m, m);
    }
    memcpy(o, m, sizeof(m));
    return 0;
}

static void store(const mat3 in, float out[3][3])
{
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            out[i][j] = (float)in[i][j];
}

CRAW_API int craw_colorspace_from_xyz_d65(enum CRAWColorSpace cs, float m[3][3])
{
    mat3 to, from;
    int ret;
    if (!m)
        return CRAW_ERROR(EINVAL);
    if ((ret = to_xyz_d65(cs, to)) < 0 || (ret = mat_inv(to, from)) < 0)
        return ret;
    store(from, m);
    return 0;
}

CRAW_API int craw_colorspace_to_xyz_d65(enum CRAWColorSpace cs, float m[3][3])
{
    mat3 to;
    int ret;
    if (!m)
        return CRAW_ERROR(EINVAL);
    if ((ret = to_xyz_d65(cs, to)) < 0)
        return ret;
    store(to, m);
    return 0;
}

/* Krystek (1985), "An algorithm to calculate correlated colour
 * temperature", Color Research & Application 10(1): the Planckian locus
 * in CIE 1960 uv as two rational functions of T, then uv -> xy. */
CRAW_API int craw_planckian_xy(float cct, float xy[2])
{
    double t, u, v, d;
    if (!xy || !isfinite(cct))
        return CRAW_ERROR(EINVAL);
    t = fmin(fmax((double)cct, 1000.0), 15000.0);
    u = (0.860117757 + 1.54118254e-4 * t + 1.28641212e-7 * t * t) /
        (1.0 + 8.42420235e-4 * t + 7.08145163e-7 * t * t);
    v = (0.317398726 + 4.22806245e-5 * t + 4.20481691e-8 * t * t) /
        (1.0 - 2.89741816e-5 * t + 1.61456053e-7 * t * t);
    d = 2.0 * u - 8.0 * v + 4.0;
    xy[0] = (float)(3.0 * u / d);
    xy[1] = (float)(2.0 * v / d);
    return 0;
}

CRAW_API int craw_bradford_adaptation(const float src[2], const float dst[2], float m[3][3])
{
    double s[2], d[2];
    mat3 cat;
    if (!src || !dst || !m)
        return CRAW_ERROR(EINVAL);
    s[0] = src[0]; s[1] = src[1];
    d[0] = dst[0]; d[1] = dst[1];
    if (!(s[1] > 0.0) || !(d[1] > 0.0))
        return CRAW_ERROR(EINVAL);
    if (bradford(s, d, cat) < 0)
        return CRAW_ERROR(EINVAL);
    store(cat, m);
    return 0;
}
