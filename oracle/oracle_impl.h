/*
 * Oracle restatement of the reference's CPU implementation of the
 * frame-development path, written once over a scalar type R and
 * instantiated twice by craw_oracle.c: in float, where it follows the
 * reference's float arithmetic operation for operation, and in double, the
 * FP64 run the GPU results are also measured against.
 *
 * TEST INFRASTRUCTURE ONLY: only tests/, the smoke check and the
 * CPU-baseline leg of bench.py may use it, as the oracle the GPU results
 * are compared with, and never as the thing measured or shipped.
 *
 * Every function cites the reference file:line it restates.
 * Expected macros: R (float or double), SFX(name) (name##_f32 / _f64),
 * R_SQRT, R_EXP, R_LOG, R_POW, R_RINT, R_FABS, R_FLOOR.
 */

/* ------------------------------------------------------------ borders */

/* Mirror without repeating the edge sample, looping for stencils wider
 * than the image; reference lib/ref/ref_debayer.c:21-34 (the plane mirror
 * of lib/ref/ref_denoise.c:63-76 is the same function). */
static inline int SFX(orc_mirror)(int v, int n)
{
    if (n < 2)
        return 0;
    while (v < 0 || v >= n) {
        if (v < 0)
            v = -v;
        if (v >= n)
            v = 2 * n - 2 - v;
    }
    return v;
}

static inline R SFX(orc_at)(const R *p, int w, int h, int x, int y)
{
    return p[(size_t)SFX(orc_mirror)(y, h) * w + SFX(orc_mirror)(x, w)];
}

/* --------------------------------------------------------------- prep */

/* Normalise, white balance, clip at 1.0: reference
 * lib/ref/ref_debayer.c:42-63. Channel of site s for RGGB is 0,1,1,2. */
static void SFX(orc_prep)(const uint16_t *bayer, int w, int h, size_t stride,
                          const CRAWProfile *p, const R wb[3], R *v)
{
    static const int chan[4] = { 0, 1, 1, 2 };
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            int s = (y & 1) * 2 + (x & 1);
            R raw = (R)bayer[(size_t)y * stride + x] * ((R)1 / (R)65535);
            R t = (raw - (R)p->black_level[s]) /
                  ((R)p->white_level[s] - (R)p->black_level[s]);
            t *= wb[chan[s]];
            v[(size_t)y * w + x] = t < (R)1 ? t : (R)1;
        }
    }
}

/* ----------------------------------------------------------- debayers */

#define ORC_V(dx, dy) SFX(orc_at)(v, w, h, x + (dx), y + (dy))

/* Bilinear, reference lib/ref/ref_debayer.c:65-96. */
static void SFX(orc_bilinear)(const R *v, int w, int h, R *rgb)
{
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            R *o = &rgb[((size_t)y * w + x) * 4];
            int s = (y & 1) * 2 + (x & 1);
            R edge = (R)0.25 * (ORC_V(0, -1) + ORC_V(0, 1) + ORC_V(-1, 0) + ORC_V(1, 0));
            R corner = (R)0.25 * (ORC_V(-1, -1) + ORC_V(1, -1) + ORC_V(-1, 1) + ORC_V(1, 1));
            R horiz = (R)0.5 * (ORC_V(-1, 0) + ORC_V(1, 0));
            R vert = (R)0.5 * (ORC_V(0, -1) + ORC_V(0, 1));
            R c = ORC_V(0, 0);
            if (s == 0)      { o[0] = c;      o[1] = edge; o[2] = corner; }
            else if (s == 1) { o[0] = horiz;  o[1] = c;    o[2] = vert; }
            else if (s == 2) { o[0] = vert;   o[1] = c;    o[2] = horiz; }
            else             { o[0] = corner; o[1] = edge; o[2] = c; }
            o[3] = 1;
        }
    }
}

/* Malvar-He-Cutler kernels, reference lib/ref/ref_debayer.c:98-176. */
static inline R SFX(orc_mhc_g)(const R *v, int w, int h, int x, int y)
{
    return ((R)4 * ORC_V(0, 0)
            + (R)2 * (ORC_V(0, -1) + ORC_V(0, 1) + ORC_V(-1, 0) + ORC_V(1, 0))
            - (ORC_V(0, -2) + ORC_V(0, 2) + ORC_V(-2, 0) + ORC_V(2, 0))) * (R)0.125;
}

static inline R SFX(orc_mhc_h)(const R *v, int w, int h, int x, int y)
{
    return ((R)5 * ORC_V(0, 0)
            + (R)4 * (ORC_V(-1, 0) + ORC_V(1, 0))
            - (ORC_V(-1, -1) + ORC_V(1, -1) + ORC_V(-1, 1) + ORC_V(1, 1) + ORC_V(-2, 0) + ORC_V(2, 0))
            + (R)0.5 * (ORC_V(0, -2) + ORC_V(0, 2))) * (R)0.125;
}

static inline R SFX(orc_mhc_v)(const R *v, int w, int h, int x, int y)
{
    return ((R)5 * ORC_V(0, 0)
            + (R)4 * (ORC_V(0, -1) + ORC_V(0, 1))
            - (ORC_V(-1, -1) + ORC_V(1, -1) + ORC_V(-1, 1) + ORC_V(1, 1) + ORC_V(0, -2) + ORC_V(0, 2))
            + (R)0.5 * (ORC_V(-2, 0) + ORC_V(2, 0))) * (R)0.125;
}

static inline R SFX(orc_mhc_d)(const R *v, int w, int h, int x, int y)
{
    return ((R)6 * ORC_V(0, 0)
            + (R)2 * (ORC_V(-1, -1) + ORC_V(1, -1) + ORC_V(-1, 1) + ORC_V(1, 1))
            - (R)1.5 * (ORC_V(0, -2) + ORC_V(0, 2) + ORC_V(-2, 0) + ORC_V(2, 0))) * (R)0.125;
}

static void SFX(orc_mhc)(const R *v, int w, int h, R *rgb)
{
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            R *o = &rgb[((size_t)y * w + x) * 4];
            int s = (y & 1) * 2 + (x & 1);
            R c = ORC_V(0, 0);
            if (s == 0) {
                o[0] = c;
                o[1] = SFX(orc_mhc_g)(v, w, h, x, y);
                o[2] = SFX(orc_mhc_d)(v, w, h, x, y);
            } else if (s == 1) {
                o[0] = SFX(orc_mhc_h)(v, w, h, x, y);
                o[1] = c;
                o[2] = SFX(orc_mhc_v)(v, w, h, x, y);
            } else if (s == 2) {
                o[0] = SFX(orc_mhc_v)(v, w, h, x, y);
                o[1] = c;
                o[2] = SFX(orc_mhc_h)(v, w, h, x, y);
            } else {
                o[0] = SFX(orc_mhc_d)(v, w, h, x, y);
                o[1] = SFX(orc_mhc_g)(v, w, h, x, y);
                o[2] = c;
            }
            o[3] = 1;
        }
    }
}

/* 3x3 mean, mirrored: reference lib/ref/ref_debayer.c:178-190. */
static inline R SFX(orc_box3)(const R *s, int w, int h, int x, int y)
{
    R acc = 0;
    for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++)
            acc += SFX(orc_at)(s, w, h, x + dx, y + dy);
    return acc * ((R)1 / (R)9);
}

#define ORC_RCD_EPS ((R)1e-5f)

/* The low-pass ratio correction, reference lib/ref/ref_debayer.c:192-202. */
static inline R SFX(orc_rcd_ratio)(R a, R b)
{
    a = a > 0 ? a : 0;
    b = b > 0 ? b : 0;
    return (a - b) / (a + b + ORC_RCD_EPS);
}

/* RCD in full-image sweeps, reference lib/ref/ref_debayer.c:204-395. */
static int SFX(orc_rcd)(const R *v, int w, int h, R *rgb)
{
    size_t n = (size_t)w * h;
    R *lp = malloc(n * sizeof(R)), *wv = malloc(n * sizeof(R)), *wp = malloc(n * sizeof(R));
    R *gp = malloc(n * sizeof(R)), *cp = calloc(n, sizeof(R));
    R *ga = malloc(n * sizeof(R)), *gb = malloc(n * sizeof(R));
    int ret = 0;

    if (!lp || !wv || !wp || !gp || !cp || !ga || !gb) {
        ret = -ENOMEM;
        goto done;
    }
#define ORC_L(dx, dy) SFX(orc_at)(lp, w, h, x + (dx), y + (dy))
#define ORC_G(dx, dy) SFX(orc_at)(gp, w, h, x + (dx), y + (dy))
#define ORC_C(dx, dy) SFX(orc_at)(cp, w, h, x + (dx), y + (dy))
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++)
            lp[(size_t)y * w + x] =
                ((R)4 * ORC_V(0, 0)
                 + (R)2 * (ORC_V(0, -1) + ORC_V(0, 1) + ORC_V(-1, 0) + ORC_V(1, 0))
                 + ORC_V(-1, -1) + ORC_V(1, -1) + ORC_V(-1, 1) + ORC_V(1, 1)) * ((R)1 / (R)16);

    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            size_t i = (size_t)y * w + x;
            ga[i] = R_FABS(ORC_V(0, -1) - ORC_V(0, 1))
                  + R_FABS((R)2 * ORC_V(0, 0) - ORC_V(0, -2) - ORC_V(0, 2));
            gb[i] = R_FABS(ORC_V(-1, 0) - ORC_V(1, 0))
                  + R_FABS((R)2 * ORC_V(0, 0) - ORC_V(-2, 0) - ORC_V(2, 0));
        }
    }
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            R vs = SFX(orc_box3)(ga, w, h, x, y);
            R hs = SFX(orc_box3)(gb, w, h, x, y);
            wv[(size_t)y * w + x] = hs / (hs + vs + ORC_RCD_EPS);
        }
    }
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            size_t i = (size_t)y * w + x;
            ga[i] = R_FABS(ORC_V(-1, 1) - ORC_V(1, -1))
                  + R_FABS((R)2 * ORC_V(0, 0) - ORC_V(-2, 2) - ORC_V(2, -2));
            gb[i] = R_FABS(ORC_V(-1, -1) - ORC_V(1, 1))
                  + R_FABS((R)2 * ORC_V(0, 0) - ORC_V(-2, -2) - ORC_V(2, 2));
        }
    }
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            R ps = SFX(orc_box3)(ga, w, h, x, y);
            R qs = SFX(orc_box3)(gb, w, h, x, y);
            wp[(size_t)y * w + x] = qs / (ps + qs + ORC_RCD_EPS);
        }
    }

    /* Green at the R and B sites. */
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            size_t i = (size_t)y * w + x;
            int s = (y & 1) * 2 + (x & 1);
            R l00, gv, gh, wt;
            if (s == 1 || s == 2) {
                gp[i] = v[i];
                continue;
            }
            l00 = ORC_L(0, 0);
            gv = (R)0.5 * (ORC_V(0, -1) * ((R)1 + SFX(orc_rcd_ratio)(l00, ORC_L(0, -2)))
                         + ORC_V(0, 1) * ((R)1 + SFX(orc_rcd_ratio)(l00, ORC_L(0, 2))));
            gh = (R)0.5 * (ORC_V(-1, 0) * ((R)1 + SFX(orc_rcd_ratio)(l00, ORC_L(-2, 0)))
                         + ORC_V(1, 0) * ((R)1 + SFX(orc_rcd_ratio)(l00, ORC_L(2, 0))));
            wt = wv[i];
            gp[i] = wt * gv + ((R)1 - wt) * gh;
        }
    }

    /* The missing colour at the R and B sites. */
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            size_t i = (size_t)y * w + x;
            int s = (y & 1) * 2 + (x & 1);
            R g00, c, wt;
            R *o = &rgb[i * 4];
            if (s == 1 || s == 2)
                continue;
            g00 = gp[i];
            wt = wp[i];
            c = wt * (g00 + (R)0.5 * ((ORC_V(-1, 1) - ORC_G(-1, 1)) + (ORC_V(1, -1) - ORC_G(1, -1))))
              + ((R)1 - wt) * (g00 + (R)0.5 * ((ORC_V(-1, -1) - ORC_G(-1, -1)) + (ORC_V(1, 1) - ORC_G(1, 1))));
            cp[i] = c;
            o[0] = s == 0 ? v[i] : c;
            o[1] = g00;
            o[2] = s == 0 ? c : v[i];
            o[3] = 1;
        }
    }

    /* Both missing colours at the G sites. */
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            size_t i = (size_t)y * w + x;
            int s = (y & 1) * 2 + (x & 1);
            R g00, wt, dh, dv, eh, ev, ch, cv;
            R *o = &rgb[i * 4];
            if (s == 0 || s == 3)
                continue;
            g00 = gp[i];
            wt = wv[i];
            dh = (R)0.5 * ((ORC_V(-1, 0) - ORC_G(-1, 0)) + (ORC_V(1, 0) - ORC_G(1, 0)));
            ev = (R)0.5 * ((ORC_C(0, -1) - ORC_G(0, -1)) + (ORC_C(0, 1) - ORC_G(0, 1)));
            ch = wt * (g00 + ev) + ((R)1 - wt) * (g00 + dh);
            dv = (R)0.5 * ((ORC_V(0, -1) - ORC_G(0, -1)) + (ORC_V(0, 1) - ORC_G(0, 1)));
            eh = (R)0.5 * ((ORC_C(-1, 0) - ORC_G(-1, 0)) + (ORC_C(1, 0) - ORC_G(1, 0)));
            cv = wt * (g00 + dv) + ((R)1 - wt) * (g00 + eh);
            o[0] = s == 1 ? ch : cv;
            o[1] = v[i];
            o[2] = s == 1 ? cv : ch;
            o[3] = 1;
        }
    }
#undef ORC_L
#undef ORC_G
#undef ORC_C
done:
    free(lp); free(wv); free(wp); free(gp); free(cp); free(ga); free(gb);
    return ret;
}
#undef ORC_V

/* Debayer of a prepped mosaic, reference lib/ref/ref_debayer.c:436-455. */
ORC_API int SFX(orc_debayer_mosaic)(const R *v, uint32_t width, uint32_t height,
                            int method, R *rgb)
{
    int w = (int)width, h = (int)height;

    if (!v || !rgb || w < 2 || h < 2 || (w & 1) || (h & 1))
        return -EINVAL;
    switch (method) {
    case CRAW_DEBAYER_BILINEAR: SFX(orc_bilinear)(v, w, h, rgb); return 0;
    case CRAW_DEBAYER_MHC:      SFX(orc_mhc)(v, w, h, rgb); return 0;
    case CRAW_DEBAYER_RCD:      return SFX(orc_rcd)(v, w, h, rgb);
    default:                    return -EINVAL;
    }
}

/* Prep then debayer, reference lib/ref/ref_debayer.c:397-434. */
ORC_API int SFX(orc_debayer_wb)(const uint16_t *bayer, uint32_t width, uint32_t height,
                        size_t stride, const CRAWProfile *profile,
                        const float wb[3], int method, R *rgb)
{
    R wbr[3], *v;
    int ret;

    if (!bayer || !profile || !wb || !rgb)
        return -EINVAL;
    if ((unsigned)method >= CRAW_DEBAYER_NB)
        return -EINVAL;
    if (profile->cfa != CRAW_CFA_RGGB)
        return -ENOTSUP;
    if (width < 2 || height < 2 || (width & 1) || (height & 1) || stride < width)
        return -EINVAL;
    for (int s = 0; s < 4; s++)
        if (!(profile->white_level[s] > profile->black_level[s]))
            return -EINVAL;
    for (int c = 0; c < 3; c++)
        wbr[c] = (R)wb[c];
    v = malloc((size_t)width * height * sizeof(R));
    if (!v)
        return -ENOMEM;
    SFX(orc_prep)(bayer, (int)width, (int)height, stride, profile, wbr, v);
    ret = SFX(orc_debayer_mosaic)(v, width, height, method, rgb);
    free(v);
    return ret;
}

/* ------------------------------------------------------------ denoise */

#define ORC_DN_S 3                 /* search radius, reference pipeline.c:261 */
#define ORC_DN_P 1                 /* patch radius, reference pipeline.c:262 */
#define ORC_DN_GUARD_LO ((R)0.90f) /* reference ref_denoise.c:20 */
#define ORC_DN_GUARD_HI ((R)1.00f)
#define ORC_DN_VAR_MIN ((R)1.0e-4f)

/* The generalised Anscombe transform and its constants, reference
 * lib/ref/ref_denoise.c:25-58. */
struct SFX(orc_gat) { R a, c, sc, fwd, inv, off, t0; };

static void SFX(orc_gat_init)(struct SFX(orc_gat) *g, R a, R b)
{
    g->a = a;
    g->c = (R)3 * a * a / (R)8 + (b > 0 ? b : 0);
    g->sc = R_SQRT(g->c);
    g->fwd = (R)2 / a;
    g->inv = a / (R)4;
    g->off = g->c / a;
    g->t0 = g->fwd * g->sc;
}

static inline R SFX(orc_gat_fwd)(const struct SFX(orc_gat) *g, R u)
{
    if (u >= 0)
        return g->fwd * R_SQRT(g->a * u + g->c);
    return g->t0 + u / g->sc;
}

static inline R SFX(orc_gat_inv)(const struct SFX(orc_gat) *g, R t)
{
    if (t >= g->t0)
        return g->inv * t * t - g->off;
    return (t - g->t0) * g->sc;
}

/* Temporal weight of the previous frame at plane sample (i, k): 3x3 of
 * (prev - cur)^2, reference lib/ref/ref_denoise.c:78-99. */
static R SFX(orc_alpha)(const R *cur, const R *prev, int w2, int h2, int i, int k,
                        R alpha_max, R inv_h2)
{
    R d2 = 0;
    for (int ky = -1; ky <= 1; ky++) {
        for (int kx = -1; kx <= 1; kx++) {
            size_t n = (size_t)SFX(orc_mirror)(k + ky, h2) * w2 + SFX(orc_mirror)(i + kx, w2);
            R e = prev[n] - cur[n];
            d2 += e * e;
        }
    }
    R x = d2 * ((R)1 / (R)9) * inv_h2 - (R)2;
    return alpha_max * R_EXP(-(x > 0 ? x : 0));
}

/* The variance as the state keeps it: its square root in eight bits,
 * reference lib/ref/ref_denoise.c:101-107. */
static inline R SFX(orc_var_store)(R v)
{
    R c = v < 0 ? 0 : (v > 1 ? 1 : v);
    R q = R_RINT(R_SQRT(c) * (R)255) * ((R)1 / (R)255);
    return q * q;
}

/* NLM at one sample, 7x7 search, 3x3 patch, reference
 * lib/ref/ref_denoise.c:109-154. mx/my point at the mirrored column/row
 * tables entry of the sample itself. */
static R SFX(orc_nlm)(const R *plane, const R *var, int w2, const int *mx,
                      const int *my, R inv_h2)
{
    const int sr = ORC_DN_S, pr = ORC_DN_P;
    const R inv_np = (R)1 / (R)((2 * pr + 1) * (2 * pr + 1));
    R cpch[(2 * ORC_DN_P + 1) * (2 * ORC_DN_P + 1)];
    R acc = 0, wsum = 0;
    int n = 0;

    for (int ky = -pr; ky <= pr; ky++)
        for (int kx = -pr; kx <= pr; kx++)
            cpch[n++] = plane[(size_t)my[ky] * w2 + mx[kx]];

    for (int dy = -sr; dy <= sr; dy++) {
        for (int dx = -sr; dx <= sr; dx++) {
            R d2 = 0, wgt, x;
            n = 0;
            for (int ky = -pr; ky <= pr; ky++) {
                for (int kx = -pr; kx <= pr; kx++) {
                    R e = cpch[n++] - plane[(size_t)my[dy + ky] * w2 + mx[dx + kx]];
                    d2 += e * e;
                }
            }
            if (var) {
                R vc = var[(size_t)my[0] * w2 + mx[0]];
                R v2 = vc + var[(size_t)my[dy] * w2 + mx[dx]];
                x = d2 * inv_np * inv_h2 - v2;
                wgt = R_EXP(-(x > 0 ? x : 0) / vc);
            } else {
                x = d2 * inv_np * inv_h2 - (R)2;
                wgt = R_EXP(-(x > 0 ? x : 0));
            }
            R sv = plane[(size_t)my[dy] * w2 + mx[dx]];
            wsum += wgt;
            acc += wgt * sv;
        }
    }
    return acc / wsum;
}

/* Temporal average + VST + NLM on the four CFA planes, writing a denoised
 * R16 mosaic and (alpha_max > 0) the next temporal state: `next` is
 * 2 * width * height values, the level of every sample then the variance
 * left in it. Reference lib/ref/ref_denoise.c:168-336. */
ORC_API int SFX(orc_denoise_temporal)(const uint16_t *bayer, uint32_t width, uint32_t height,
                              size_t stride, const CRAWProfile *profile,
                              const CRAWNoiseModel *model, float strength,
                              float alpha_max, const R *prev, R *next,
                              uint16_t *out, size_t out_stride)
{
    const int sr = ORC_DN_S, pr = ORC_DN_P, rad = sr + pr;
    const R guard_inv = (R)1 / (ORC_DN_GUARD_HI - ORC_DN_GUARD_LO);
    struct SFX(orc_gat) g;
    R h, inv_h2;
    R *plane = NULL, *cur = NULL, *tprev = NULL, *var = NULL;
    int *mx = NULL, *my = NULL;
    int w2, h2, ret = 0;

    if (!bayer || !profile || !model || !out)
        return -EINVAL;
    if (profile->cfa != CRAW_CFA_RGGB)
        return -ENOTSUP;
    if ((width & 1) || (height & 1) ||
        width < (uint32_t)(2 * (rad + 2)) || height < (uint32_t)(2 * (rad + 2)))
        return -EINVAL;
    if (stride < width || out_stride < width)
        return -EINVAL;
    if (!(model->a > 0.0f))
        return -EINVAL;
    if (!(strength >= 0.0f) || !(alpha_max >= 0.0f) || !(alpha_max <= 1.0f) ||
        !(strength > 0.0f || alpha_max > 0.0f))
        return -EINVAL;
    if (alpha_max > 0.0f && !next)
        return -EINVAL;
    if (!(alpha_max > 0.0f))
        prev = NULL;
    for (int s = 0; s < 4; s++)
        if (!(profile->white_level[s] > profile->black_level[s]))
            return -EINVAL;

    SFX(orc_gat_init)(&g, (R)model->a, (R)model->b);
    h = strength > 0.0f ? (R)strength : (R)1;
    inv_h2 = (R)1 / (h * h);
    w2 = (int)(width / 2);
    h2 = (int)(height / 2);

    plane = malloc((size_t)w2 * h2 * sizeof(R));
    mx = malloc((size_t)(w2 + 2 * rad) * sizeof(int));
    my = malloc((size_t)(h2 + 2 * rad) * sizeof(int));
    if (prev) {
        cur = malloc((size_t)w2 * h2 * sizeof(R));
        tprev = malloc((size_t)w2 * h2 * sizeof(R));
        var = malloc((size_t)w2 * h2 * sizeof(R));
    }
    if (!plane || !mx || !my || (prev && (!cur || !tprev || !var))) {
        ret = -ENOMEM;
        goto done;
    }
    for (int i = 0; i < w2 + 2 * rad; i++)
        mx[i] = SFX(orc_mirror)(i - rad, w2);
    for (int k = 0; k < h2 + 2 * rad; k++)
        my[k] = SFX(orc_mirror)(k - rad, h2);

    for (int pl = 0; pl < 4; pl++) {
        int px = pl & 1, py = pl >> 1;
        R black = (R)profile->black_level[pl];
        R range = (R)profile->white_level[pl] - (R)profile->black_level[pl];
        R inv_range = (R)1 / range;

        for (int k = 0; k < h2; k++) {
            for (int i = 0; i < w2; i++) {
                size_t mp = (size_t)(2 * k + py) * width + 2 * i + px;
                R raw = (R)bayer[(size_t)(2 * k + py) * stride + 2 * i + px] * ((R)1 / (R)65535);
                R t = SFX(orc_gat_fwd)(&g, (raw - black) * inv_range);
                if (prev) {
                    cur[(size_t)k * w2 + i] = t;
                    tprev[(size_t)k * w2 + i] = SFX(orc_gat_fwd)(&g, prev[mp]);
                }
                plane[(size_t)k * w2 + i] = t;
            }
        }
        if (prev) {
            const R *prev_var = prev + (size_t)width * height;
            for (int k = 0; k < h2; k++) {
                for (int i = 0; i < w2; i++) {
                    size_t c = (size_t)k * w2 + i;
                    size_t mp = (size_t)(2 * k + py) * width + 2 * i + px;
                    R a = SFX(orc_alpha)(cur, tprev, w2, h2, i, k, (R)alpha_max, inv_h2);
                    R vv = ((R)1 - a) * ((R)1 - a) + a * a * prev_var[mp];
                    plane[c] = cur[c] * ((R)1 - a) + tprev[c] * a;
                    var[c] = vv > ORC_DN_VAR_MIN ? vv : ORC_DN_VAR_MIN;
                }
            }
        }
        if (alpha_max > 0.0f) {
            R *next_var = next + (size_t)width * height;
            for (int k = 0; k < h2; k++) {
                for (int i = 0; i < w2; i++) {
                    size_t mp = (size_t)(2 * k + py) * width + 2 * i + px;
                    next[mp] = SFX(orc_gat_inv)(&g, plane[(size_t)k * w2 + i]);
                    next_var[mp] = prev ? SFX(orc_var_store)(var[(size_t)k * w2 + i]) : (R)1;
                }
            }
        }
        for (int k = 0; k < h2; k++) {
            for (int i = 0; i < w2; i++) {
                R u, gr, raw0, u0, rawo;
                if (strength > 0.0f)
                    u = SFX(orc_gat_inv)(&g, SFX(orc_nlm)(plane, prev ? var : NULL, w2,
                                                          mx + rad + i, my + rad + k, inv_h2));
                else
                    u = SFX(orc_gat_inv)(&g, plane[(size_t)k * w2 + i]);
                raw0 = (R)bayer[(size_t)(2 * k + py) * stride + 2 * i + px] * ((R)1 / (R)65535);
                u0 = (raw0 - black) * inv_range;
                gr = (u0 - ORC_DN_GUARD_LO) * guard_inv;
                gr = gr < 0 ? 0 : (gr > 1 ? 1 : gr);
                u = u + (u0 - u) * gr;
                rawo = black + u * range;
                rawo = rawo < 0 ? 0 : (rawo > 1 ? 1 : rawo);
                out[(size_t)(2 * k + py) * out_stride + 2 * i + px] =
                    (uint16_t)R_RINT(rawo * (R)65535);
            }
        }
    }
done:
    free(var); free(tprev); free(cur); free(my); free(mx); free(plane);
    return ret;
}

/* ------------------------------------------------------------- chroma */

#define ORC_CD_RADIUS 4
#define ORC_CD_INV_2S2 ((R)(1.0f / (2.0f * 2.0f * 2.0f)))
#define ORC_CD_RANGE_K ((R)0.35f)
#define ORC_CD_CHROMA_K ((R)0.35f)
#define ORC_CD_RANGE_EPS ((R)0.02f)

static inline int SFX(orc_cd_mirror)(int v, int n)
{
    if (v < 0)
        return -v;
    if (v >= n)
        return 2 * n - 2 - v;
    return v;
}

/* Chroma denoise in place on RGBA, reference lib/ref/ref_chroma.c:22-158. */
ORC_API int SFX(orc_chroma_denoise)(R *rgb, uint32_t width, uint32_t height, float strength)
{
    int w = (int)width, h = (int)height, wq, hq, ret = 0;
    R *down, *blur, s = (R)strength;

    if (!rgb || width < 4 * (ORC_CD_RADIUS + 1) || height < 4 * (ORC_CD_RADIUS + 1))
        return -EINVAL;
    if (!(strength > 0.0f) || !(strength <= 1.0f))
        return -EINVAL;
    wq = (w + 3) / 4;
    hq = (h + 3) / 4;
    down = malloc((size_t)wq * hq * 3 * sizeof(R));
    blur = malloc((size_t)wq * hq * 3 * sizeof(R));
    if (!down || !blur) {
        ret = -ENOMEM;
        goto done;
    }
    for (int qy = 0; qy < hq; qy++) {
        for (int qx = 0; qx < wq; qx++) {
            R sum[3] = { 0, 0, 0 }, n = 0;
            R *o = &down[3 * ((size_t)qy * wq + qx)];
            for (int j = 0; j < 4; j++) {
                for (int i = 0; i < 4; i++) {
                    int x = 4 * qx + i, y = 4 * qy + j;
                    const R *px;
                    if (x >= w || y >= h)
                        continue;
                    px = &rgb[4 * ((size_t)y * w + x)];
                    sum[0] += px[0] - px[1];
                    sum[1] += px[2] - px[1];
                    sum[2] += px[1];
                    n += 1;
                }
            }
            for (int c = 0; c < 3; c++)
                o[c] = sum[c] / n;
        }
    }
    for (int qy = 0; qy < hq; qy++) {
        for (int qx = 0; qx < wq; qx++) {
            const R *c = &down[3 * ((size_t)qy * wq + qx)];
            R *o = &blur[3 * ((size_t)qy * wq + qx)];
            R level = (c[2] > 0 ? c[2] : 0) + ORC_CD_RANGE_EPS;
            R inv_range = (R)1 / (ORC_CD_RANGE_K * level);
            R inv_chroma = (R)1 / (ORC_CD_CHROMA_K * level);
            R acc0 = 0, acc1 = 0, wsum = 0;
            for (int dy = -ORC_CD_RADIUS; dy <= ORC_CD_RADIUS; dy++) {
                int sy = SFX(orc_cd_mirror)(qy + dy, hq);
                for (int dx = -ORC_CD_RADIUS; dx <= ORC_CD_RADIUS; dx++) {
                    int sx = SFX(orc_cd_mirror)(qx + dx, wq);
                    const R *sp = &down[3 * ((size_t)sy * wq + sx)];
                    R dg = (sp[2] - c[2]) * inv_range;
                    R dd0 = (sp[0] - c[0]) * inv_chroma, dd1 = (sp[1] - c[1]) * inv_chroma;
                    R wgt = R_EXP(-(R)(dx * dx + dy * dy) * ORC_CD_INV_2S2 - dg * dg
                                  - dd0 * dd0 - dd1 * dd1);
                    acc0 += wgt * sp[0];
                    acc1 += wgt * sp[1];
                    wsum += wgt;
                }
            }
            o[0] = acc0 / wsum;
            o[1] = acc1 / wsum;
            o[2] = c[2];
        }
    }
    for (int y = 0; y < h; y++) {
        R fy = ((R)y + (R)0.5) * (R)0.25 - (R)0.5;
        R fly = R_FLOOR(fy), ty = fy - fly;
        int y0 = CRAW_CLAMP((int)fly, 0, hq - 1), y1 = CRAW_CLAMP((int)fly + 1, 0, hq - 1);
        for (int x = 0; x < w; x++) {
            R fx = ((R)x + (R)0.5) * (R)0.25 - (R)0.5;
            R flx = R_FLOOR(fx), tx = fx - flx;
            int x0 = CRAW_CLAMP((int)flx, 0, wq - 1), x1 = CRAW_CLAMP((int)flx + 1, 0, wq - 1);
            R w00 = ((R)1 - tx) * ((R)1 - ty), w10 = tx * ((R)1 - ty);
            R w01 = ((R)1 - tx) * ty, w11 = tx * ty;
            const R *d00 = &down[3 * ((size_t)y0 * wq + x0)], *d10 = &down[3 * ((size_t)y0 * wq + x1)];
            const R *d01 = &down[3 * ((size_t)y1 * wq + x0)], *d11 = &down[3 * ((size_t)y1 * wq + x1)];
            const R *b00 = &blur[3 * ((size_t)y0 * wq + x0)], *b10 = &blur[3 * ((size_t)y0 * wq + x1)];
            const R *b01 = &blur[3 * ((size_t)y1 * wq + x0)], *b11 = &blur[3 * ((size_t)y1 * wq + x1)];
            R *px = &rgb[4 * ((size_t)y * w + x)];
            R gg = px[1];
            R d[2] = { px[0] - gg, px[2] - gg };
            for (int c = 0; c < 2; c++) {
                R lo = w00 * d00[c] + w10 * d10[c] + w01 * d01[c] + w11 * d11[c];
                R lf = w00 * b00[c] + w10 * b10[c] + w01 * b01[c] + w11 * b11[c];
                d[c] += s * (lf - lo);
            }
            px[0] = gg + d[0];
            px[2] = gg + d[1];
        }
    }
done:
    free(blur);
    free(down);
    return ret;
}

/* -------------------------------------------------------------- colour */

/* ACES 1.3 RGC on one AP1 triple, reference lib/gamut.c:61-92. */
static void SFX(orc_gamut_compress)(const struct orc_gamut *gc, R rgb[3])
{
    R ach = rgb[0] > rgb[1] ? rgb[0] : rgb[1];
    ach = ach > rgb[2] ? ach : rgb[2];
    if (ach == 0)
        return;
    R mag = R_FABS(ach);
    for (int i = 0; i < 3; i++) {
        R thr = (R)gc->thr[i], scl = (R)gc->scl[i];
        R d = (ach - rgb[i]) / mag;
        if (d < thr)
            continue;
        R nd = (d - thr) / scl;
        R p = R_POW(nd, (R)gc->pwr);
        d = thr + scl * nd / R_POW((R)1 + p, (R)gc->inv_pwr);
        rgb[i] = ach - d * mag;
    }
}

/* Matrix, gain, exposure, output space, RGC, clamp: in place on RGBA,
 * reference lib/ref/ref_color.c:10-76. */
ORC_API int SFX(orc_color)(R *rgb, uint32_t width, uint32_t height,
                   const CRAWFrameParams *fp, int out_space)
{
    CRAWColorParams par;
    double m_out_d[3][3];
    struct orc_gamut gc;
    R m_out[3][3], c2x[3][3], scale;
    bool clamp_neg, compress;
    int ret;

    if (!rgb || !fp || !fp->profile)
        return -EINVAL;
    ret = orc_profile_eval(fp->profile, fp->wb_mode, &fp->illuminant, &par);
    if (ret < 0)
        return ret;
    ret = orc_colorspace_from_xyz_d(out_space, m_out_d);
    if (ret < 0)
        return ret;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            m_out[i][j] = (R)SFX(orc_mstore)(m_out_d[i][j]);
            c2x[i][j] = (R)par.cam_to_xyz[i][j];
        }
    scale = (R)par.gain * R_EXP2((R)fp->exposure_stops);
    clamp_neg = (fp->flags & CRAW_FRAME_FLAG_CLAMP_NEGATIVE) != 0;
    compress = out_space == CRAW_CS_ACES_AP1_LINEAR &&
               !(fp->flags & CRAW_FRAME_FLAG_NO_GAMUT_COMPRESSION);
    orc_gamut_params(&gc);

    for (size_t i = 0; i < (size_t)width * height; i++) {
        R *px = &rgb[i * 4], xyz[3], out[3];
        for (int r = 0; r < 3; r++)
            xyz[r] = (c2x[r][0] * px[0] + c2x[r][1] * px[1] + c2x[r][2] * px[2]) * scale;
        for (int r = 0; r < 3; r++)
            out[r] = m_out[r][0] * xyz[0] + m_out[r][1] * xyz[1] + m_out[r][2] * xyz[2];
        if (compress)
            SFX(orc_gamut_compress)(&gc, out);
        if (clamp_neg)
            for (int r = 0; r < 3; r++)
                out[r] = out[r] > 0 ? out[r] : 0;
        px[0] = out[0];
        px[1] = out[1];
        px[2] = out[2];
        px[3] = 1;
    }
    return 0;
}

/* ------------------------------------------------ highlight reconstruction */

/* The reference's constants, lib/ref/ref_highlight.c:16-21. */
#define ORC_HL_U_LO ((R)0.92f)
#define ORC_HL_U_HI ((R)0.98f)
#define ORC_HL_EPS ((R)1e-4f)
#define ORC_HL_LOG_MAX ((R)2.0f)
#define ORC_HL_W_SAT ((R)1.0f)
#define ORC_HL_DILATE 3
#define ORC_HL_LEVELS 16

/* Channel of CFA site s (RGGB: R, Gr, Gb, B). */
static inline int SFX(orc_hl_chan)(int s) { return s == 0 ? 0 : (s == 3 ? 2 : 1); }

static inline R SFX(orc_hl_clampr)(R v, R lo, R hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* smoothstep(e0, e1, v): reference lib/ref/ref_highlight.c:41-47. */
static inline R SFX(orc_hl_smooth)(R e0, R e1, R v)
{
    R t = SFX(orc_hl_clampr)((v - e0) / (e1 - e0), (R)0, (R)1);
    return t * t * ((R)3 - (R)2 * t);
}

/* One pyramid level: w x h texels of (c0, c1, weight). */
struct SFX(orc_hl_level) {
    int w, h;
    R *t;
};

/* A level's colour at texel (x, y) clamped to its edge; the top level
 * still holds sums and is normalised here (ref_highlight.c:57-70). */
static void SFX(orc_hl_texel)(const struct SFX(orc_hl_level) *l, int x, int y, int top, R out[2])
{
    x = x < 0 ? 0 : (x >= l->w ? l->w - 1 : x);
    y = y < 0 ? 0 : (y >= l->h ? l->h - 1 : y);
    const R *t = &l->t[((size_t)y * l->w + x) * 3];
    if (top) {
        out[0] = t[2] > (R)0 ? t[0] / t[2] : (R)0;
        out[1] = t[2] > (R)0 ? t[1] / t[2] : (R)0;
    } else {
        out[0] = t[0];
        out[1] = t[1];
    }
}

/* Bilinear at (px, py) in texel coordinates, x mixed first
 * (ref_highlight.c:74-93). */
static void SFX(orc_hl_sample)(const struct SFX(orc_hl_level) *l, R px, R py, int top, R out[2])
{
    R fx0 = R_FLOOR(px), fy0 = R_FLOOR(py), fx = px - fx0, fy = py - fy0;
    int x0 = (int)fx0, y0 = (int)fy0;
    R c00[2], c10[2], c01[2], c11[2];
    SFX(orc_hl_texel)(l, x0, y0, top, c00);
    SFX(orc_hl_texel)(l, x0 + 1, y0, top, c10);
    SFX(orc_hl_texel)(l, x0, y0 + 1, top, c01);
    SFX(orc_hl_texel)(l, x0 + 1, y0 + 1, top, c11);
    for (int i = 0; i < 2; i++) {
        R a = c00[i] * ((R)1 - fx) + c10[i] * fx;
        R b = c01[i] * ((R)1 - fx) + c11[i] * fx;
        out[i] = a * ((R)1 - fy) + b * fy;
    }
}

/* The rebuilt, balanced mosaic of a frame whose highlights clipped:
 * reference lib/ref/ref_highlight.c:95-335 (DESIGN 18). Every site gets
 * u * wb of its channel; sites near the clip (a > 0) are lifted toward the
 * level their unclipped neighbours and the colour field predict. The
 * colour field is a pyramid of log-chroma averages of the unclipped
 * quads, pulled up to 1x1 and pushed back down. Output rounded to fp16. */
ORC_API int SFX(orc_highlights)(const uint16_t *bayer, uint32_t width, uint32_t height,
                                size_t stride, const CRAWProfile *profile, const float wb[3],
                                R *out)
{
    struct SFX(orc_hl_level) lv[ORC_HL_LEVELS];
    const int w = (int)width, h = (int)height, qw = w / 2, qh = h / 2;
    int nl = 0, ret = 0;
    R *uv, *av, *qa;

    if (!bayer || !profile || !wb || !out)
        return -EINVAL;
    if (width < 8 || height < 8 || (width & 1) || (height & 1) || stride < width)
        return -EINVAL;
    memset(lv, 0, sizeof(lv));
    uv = malloc((size_t)w * h * sizeof(R));
    av = malloc((size_t)w * h * sizeof(R));
    qa = malloc((size_t)qw * qh * sizeof(R));
    if (!uv || !av || !qa) {
        ret = -ENOMEM;
        goto done;
    }
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const int s = (y & 1) * 2 + (x & 1);
            const R inv = (R)1.0f / ((R)profile->white_level[s] - (R)profile->black_level[s]);
            const R raw = (R)bayer[(size_t)y * stride + x] * (R)(1.0f / 65535.0f);
            const R u = (raw - (R)profile->black_level[s]) * inv;
            uv[(size_t)y * w + x] = u;
            av[(size_t)y * w + x] = SFX(orc_hl_smooth)(ORC_HL_U_LO, ORC_HL_U_HI, u);
        }
    for (int qy = 0; qy < qh; qy++)
        for (int qx = 0; qx < qw; qx++) {
            R m = 0;
            for (int s = 0; s < 4; s++) {
                R a = av[(size_t)(2 * qy + (s >> 1)) * w + 2 * qx + (s & 1)];
                m = a > m ? a : m;
            }
            qa[(size_t)qy * qw + qx] = m;
        }
    /* Level sizes: 4x4 pixels a texel at level 0, halving (rounded up) to 1x1. */
    for (int lw = (w + 3) / 4, lh = (h + 3) / 4;; lw = (lw + 1) / 2, lh = (lh + 1) / 2) {
        if (nl == ORC_HL_LEVELS) {
            ret = -EINVAL;
            goto done;
        }
        lv[nl].w = lw;
        lv[nl].h = lh;
        if (!(lv[nl].t = calloc((size_t)lw * lh * 3, sizeof(R)))) {
            ret = -ENOMEM;
            goto done;
        }
        nl++;
        if (lw == 1 && lh == 1)
            break;
    }
    /* Level 0: the log chroma of each unclipped quad, weighted by how far
     * it is from every clip within ORC_HL_DILATE quads and how bright it is. */
    for (int by = 0; by < lv[0].h; by++)
        for (int bx = 0; bx < lv[0].w; bx++) {
            R acc[3] = { 0, 0, 0 };
            for (int j = 0; j < 2; j++)
                for (int i = 0; i < 2; i++) {
                    const int qx = 2 * bx + i, qy = 2 * by + j;
                    R amax = 0, umax = 0, rgb[3] = { 0, 0, 0 };
                    if (qx >= qw || qy >= qh)
                        continue;
                    for (int dy = -ORC_HL_DILATE; dy <= ORC_HL_DILATE; dy++)
                        for (int dx = -ORC_HL_DILATE; dx <= ORC_HL_DILATE; dx++) {
                            const int nx = qx + dx, ny = qy + dy;
                            if (nx < 0 || ny < 0 || nx >= qw || ny >= qh)
                                continue;
                            const R q = qa[(size_t)ny * qw + nx];
                            amax = q > amax ? q : amax;
                        }
                    for (int s = 0; s < 4; s++) {
                        const R u = uv[(size_t)(2 * qy + (s >> 1)) * w + 2 * qx + (s & 1)];
                        const int c = SFX(orc_hl_chan)(s);
                        rgb[c] += u * (R)wb[c];
                        umax = u > umax ? u : umax;
                    }
                    rgb[1] *= (R)0.5f;
                    const R m = umax < (R)1 ? umax : (R)1;
                    const R wq = ((R)1 - amax) * m * m;
                    const R g = rgb[1] > ORC_HL_EPS ? rgb[1] : ORC_HL_EPS;
                    const R r = SFX(orc_hl_clampr)(R_LOG((rgb[0] > ORC_HL_EPS ? rgb[0] : ORC_HL_EPS) / g),
                                                   -ORC_HL_LOG_MAX, ORC_HL_LOG_MAX);
                    const R b = SFX(orc_hl_clampr)(R_LOG((rgb[2] > ORC_HL_EPS ? rgb[2] : ORC_HL_EPS) / g),
                                                   -ORC_HL_LOG_MAX, ORC_HL_LOG_MAX);
                    acc[0] += wq * r;
                    acc[1] += wq * b;
                    acc[2] += wq;
                }
            memcpy(&lv[0].t[((size_t)by * lv[0].w + bx) * 3], acc, sizeof(acc));
        }
    /* Pull: each texel the sum of its (up to) four children. */
    for (int l = 0; l + 1 < nl; l++) {
        const struct SFX(orc_hl_level) *f = &lv[l];
        struct SFX(orc_hl_level) *c = &lv[l + 1];
        for (int y = 0; y < c->h; y++)
            for (int x = 0; x < c->w; x++) {
                R acc[3] = { 0, 0, 0 };
                for (int dy = 0; dy < 2; dy++)
                    for (int dx = 0; dx < 2; dx++) {
                        const int fx = 2 * x + dx, fy = 2 * y + dy;
                        if (fx >= f->w || fy >= f->h)
                            continue;
                        for (int k = 0; k < 3; k++)
                            acc[k] += f->t[((size_t)fy * f->w + fx) * 3 + k];
                    }
                memcpy(&c->t[((size_t)y * c->w + x) * 3], acc, sizeof(acc));
            }
    }
    /* Push: from under the top to level 0, each texel blended from the
     * coarser level's bilinear colour toward its own mean by its weight. */
    for (int l = nl - 2; l >= 0; l--) {
        struct SFX(orc_hl_level) *f = &lv[l];
        const struct SFX(orc_hl_level) *c = &lv[l + 1];
        const int top = l + 2 == nl;
        for (int y = 0; y < f->h; y++)
            for (int x = 0; x < f->w; x++) {
                R *t = &f->t[((size_t)y * f->w + x) * 3], up[2];
                SFX(orc_hl_sample)(c, ((R)x + (R)0.5f) * (R)0.5f - (R)0.5f,
                                   ((R)y + (R)0.5f) * (R)0.5f - (R)0.5f, top, up);
                if (t[2] > (R)0) {
                    const R s = t[2] / ORC_HL_W_SAT < (R)1 ? t[2] / ORC_HL_W_SAT : (R)1;
                    t[0] = up[0] + s * (t[0] / t[2] - up[0]);
                    t[1] = up[1] + s * (t[1] / t[2] - up[1]);
                } else {
                    t[0] = up[0];
                    t[1] = up[1];
                }
            }
    }
    /* Fill. */
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const size_t o = (size_t)y * w + x;
            const int c = SFX(orc_hl_chan)((y & 1) * 2 + (x & 1));
            const R xc = uv[o] * (R)wb[c], a = av[o];
            R res = xc;
            if (a > (R)0) {
                R sum[3] = { 0, 0, 0 }, n[3] = { 0, 0, 0 }, am[3] = { 0, 0, 0 }, lf[2], lrho[3];
                SFX(orc_hl_sample)(&lv[0], (R)(x >> 1) * (R)0.5f - (R)0.25f,
                                   (R)(y >> 1) * (R)0.5f - (R)0.25f, 0, lf);
                lrho[0] = lf[0];
                lrho[1] = 0;
                lrho[2] = lf[1];
                for (int dy = -1; dy <= 1; dy++)
                    for (int dx = -1; dx <= 1; dx++) {
                        const int nx = SFX(orc_mirror)(x + dx, w), ny = SFX(orc_mirror)(y + dy, h);
                        const int k = SFX(orc_hl_chan)((ny & 1) * 2 + (nx & 1));
                        const size_t no = (size_t)ny * w + nx;
                        if (k == c)
                            continue;
                        sum[k] += uv[no] * (R)wb[k];
                        n[k] += (R)1;
                        am[k] = av[no] > am[k] ? av[no] : am[k];
                    }
                const int k1 = c == 0 ? 1 : 0, k2 = c == 2 ? 1 : 2;
                const R a1 = (R)1 - am[k1], a2 = (R)1 - am[k2];
                const R m1 = sum[k1] / n[k1], m2 = sum[k2] / n[k2];
                const R l1 = R_LOG(m1 > ORC_HL_EPS ? m1 : ORC_HL_EPS) - lrho[k1];
                const R l2 = R_LOG(m2 > ORC_HL_EPS ? m2 : ORC_HL_EPS) - lrho[k2];
                const R lc = R_LOG(xc > ORC_HL_EPS ? xc : ORC_HL_EPS) - lrho[c];
                const R A = a1 + a2;
                const R lmax = lc > (l1 > l2 ? l1 : l2) ? lc : (l1 > l2 ? l1 : l2);
                const R lfull = R_EXP(lmax);
                const R lpart = A > (R)0 ? R_EXP((a1 * l1 + a2 * l2) / A) : lfull;
                const R L = lfull + (A < (R)1 ? A : (R)1) * (lpart - lfull);
                const R lift = L * R_EXP(lrho[c]) - xc;
                res = xc + a * (lift > (R)0 ? lift : (R)0);
            }
            out[o] = (R)orc_to_half((float)res);
        }
done:
    for (int i = 0; i < nl; i++)
        free(lv[i].t);
    free(uv);
    free(av);
    free(qa);
    return ret;
}

/* --------------------------------------------------------- whole frame */

/* One frame through the chain, reference lib/ref/ref_color.c:91-230,
 * restricted to the stages of this path (denoise, debayer, chroma,
 * colour). A single frame has no history: with the temporal flag the
 * average runs as on a first frame. */
ORC_API int SFX(orc_process)(const uint16_t *bayer, uint32_t width, uint32_t height,
                     size_t stride, const CRAWPipelineParams *params,
                     const CRAWFrameParams *fp, R *out)
{
    uint16_t *clean = NULL;
    R *state = NULL;
    float strength, alpha_max;
    int ret;

    if (!params || !fp || !fp->profile)
        return -EINVAL;
    if (params->width && (params->width != width || params->height != height))
        return -EINVAL;
    if (params->cfa != fp->profile->cfa)
        return -EINVAL;
    strength = (params->flags & CRAW_PIPELINE_FLAG_DENOISE) ? fp->denoise_strength : 0.0f;
    alpha_max = (params->flags & CRAW_PIPELINE_FLAG_TEMPORAL_DENOISE)
              ? fp->denoise_temporal_strength : 0.0f;
    strength = strength > 0.0f ? strength : 0.0f;
    alpha_max = alpha_max > 0.0f ? alpha_max : 0.0f;
    if (strength > 0.0f || alpha_max > 0.0f) {
        CRAWNoiseModel nm;
        ret = orc_noise_model(fp, &nm);
        if (ret < 0)
            return ret;
        clean = malloc((size_t)width * height * sizeof(*clean));
        if (alpha_max > 0.0f)
            state = malloc(2 * (size_t)width * height * sizeof(R));
        if (!clean || (alpha_max > 0.0f && !state)) {
            ret = -ENOMEM;
            goto done;
        }
        ret = SFX(orc_denoise_temporal)(bayer, width, height, stride, fp->profile, &nm,
                                        strength, alpha_max, NULL, state, clean, width);
        if (ret < 0)
            goto done;
        bayer = clean;
        stride = width;
    }
    {
        CRAWColorParams par;
        ret = orc_profile_eval(fp->profile, fp->wb_mode, &fp->illuminant, &par);
        if (ret < 0)
            goto done;
        if ((params->flags & CRAW_PIPELINE_FLAG_HIGHLIGHT_RECONSTRUCTION) &&
            (fp->flags & CRAW_FRAME_FLAG_HIGHLIGHT_RECONSTRUCTION)) {
            /* The rebuilt mosaic replaces the prep and its clip
             * (ref_color.c:146-160). */
            R *v = malloc((size_t)width * height * sizeof(R));
            if (!v) {
                ret = -ENOMEM;
                goto done;
            }
            ret = SFX(orc_highlights)(bayer, width, height, stride, fp->profile, par.wb, v);
            if (ret >= 0)
                ret = SFX(orc_debayer_mosaic)(v, width, height, params->debayer, out);
            free(v);
        } else {
            ret = SFX(orc_debayer_wb)(bayer, width, height, stride, fp->profile, par.wb,
                                      params->debayer, out);
        }
        if (ret < 0)
            goto done;
    }
    if ((params->flags & CRAW_PIPELINE_FLAG_CHROMA_DENOISE) && fp->denoise_chroma_strength > 0.0f) {
        ret = SFX(orc_chroma_denoise)(out, width, height, fp->denoise_chroma_strength);
        if (ret < 0)
            goto done;
    }
    ret = SFX(orc_color)(out, width, height, fp,
                         fp->out_space_set ? (int)fp->out_space : (int)params->out_space);
done:
    free(state);
    free(clean);
    return ret;
}
