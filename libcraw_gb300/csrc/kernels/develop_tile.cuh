/*
 * The fused develop stage, tile bodies: prep + debayer + epilogue in one launch.
 *
 * One CTA develops a TW x TH tile of the frame. It loads the tile's
 * mosaic with the debayer's apron into shared memory, prepped (normalise,
 * white balance, clip: reference lib/ref/ref_debayer.c:42-63), debayers
 * it there, and then, per pixel, either applies the colour stage and
 * writes the caller's RGBA image, or (chroma denoise on) writes the
 * camera RGB intermediate and the 4x4 block means the chroma pass works
 * on. The AWB statistic of every 8x8 block is formed from the tile in
 * shared memory in the same pass. The only HBM traffic is the mosaic in
 * (2 B/px) and the output (16 or 8 B/px), plus 8 B per 64 px of AWB
 * records.
 *
 * Borders: every array of the RCD holds at a position outside the frame
 * the value its pass computed at the position that mirrors there, which
 * is what the reference's full-image sweeps read through their mirrored
 * fetches (lib/ref/ref_debayer.c:36-40). A tile whose aprons lie inside
 * the frame skips the mirror arithmetic.
 */
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace craw_dev {


constexpr int kBilinear = 0, kMhc = 1, kRcd = 2;

template <int M> struct Apron { static constexpr int v = M == kBilinear ? 1 : (M == kMhc ? 2 : 5); };

#define RCD_EPS 1e-5f

/* A tile-local array with an apron: element (x, y) for x in [-a, W+a). */
template <int W, int H, int A, typename T> struct Tile {
    static constexpr int SX = W + 2 * A, SY = H + 2 * A, N = SX * SY;
    T *p;
    CRAW_DEV T &at(int x, int y) const { return p[(y + A) * SX + (x + A)]; }
};

/* Maps tile position q of an array of apron a to the tile position of the
 * frame position it mirrors to, kept inside the array (which only matters
 * for tiles hanging far past a small frame's edge, where the position is
 * not needed by any pixel inside the frame). */
struct Frame {
    int x0, y0, w, h;
    bool interior;
    template <bool INTERIOR>
    CRAW_DEV void map(int qx, int qy, int a, int tw, int th, int &px, int &py) const
    {
        if constexpr (INTERIOR) {
            px = qx;
            py = qy;
        } else {
            px = craw_mirror(x0 + qx, w) - x0;
            py = craw_mirror(y0 + qy, h) - y0;
            px = px < -a ? -a : (px > tw - 1 + a ? tw - 1 + a : px);
            py = py < -a ? -a : (py > th - 1 + a ? th - 1 + a : py);
        }
    }
};

template <int TW, int TH, int NT, int A, typename VT>
CRAW_DEV void load_prepped(const CRAWKDevelop &k, const CRAWKDevelopIO &io, const Frame &f,
                           VT &v)
{
    for (int i = threadIdx.x; i < VT::N; i += NT) {
        int x = f.x0 + i % VT::SX - A, y = f.y0 + i / VT::SX - A;
        if (!f.interior) {
            x = craw_mirror(x, f.w);
            y = craw_mirror(y, f.h);
        }
        uint16_t raw = 0;
        if (craw_in_bounds(x >= 0 && x < k.width && y >= 0 && y < k.height, io.err))
            raw = __ldg((const uint16_t *)((const char *)io.src + (size_t)y * io.src_pitch) + x);
        v.p[i] = io.src_f16 ? __half2float(__ushort_as_half(raw)) : craw_prep(k, raw, (y & 1) * 2 + (x & 1));
    }
}

/* ------------------------------------------------------------ bilinear */

template <typename VT>
CRAW_DEV void bilinear_px(const VT &v, int x, int y, int s, float o[3])
{
#define V(dx, dy) v.at(x + (dx), y + (dy))
    float c = V(0, 0);
    if (s == 0 || s == 3) {
        float edge = 0.25f * (V(0, -1) + V(0, 1) + V(-1, 0) + V(1, 0));
        float corner = 0.25f * (V(-1, -1) + V(1, -1) + V(-1, 1) + V(1, 1));
        o[0] = s == 0 ? c : corner;
        o[1] = edge;
        o[2] = s == 0 ? corner : c;
    } else {
        float horiz = 0.5f * (V(-1, 0) + V(1, 0));
        float vert = 0.5f * (V(0, -1) + V(0, 1));
        o[0] = s == 1 ? horiz : vert;
        o[1] = c;
        o[2] = s == 1 ? vert : horiz;
    }
#undef V
}

/* ----------------------------------------------------------------- MHC */

template <typename VT>
CRAW_DEV void mhc_px(const VT &v, int x, int y, int s, float o[3])
{
#define V(dx, dy) v.at(x + (dx), y + (dy))
    float c = V(0, 0);
    float cross = V(0, -1) + V(0, 1) + V(-1, 0) + V(1, 0);
    float axial2 = V(0, -2) + V(0, 2) + V(-2, 0) + V(2, 0);
    float diag = V(-1, -1) + V(1, -1) + V(-1, 1) + V(1, 1);
    if (s == 0 || s == 3) {
        float g = (4.0f * c + 2.0f * cross - axial2) * 0.125f;
        float d = (6.0f * c + 2.0f * diag - 1.5f * axial2) * 0.125f;
        o[0] = s == 0 ? c : d;
        o[1] = g;
        o[2] = s == 0 ? d : c;
    } else {
        float hz = (5.0f * c + 4.0f * (V(-1, 0) + V(1, 0)) - (diag + V(-2, 0) + V(2, 0))
                    + 0.5f * (V(0, -2) + V(0, 2))) * 0.125f;
        float vt = (5.0f * c + 4.0f * (V(0, -1) + V(0, 1)) - (diag + V(0, -2) + V(0, 2))
                    + 0.5f * (V(-2, 0) + V(2, 0))) * 0.125f;
        o[0] = s == 1 ? hz : vt;
        o[1] = c;
        o[2] = s == 1 ? vt : hz;
    }
#undef V
}

/* ----------------------------------------------------------------- RCD */

CRAW_DEV float rcd_ratio(float a, float b)
{
    a = fmaxf(a, 0.0f);
    b = fmaxf(b, 0.0f);
    return __fdividef(a - b, a + b + RCD_EPS);
}

/* The RCD passes of reference lib/ref/ref_debayer.c:204-395 on a tile,
 * inwards one ring of apron per step: L (4), directions (3), weights (2),
 * green (2), colour at R/B (1), then the output pixels. */
template <int TW, int TH, int NT>
struct RcdTile {
    Tile<TW, TH, 5, float> v;
    Tile<TW, TH, 4, float> l;
    Tile<TW, TH, 3, float4> d;
    Tile<TW, TH, 2, float2> w;
    Tile<TW, TH, 2, float> g;
    Tile<TW, TH, 1, float> c;
    static constexpr int floats = Tile<TW, TH, 5, float>::N + Tile<TW, TH, 4, float>::N +
                                  4 * Tile<TW, TH, 3, float>::N + 2 * Tile<TW, TH, 2, float>::N +
                                  Tile<TW, TH, 2, float>::N + Tile<TW, TH, 1, float>::N;

    CRAW_DEV void carve(float *base)
    {
        d.p = reinterpret_cast<float4 *>(base);           base += 4 * decltype(d)::N;
        w.p = reinterpret_cast<float2 *>(base);           base += 2 * decltype(w)::N;
        v.p = base;                                       base += decltype(v)::N;
        l.p = base;                                       base += decltype(l)::N;
        g.p = base;                                       base += decltype(g)::N;
        c.p = base;
    }

    template <bool IN>
    CRAW_DEV void run(const Frame &f)
    {
        /* Low pass, apron 4. */
        for (int i = threadIdx.x; i < decltype(l)::N; i += NT) {
            int px, py;
            f.template map<IN>(i % decltype(l)::SX - 4, i / decltype(l)::SX - 4, 4, TW, TH, px, py);
#define V(dx, dy) v.at(px + (dx), py + (dy))
            l.p[i] = (4.0f * V(0, 0) + 2.0f * (V(0, -1) + V(0, 1) + V(-1, 0) + V(1, 0))
                      + V(-1, -1) + V(1, -1) + V(-1, 1) + V(1, 1)) * (1.0f / 16.0f);
        }
        /* Vertical, horizontal and the two diagonal discriminations, apron 3. */
        for (int i = threadIdx.x; i < decltype(d)::N; i += NT) {
            int px, py;
            f.template map<IN>(i % decltype(d)::SX - 3, i / decltype(d)::SX - 3, 3, TW, TH, px, py);
            float c2 = 2.0f * V(0, 0);
            float4 r;
            r.x = fabsf(V(0, -1) - V(0, 1)) + fabsf(c2 - V(0, -2) - V(0, 2));
            r.y = fabsf(V(-1, 0) - V(1, 0)) + fabsf(c2 - V(-2, 0) - V(2, 0));
            r.z = fabsf(V(-1, 1) - V(1, -1)) + fabsf(c2 - V(-2, 2) - V(2, -2));
            r.w = fabsf(V(-1, -1) - V(1, 1)) + fabsf(c2 - V(-2, -2) - V(2, 2));
            d.p[i] = r;
        }
        __syncthreads();
        /* Weights from 3x3 means of the discriminations, apron 2. */
        for (int i = threadIdx.x; i < decltype(w)::N; i += NT) {
            int px, py;
            f.template map<IN>(i % decltype(w)::SX - 2, i / decltype(w)::SX - 2, 2, TW, TH, px, py);
            float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int dy = -1; dy <= 1; dy++)
#pragma unroll
                for (int dx = -1; dx <= 1; dx++) {
                    float4 t = d.at(px + dx, py + dy);
                    s.x += t.x; s.y += t.y; s.z += t.z; s.w += t.w;
                }
            float vs = s.x * (1.0f / 9.0f), hs = s.y * (1.0f / 9.0f);
            float ps = s.z * (1.0f / 9.0f), qs = s.w * (1.0f / 9.0f);
            w.p[i] = make_float2(__fdividef(hs, hs + vs + RCD_EPS), __fdividef(qs, ps + qs + RCD_EPS));
        }
        __syncthreads();
        /* Green at the R and B sites, apron 2. */
        for (int i = threadIdx.x; i < decltype(g)::N; i += NT) {
            int px, py;
            f.template map<IN>(i % decltype(g)::SX - 2, i / decltype(g)::SX - 2, 2, TW, TH, px, py);
            int s = ((f.y0 + py) & 1) * 2 + ((f.x0 + px) & 1);
            if (s == 1 || s == 2) {
                g.p[i] = V(0, 0);
                continue;
            }
#define L(dx, dy) l.at(px + (dx), py + (dy))
            float l00 = L(0, 0);
            float gv = 0.5f * (V(0, -1) * (1.0f + rcd_ratio(l00, L(0, -2)))
                             + V(0, 1) * (1.0f + rcd_ratio(l00, L(0, 2))));
            float gh = 0.5f * (V(-1, 0) * (1.0f + rcd_ratio(l00, L(-2, 0)))
                             + V(1, 0) * (1.0f + rcd_ratio(l00, L(2, 0))));
#undef L
            float wt = w.at(px, py).x;
            g.p[i] = wt * gv + (1.0f - wt) * gh;
        }
        __syncthreads();
        /* The missing colour at the R and B sites, apron 1. */
        for (int i = threadIdx.x; i < decltype(c)::N; i += NT) {
            int px, py;
            f.template map<IN>(i % decltype(c)::SX - 1, i / decltype(c)::SX - 1, 1, TW, TH, px, py);
            int s = ((f.y0 + py) & 1) * 2 + ((f.x0 + px) & 1);
            if (s == 1 || s == 2)
                continue;
#define G(dx, dy) g.at(px + (dx), py + (dy))
            float g00 = G(0, 0), wt = w.at(px, py).y;
            c.p[i] = wt * (g00 + 0.5f * ((V(-1, 1) - G(-1, 1)) + (V(1, -1) - G(1, -1))))
                   + (1.0f - wt) * (g00 + 0.5f * ((V(-1, -1) - G(-1, -1)) + (V(1, 1) - G(1, 1))));
        }
        __syncthreads();
    }

    /* The output pixel at tile position (x, y), inside the frame. */
    CRAW_DEV void pixel(int x, int y, int s, float o[3]) const
    {
        const int px = x, py = y;
        if (s == 0 || s == 3) {
            float cc = c.at(px, py);
            o[0] = s == 0 ? V(0, 0) : cc;
            o[1] = G(0, 0);
            o[2] = s == 0 ? cc : V(0, 0);
            return;
        }
#define C(dx, dy) c.at(px + (dx), py + (dy))
        float g00 = G(0, 0), wt = w.at(px, py).x;
        float dh = 0.5f * ((V(-1, 0) - G(-1, 0)) + (V(1, 0) - G(1, 0)));
        float ev = 0.5f * ((C(0, -1) - G(0, -1)) + (C(0, 1) - G(0, 1)));
        float ch = wt * (g00 + ev) + (1.0f - wt) * (g00 + dh);
        float dv = 0.5f * ((V(0, -1) - G(0, -1)) + (V(0, 1) - G(0, 1)));
        float eh = 0.5f * ((C(-1, 0) - G(-1, 0)) + (C(1, 0) - G(1, 0)));
        float cv = wt * (g00 + dv) + (1.0f - wt) * (g00 + eh);
        o[0] = s == 1 ? ch : cv;
        o[1] = V(0, 0);
        o[2] = s == 1 ? cv : ch;
#undef C
#undef G
#undef V
    }
};

/* ------------------------------------------- RCD arithmetic of the quads */

/* The RCD formulas of reference lib/ref/ref_debayer.c:204-395 as the quad
 * forms (tiles and strips) evaluate them, every rounding explicit, so that
 * both give the same bits whatever the compiler contracts around them. */

/* 1/x on the MUFU (x >= 1e-5 wherever it is used: no denormals). */
CRAW_DEV float rq_rcp(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

/* 1 + (a - b) / (a + b + eps) for low passes a, b already clamped at 0
 * (the reference clamps them where it forms the ratio; they are stored
 * clamped, which they are used for only). */
CRAW_DEV float rq_ratio1(float a, float b)
{
    return __fmaf_rn(__fsub_rn(a, b), rq_rcp(__fadd_rn(__fadd_rn(a, b), RCD_EPS)), 1.0f);
}

/* The low pass at a site from its 3x3 window (n, s, w, e: the cross; the
 * four diagonals), clamped at 0 for the ratios it feeds. */
CRAW_DEV float rq_lowpass(float c, float n, float s, float w, float e, float nw, float ne, float sw, float se)
{
    float t = __fmaf_rn(4.0f, c, __fmul_rn(2.0f, __fadd_rn(__fadd_rn(__fadd_rn(n, s), w), e)));
    t = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(t, nw), ne), sw), se);
    return fmaxf(__fmul_rn(t, 1.0f / 16.0f), 0.0f);
}

/* One discrimination: |a1 - b1| + |2c - a2 - b2| (c2 = 2c). */
CRAW_DEV float rq_disc(float c2, float a1, float b1, float a2, float b2)
{
    return __fadd_rn(fabsf(__fsub_rn(a1, b1)), fabsf(__fsub_rn(__fsub_rn(c2, a2), b2)));
}

/* The (V, H, P, Q) discriminations of the site at the centre of a 5x5
 * window, w[r][c] for r, c in 0..4. */
template <typename WIN>
CRAW_DEV float4 rq_disc4(const WIN &w)
{
    const float c2 = __fmul_rn(2.0f, w(2, 2));
    float4 d;
    d.x = rq_disc(c2, w(1, 2), w(3, 2), w(0, 2), w(4, 2));
    d.y = rq_disc(c2, w(2, 1), w(2, 3), w(2, 0), w(2, 4));
    d.z = rq_disc(c2, w(3, 1), w(1, 3), w(4, 0), w(0, 4));
    d.w = rq_disc(c2, w(1, 1), w(3, 3), w(0, 0), w(4, 4));
    return d;
}

CRAW_DEV float4 rq_add4(float4 a, float4 b)
{
    return make_float4(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z), __fadd_rn(a.w, b.w));
}

/* The vertical weight from the 3x3 sums of (V, H, P, Q), and the diagonal
 * one. */
CRAW_DEV float rq_wv(float4 s)
{
    const float vs = __fmul_rn(s.x, 1.0f / 9.0f), hs = __fmul_rn(s.y, 1.0f / 9.0f);
    return __fmul_rn(hs, rq_rcp(__fadd_rn(__fadd_rn(hs, vs), RCD_EPS)));
}
CRAW_DEV float rq_wp(float4 s)
{
    const float ps = __fmul_rn(s.z, 1.0f / 9.0f), qs = __fmul_rn(s.w, 1.0f / 9.0f);
    return __fmul_rn(qs, rq_rcp(__fadd_rn(__fadd_rn(ps, qs), RCD_EPS)));
}

/* wt a + (1 - wt) b. */
CRAW_DEV float rq_blend(float wt, float a, float b)
{
    return __fmaf_rn(wt, a, __fmul_rn(__fsub_rn(1.0f, wt), b));
}

/* Green at an R or B site: its low pass l0, the vertical neighbours vu, vd
 * (low passes lu, ld two rows away), the horizontal vl, vr (ll, lr), and
 * the site's vertical weight wt. */
CRAW_DEV float rq_green(float wt, float l0, float vu, float lu, float vd, float ld, float vl, float ll, float vr,
                        float lr)
{
    const float gv = __fmul_rn(0.5f, __fmaf_rn(vu, rq_ratio1(l0, lu), __fmul_rn(vd, rq_ratio1(l0, ld))));
    const float gh = __fmul_rn(0.5f, __fmaf_rn(vl, rq_ratio1(l0, ll), __fmul_rn(vr, rq_ratio1(l0, lr))));
    return rq_blend(wt, gv, gh);
}

/* g + (a + b) / 2. */
CRAW_DEV float rq_half_sum(float g, float a, float b)
{
    return __fmaf_rn(0.5f, __fadd_rn(a, b), g);
}

/* The missing colour at an R or B site from the colour differences on its
 * diagonals (sw + ne against nw + se), by its diagonal weight wt. */
CRAW_DEV float rq_cross(float wt, float g00, float dsw, float dne, float dnw, float dse)
{
    return rq_blend(wt, rq_half_sum(g00, dsw, dne), rq_half_sum(g00, dnw, dse));
}

/* R and B at a green site: horizontal (dh: the row's colour differences,
 * ev: the column's of the other colour) against vertical (dv, eh). */
CRAW_DEV void rq_green_site(float wt, float g00, float dh0, float dh1, float ev0, float ev1, float dv0,
                            float dv1, float eh0, float eh1, float &ch, float &cv)
{
    ch = rq_blend(wt, rq_half_sum(g00, ev0, ev1), rq_half_sum(g00, dh0, dh1));
    cv = rq_blend(wt, rq_half_sum(g00, dv0, dv1), rq_half_sum(g00, eh0, eh1));
}

/* ------------------------------------------------------- RCD, by quads */

/* The RCD of an interior tile (all aprons inside the frame), one thread
 * per 2x2 CFA quad (R at (0,0), Gr (1,0), Gb (0,1), B (1,1)): the site of
 * every value is static, the neighbours a quad's four sites share are
 * read once, and shared memory moves in float2 and float4. Same passes,
 * same formulas as the per-pixel version above, evaluated by the rq_*
 * helpers with every rounding explicit (the strips evaluate them the same
 * way), and the 3x3 sums of the discriminations taken as rows of three and
 * then three rows.
 *
 * Arrays (tile-relative pixel or quad coordinates, their ranges):
 *   Vp float   pixels [-6, TW+6) x [-6, TH+6)   the prepped mosaic
 *   Lq float2  quads  [-2, QW+2) x [-2, QH+2)   low pass at R and at B
 *   Dp float4  pixels [-4, TW+4) x [-4, TH+4)   (V, H, P, Q) discriminations
 *   Wp float2  pixels [-2, TW+2) x [-2, TH+2)   (wv, wp) weights
 *   Gq float2  quads  [-1, QW+1) x [-1, QH+1)   green at R and at B
 *   Cq float2  quads  [-1, QW+1) x [-1, QH+1)   B at R, R at B
 * Dp and Wp are stored as an even-column and an odd-column plane, so that
 * the threads of a warp, one quad each, read consecutive elements of a
 * plane rather than every other one. The output planes reuse Dp's space
 * once the weights exist. */
template <int TW, int TH, int NT>
struct RcdQuads {
    static constexpr int QW = TW / 2, QH = TH / 2;
    static constexpr int VS = TW + 12, DS = TW + 8, WS = TW + 4, LS = QW + 4, GS = QW + 2;
    static constexpr int VN = (TH + 12) * VS, DN = (TH + 8) * DS, WN = (TH + 4) * WS;
    static constexpr int LN = (QH + 4) * LS, GN = (QH + 2) * GS;
    static constexpr int DQ = DS / 2, WQ = WS / 2;           /* elements per plane row */
    static constexpr int floats = 4 * DN + 2 * WN + 2 * LN + 4 * GN + VN;
    static_assert(3 * TW * TH <= 4 * DN, "the output fits in D's space");

    float4 *Dp;
    float2 *Wp, *Lq, *Gq, *Cq;
    float *Vp;
    float *rgb;   /* planar R, G, B of the tile */

    CRAW_DEV void carve(float *base)
    {
        Dp = reinterpret_cast<float4 *>(base);
        Wp = reinterpret_cast<float2 *>(base + 4 * DN);
        Lq = reinterpret_cast<float2 *>(base + 4 * DN + 2 * WN);
        Gq = reinterpret_cast<float2 *>(base + 4 * DN + 2 * WN + 2 * LN);
        Cq = reinterpret_cast<float2 *>(base + 4 * DN + 2 * WN + 2 * LN + 2 * GN);
        Vp = base + 4 * DN + 2 * WN + 2 * LN + 4 * GN;
        rgb = base;
    }

    CRAW_DEV float V(int x, int y) const { return Vp[(y + 6) * VS + x + 6]; }
    CRAW_DEV float2 V2(int x, int y) const
    {
        return *reinterpret_cast<const float2 *>(&Vp[(y + 6) * VS + x + 6]);
    }
    CRAW_DEV float4 &D(int x, int y) const
    {
        const int xx = x + 4;
        return Dp[(xx & 1) * (DN / 2) + (y + 4) * DQ + (xx >> 1)];
    }
    CRAW_DEV float2 &W(int x, int y) const
    {
        const int xx = x + 2;
        return Wp[(xx & 1) * (WN / 2) + (y + 2) * WQ + (xx >> 1)];
    }
    CRAW_DEV float2 &Lat(int qx, int qy) const { return Lq[(qy + 2) * LS + qx + 2]; }
    CRAW_DEV float2 &G(int qx, int qy) const { return Gq[(qy + 1) * GS + qx + 1]; }
    CRAW_DEV float2 &Cat(int qx, int qy) const { return Cq[(qy + 1) * GS + qx + 1]; }

    /* Quad (qx, qy) of the tile prepped into V from its two rows of
     * samples (a: R, Gr; b: Gb, B; 16 bits each). */
    CRAW_DEV void put_quad(const CRAWKDevelop &k, const CRAWKDevelopIO &io, int qx, int qy, uint32_t a, uint32_t b)
    {
        float2 top, bot;
        if (io.src_f16) {   /* rebuilt highlights: fp16, already prepped */
            top = __half22float2(*reinterpret_cast<const __half2 *>(&a));
            bot = __half22float2(*reinterpret_cast<const __half2 *>(&b));
        } else {
            top = make_float2(craw_prep(k, (uint16_t)(a & 0xffff), 0), craw_prep(k, (uint16_t)(a >> 16), 1));
            bot = make_float2(craw_prep(k, (uint16_t)(b & 0xffff), 2), craw_prep(k, (uint16_t)(b >> 16), 3));
        }
        *reinterpret_cast<float2 *>(&Vp[(2 * qy + 6) * VS + 2 * qx + 6]) = top;
        *reinterpret_cast<float2 *>(&Vp[(2 * qy + 7) * VS + 2 * qx + 6]) = bot;
    }

    /* The prepped mosaic of the tile and its apron: two u32 (two samples
     * each) per quad. */
    CRAW_DEV void load(const CRAWKDevelop &k, const CRAWKDevelopIO &io, int x0, int y0)
    {
        constexpr int QX = QW + 6, QY = QH + 6;
        for (int i = threadIdx.x; i < QX * QY; i += NT) {
            int qx, qy;
            craw_row_item<QX, QY>(i, qx, qy);
            qx -= 3;
            qy -= 3;
            int x = x0 + 2 * qx, y = y0 + 2 * qy;
            const char *r0 = (const char *)io.src + (size_t)y * io.src_pitch;
            uint32_t a = 0, b = 0;
            if (craw_in_bounds(x >= 0 && x + 1 < k.width && y >= 0 && y + 1 < k.height, io.err)) {
                a = __ldg(reinterpret_cast<const uint32_t *>(r0) + x / 2);
                b = __ldg(reinterpret_cast<const uint32_t *>(r0 + io.src_pitch) + x / 2);
            }
            put_quad(k, io, qx, qy, a, b);
        }
    }

    /* The same from the tile's mosaic already in shared memory: `box` is
     * BW 16-bit samples a row (BW even) from frame column x0 - 8 and row
     * y0 - 6, as a TMA tile copy leaves it. */
    template <int BW>
    CRAW_DEV void load_box(const CRAWKDevelop &k, const CRAWKDevelopIO &io, const uint32_t *box)
    {
        constexpr int QX = QW + 6, QY = QH + 6;
        for (int i = threadIdx.x; i < QX * QY; i += NT) {
            int qx, qy;
            craw_row_item<QX, QY>(i, qx, qy);
            qx -= 3;
            qy -= 3;
            const uint32_t *r0 = box + (2 * qy + 6) * (BW / 2) + qx + 4;
            put_quad(k, io, qx, qy, r0[0], r0[BW / 2]);
        }
    }

    CRAW_DEV void run()
    {
        /* Low pass at R and B, and the four discriminations at every
         * pixel, from the 6x6 window around the quad. */
        for (int i = threadIdx.x; i < (QW + 4) * (QH + 4); i += NT) {
            int qx, qy;
            craw_row_item<QW + 4, QH + 4>(i, qx, qy);
            qx -= 2;
            qy -= 2;
            float v[6][6];
#pragma unroll
            for (int r = 0; r < 6; r++)
#pragma unroll
                for (int c = 0; c < 6; c += 2) {
                    float2 t = V2(2 * qx - 2 + c, 2 * qy - 2 + r);
                    v[r][c] = t.x;
                    v[r][c + 1] = t.y;
                }
            float lo[2];
#pragma unroll
            for (int s = 0; s < 2; s++) {
                const int cy = 2 + s, cx = 2 + s;
                lo[s] = rq_lowpass(v[cy][cx], v[cy - 1][cx], v[cy + 1][cx], v[cy][cx - 1], v[cy][cx + 1],
                                   v[cy - 1][cx - 1], v[cy - 1][cx + 1], v[cy + 1][cx - 1], v[cy + 1][cx + 1]);
            }
            Lat(qx, qy) = make_float2(lo[0], lo[1]);
#pragma unroll
            for (int b = 0; b < 2; b++)
#pragma unroll
                for (int a = 0; a < 2; a++) {
                    auto win = [&](int r, int c) { return v[b + r][a + c]; };
                    D(2 * qx + a, 2 * qy + b) = rq_disc4(win);
                }
        }
        __syncthreads();
        /* Weights: 3x3 means of the discriminations, as three-wide row sums
         * of a 4x4 window and then three of those rows; and in the same
         * pass, since it reads only its own quad's weights, green at R and
         * at B. */
        for (int i = threadIdx.x; i < (QW + 2) * (QH + 2); i += NT) {
            int qx, qy;
            craw_row_item<QW + 2, QH + 2>(i, qx, qy);
            qx -= 1;
            qy -= 1;
            float wv[2][2];
            float4 h[4][2];
#pragma unroll
            for (int r = 0; r < 4; r++) {
                float4 d0 = D(2 * qx - 1, 2 * qy - 1 + r), d1 = D(2 * qx, 2 * qy - 1 + r);
                float4 d2 = D(2 * qx + 1, 2 * qy - 1 + r), d3 = D(2 * qx + 2, 2 * qy - 1 + r);
                const float4 mid = rq_add4(d1, d2);
                h[r][0] = rq_add4(d0, mid);
                h[r][1] = rq_add4(mid, d3);
            }
#pragma unroll
            for (int a = 0; a < 2; a++) {
                const float4 mid = rq_add4(h[1][a], h[2][a]);
#pragma unroll
                for (int b = 0; b < 2; b++) {
                    const float4 sum = rq_add4(b == 0 ? h[0][a] : h[3][a], mid);
                    wv[b][a] = rq_wv(sum);
                    W(2 * qx + a, 2 * qy + b) = make_float2(wv[b][a], rq_wp(sum));
                }
            }
            const int x = 2 * qx, y = 2 * qy;
            float2 l0 = Lat(qx, qy), lu = Lat(qx, qy - 1), ld = Lat(qx, qy + 1);
            float2 ll = Lat(qx - 1, qy), lr = Lat(qx + 1, qy);
            const float g_r = rq_green(wv[0][0], l0.x, V(x, y - 1), lu.x, V(x, y + 1), ld.x, V(x - 1, y), ll.x,
                                       V(x + 1, y), lr.x);
            const float g_b = rq_green(wv[1][1], l0.y, V(x + 1, y), lu.y, V(x + 1, y + 2), ld.y, V(x, y + 1), ll.y,
                                       V(x + 2, y + 1), lr.y);
            G(qx, qy) = make_float2(g_r, g_b);
        }
        __syncthreads();
        /* The missing colour at R (from the B diagonals) and at B (from the
         * R diagonals); each only where a later pass reads it. */
        for (int i = threadIdx.x; i < (QW + 2) * (QH + 2); i += NT) {
            int qx, qy;
            craw_row_item<QW + 2, QH + 2>(i, qx, qy);
            qx -= 1;
            qy -= 1;
            const int x = 2 * qx, y = 2 * qy;
            float c_r = 0.0f, c_b = 0.0f;
            if (qx >= 0 && qy >= 0) {
                const float g00 = G(qx, qy).x;
                c_r = rq_cross(W(x, y).y, g00, __fsub_rn(V(x - 1, y + 1), G(qx - 1, qy).y),
                               __fsub_rn(V(x + 1, y - 1), G(qx, qy - 1).y),
                               __fsub_rn(V(x - 1, y - 1), G(qx - 1, qy - 1).y), __fsub_rn(V(x + 1, y + 1), G(qx, qy).y));
            }
            if (qx < QW && qy < QH) {
                const float g00 = G(qx, qy).y;
                c_b = rq_cross(W(x + 1, y + 1).y, g00, __fsub_rn(V(x, y + 2), G(qx, qy + 1).x),
                               __fsub_rn(V(x + 2, y), G(qx + 1, qy).x), __fsub_rn(V(x, y), G(qx, qy).x),
                               __fsub_rn(V(x + 2, y + 2), G(qx + 1, qy + 1).x));
            }
            Cat(qx, qy) = make_float2(c_r, c_b);
        }
        __syncthreads();
        /* The four output pixels of each quad, into the planar output. */
        constexpr int P = TW * TH;
        for (int i = threadIdx.x; i < QW * QH; i += NT) {
            const int qx = i % QW, qy = i / QW, x = 2 * qx, y = 2 * qy;
            float2 g0 = G(qx, qy), c0 = Cat(qx, qy);
            float2 gr = G(qx + 1, qy), cr = Cat(qx + 1, qy);   /* R of the right quad */
            float2 gd = G(qx, qy + 1), cd = Cat(qx, qy + 1);   /* R of the quad below */
            float2 gl = G(qx - 1, qy), cl = Cat(qx - 1, qy);   /* B of the left quad */
            float2 gu = G(qx, qy - 1), cu = Cat(qx, qy - 1);   /* B of the quad above */
            float2 top = V2(x, y), bot = V2(x, y + 1);         /* R, Gr / Gb, B */
            float o[4][3];
            /* R */
            o[0][0] = top.x; o[0][1] = g0.x; o[0][2] = c0.x;
            /* B */
            o[3][0] = c0.y; o[3][1] = g0.y; o[3][2] = bot.y;
            rq_green_site(W(x + 1, y).x, top.y,
                          __fsub_rn(top.x, g0.x), __fsub_rn(V(x + 2, y), gr.x),
                          __fsub_rn(cu.y, gu.y), __fsub_rn(c0.y, g0.y),
                          __fsub_rn(V(x + 1, y - 1), gu.y), __fsub_rn(bot.y, g0.y),
                          __fsub_rn(c0.x, g0.x), __fsub_rn(cr.x, gr.x), o[1][0], o[1][2]);
            o[1][1] = top.y;                                   /* Gr at (x + 1, y) */
            rq_green_site(W(x, y + 1).x, bot.x,
                          __fsub_rn(V(x - 1, y + 1), gl.y), __fsub_rn(bot.y, g0.y),
                          __fsub_rn(c0.x, g0.x), __fsub_rn(cd.x, gd.x),
                          __fsub_rn(top.x, g0.x), __fsub_rn(V(x, y + 2), gd.x),
                          __fsub_rn(cl.y, gl.y), __fsub_rn(c0.y, g0.y), o[2][2], o[2][0]);
            o[2][1] = bot.x;                                   /* Gb at (x, y + 1) */
            /* Pixels (x, y), (x + 1, y), (x, y + 1), (x + 1, y + 1) are quad
             * sites 0, 1, 2, 3. */
#pragma unroll
            for (int c = 0; c < 3; c++) {
                *reinterpret_cast<float2 *>(&rgb[c * P + y * TW + x]) = make_float2(o[0][c], o[1][c]);
                *reinterpret_cast<float2 *>(&rgb[c * P + (y + 1) * TW + x]) = make_float2(o[2][c], o[3][c]);
            }
        }
        __syncthreads();
    }
};

/* ------------------------------------------------------------- epilogue */

template <int TW, int TH, int NTH>
CRAW_DEV void awb_blocks(const CRAWKDevelop &k, const CRAWKDevelopIO &io, int x0, int y0, const float *rgb,
                         int t);

/* From the tile's camera RGB (planar in shared memory, fp32, complete):
 * the intermediate as it would be stored, then the colour stage into dst,
 * or the chroma block means, and the AWB block records. */
template <int TW, int TH, int NT>
CRAW_DEV void epilogue(const CRAWKDevelop &k, const CRAWKDevelopIO &io, int x0, int y0, float *rgb)
{
    constexpr int P = TW * TH;
    static_assert(P % 4 == 0 && TW % 8 == 0, "planes and block rows are whole float4s");
    const bool chroma = io.quarter != nullptr;
    /* With FP32 storage the AWB block sums read what the debayer left, so
     * the last warp makes them while the others run the colour stage: the
     * sums are long sequential chains over a few threads, and the tile's
     * slot on the SM is held until they end. */
    const bool awb_apart = !k.fp16 && !chroma && io.awb.rec && NT > 64;
    const int ncol = awb_apart ? NT - 32 : NT;
    if (awb_apart && (int)threadIdx.x >= ncol) {
        awb_blocks<TW, TH, 32>(k, io, x0, y0, rgb, threadIdx.x - ncol);
        return;
    }
    for (int i = threadIdx.x; i < P; i += ncol) {
        int x = x0 + i % TW, y = y0 + i / TW;
        float v[3] = { rgb[i], rgb[P + i], rgb[2 * P + i] };
        if (k.fp16) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
                v[c] = craw_round_half(v[c]);
                rgb[c * P + i] = v[c];
            }
        }
        if (x >= k.width || y >= k.height || !craw_in_bounds(x >= 0 && y >= 0, io.err))
            continue;
        if (io.inter)
            craw_store_rgba(io.inter, io.inter_pitch, x, y, k.fp16, v[0], v[1], v[2]);
        if (!chroma && io.dst) {
            float o[3];
            craw_color(k.color, v, o);
            craw_store_rgba(io.dst, io.dst_pitch, x, y, io.dst_fmt, o[0], o[1], o[2]);
        }
    }
    if ((!chroma && !io.awb.rec) || awb_apart)
        return;
    if (k.fp16)
        __syncthreads();

    if (chroma) {
        /* 4x4 block means of (R - G, B - G, G), row by row over the pixels
         * inside the frame (reference lib/ref/ref_chroma.c:49-74). */
        const int qw = (k.width + 3) / 4, qh = (k.height + 3) / 4;
        for (int b = threadIdx.x; b < (TW / 4) * (TH / 4); b += NT) {
            int bx = b % (TW / 4), by = b / (TW / 4);
            int qx = x0 / 4 + bx, qy = y0 / 4 + by;
            if (qx >= qw || qy >= qh)
                continue;
            float s0 = 0.f, s1 = 0.f, s2 = 0.f, n = 0.f;
            for (int jj = 0; jj < 4; jj++)
                for (int ii = 0; ii < 4; ii++) {
                    int x = bx * 4 + ii, y = by * 4 + jj;
                    if (x0 + x >= k.width || y0 + y >= k.height)
                        continue;
                    int j = y * TW + x;
                    float r = rgb[j], g = rgb[P + j], bl = rgb[2 * P + j];
                    s0 = __fadd_rn(s0, __fsub_rn(r, g));
                    s1 = __fadd_rn(s1, __fsub_rn(bl, g));
                    s2 = __fadd_rn(s2, g);
                    n += 1.0f;
                }
            craw_store_rgba(io.quarter, io.quarter_pitch, qx, qy, k.fp16,
                            __fdiv_rn(s0, n), __fdiv_rn(s1, n), __fdiv_rn(s2, n));
        }
        return;
    }

    awb_blocks<TW, TH, NT>(k, io, x0, y0, rgb, threadIdx.x);
}

/* The AWB records of the tile's 8x8 blocks, block means summed row by row
 * (reference lib/awb.c:239-253); thread t of NTH takes blocks t, t + NTH, ... */
template <int TW, int TH, int NTH>
CRAW_DEV void awb_blocks(const CRAWKDevelop &k, const CRAWKDevelopIO &io, int x0, int y0, const float *rgb,
                         int t)
{
    constexpr int P = TW * TH;
    const int blocks_x = (k.width + 7) / 8;
    for (int b = t; b < (TW / 8) * (TH / 8); b += NTH) {
        int bx = b % (TW / 8), by = b / (TW / 8);
        if (x0 + bx * 8 >= k.width || y0 + by * 8 >= k.height)
            continue;
        int xe = min(8, k.width - (x0 + bx * 8)), ye = min(8, k.height - (y0 + by * 8));
        float s0 = 0.f, s1 = 0.f, s2 = 0.f;
        if (xe == 8 && ye == 8) {
            /* A whole block: the same order, every row read as two 16-byte
             * loads a channel ahead of its dependent adds (rows one at a
             * time, so that the registers stay those of the rest). */
#pragma unroll 1
            for (int jj = 0; jj < 8; jj++) {
                const int j = (by * 8 + jj) * TW + bx * 8;
                const float4 r0 = *reinterpret_cast<const float4 *>(rgb + j);
                const float4 r1 = *reinterpret_cast<const float4 *>(rgb + j + 4);
                const float4 g0 = *reinterpret_cast<const float4 *>(rgb + P + j);
                const float4 g1 = *reinterpret_cast<const float4 *>(rgb + P + j + 4);
                const float4 b0 = *reinterpret_cast<const float4 *>(rgb + 2 * P + j);
                const float4 b1 = *reinterpret_cast<const float4 *>(rgb + 2 * P + j + 4);
                const float rr[8] = { r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w };
                const float gg[8] = { g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w };
                const float bb[8] = { b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w };
#pragma unroll
                for (int ii = 0; ii < 8; ii++) {
                    s0 = __fadd_rn(s0, rr[ii]);
                    s1 = __fadd_rn(s1, gg[ii]);
                    s2 = __fadd_rn(s2, bb[ii]);
                }
            }
        } else {
            for (int jj = 0; jj < ye; jj++)
                for (int ii = 0; ii < xe; ii++) {
                    int j = (by * 8 + jj) * TW + bx * 8 + ii;
                    s0 = __fadd_rn(s0, rgb[j]);
                    s1 = __fadd_rn(s1, rgb[P + j]);
                    s2 = __fadd_rn(s2, rgb[2 * P + j]);
                }
        }
        float n = (float)(xe * ye);
        const size_t ri = (size_t)(y0 / 8 + by) * blocks_x + x0 / 8 + bx;
        if (!craw_in_bounds(ri < craw_awb_blocks(k.width, k.height), io.err))
            continue;
        io.awb.rec[ri] =
            craw_awb_block(__fdiv_rn(s0, n), __fdiv_rn(s1, n), __fdiv_rn(s2, n), k.awb_wb,
                           io.awb.deferred, io.awb.nb_deferred,
                           craw_awb_blocks(k.width, k.height));
    }
}

/* ------------------------------------------------------------- kernels */

template <int METHOD, int TW, int TH, int NT> struct PixelSmem {
    static constexpr int A = Apron<METHOD>::v;
    /* Rounded to 4 floats: the planar output after it is read as float4. */
    static constexpr int work = ((METHOD == kRcd ? RcdTile<TW, TH, NT>::floats
                                                 : Tile<TW, TH, A, float>::N) + 3) & ~3;
    static constexpr int floats = work + 3 * TW * TH;
};

/* Interior tiles of the RCD by quads (QTW x QH pixels, all aprons inside
 * the frame); the per-pixel kernel below takes the rest. The single-frame
 * kernel uses QTH-row tiles with one thread per quad (QNT threads); the
 * batch kernel its own height and thread count. */
constexpr int QTW = 64, QTH = 16, QNT = 256, BTW = 32, BTH = 16;

template <int QH = QTH>
CRAW_DEV bool quad_interior(int x0, int y0, int w, int h)
{
    return x0 >= 6 && y0 >= 6 && x0 + QTW + 6 <= w && y0 + QH + 6 <= h;
}

/* One interior RCD tile at (x0, y0) by quads; NQ threads, `smem` holds
 * RcdQuads<QTW, QH, NQ>::floats floats. */
template <int QH = QTH, int NQ = QNT>
CRAW_DEV void rcd_quad_tile(const CRAWKDevelop &k, const CRAWKDevelopIO &io, int x0, int y0,
                            float *smem)
{
    RcdQuads<QTW, QH, NQ> t;
    t.carve(smem);
    t.load(k, io, x0, y0);
    __syncthreads();
    t.run();
    epilogue<QTW, QH, NQ>(k, io, x0, y0, t.rgb);
}

/* Per-pixel tiles: every bilinear and MHC tile, and the RCD tiles that the
 * quad kernel leaves (those whose QTW x QTH tile touches a border). */
/* One per-pixel tile at (x0, y0); NT threads, `smem` holds
 * PixelSmem<METHOD, TW, TH, NT>::floats floats. An RCD tile inside a
 * QTW x QH quad tile that rcd_quad_tile<QH>() takes is skipped. */
template <int METHOD, int TW, int TH, int NT, int QH = QTH>
CRAW_DEV void pixel_tile(const CRAWKDevelop &k, const CRAWKDevelopIO &io, int x0, int y0,
                         float *smem)
{
    constexpr int A = Apron<METHOD>::v;
    constexpr int PPT = TW * TH / NT;
    static_assert(TW * TH % NT == 0 && TW % 8 == 0 && TH % 8 == 0, "tile shape");
    float *rgb = smem + PixelSmem<METHOD, TW, TH, NT>::work;
    constexpr int P = TW * TH;

    Frame f;
    f.x0 = x0;
    f.y0 = y0;
    f.w = k.width;
    f.h = k.height;
    f.interior = f.x0 >= A && f.y0 >= A && f.x0 + TW + A <= k.width && f.y0 + TH + A <= k.height;

    if constexpr (METHOD == kRcd) {
        static_assert(QTW % TW == 0 && QH % TH == 0, "a quad tile is whole per-pixel tiles");
        if (quad_interior<QH>(f.x0 / QTW * QTW, f.y0 / QH * QH, k.width, k.height))
            return;
        RcdTile<TW, TH, NT> t;
        t.carve(smem);
        load_prepped<TW, TH, NT, 5>(k, io, f, t.v);
        __syncthreads();
        if (f.interior)
            t.template run<true>(f);
        else
            t.template run<false>(f);
#pragma unroll
        for (int j = 0; j < PPT; j++) {
            int i = threadIdx.x + j * NT, x = i % TW, y = i / TW;
            float o[3];
            t.pixel(x, y, ((f.y0 + y) & 1) * 2 + ((f.x0 + x) & 1), o);
            rgb[i] = o[0];
            rgb[P + i] = o[1];
            rgb[2 * P + i] = o[2];
        }
    } else {
        Tile<TW, TH, A, float> v;
        v.p = smem;
        load_prepped<TW, TH, NT, A>(k, io, f, v);
        __syncthreads();
#pragma unroll
        for (int j = 0; j < PPT; j++) {
            int i = threadIdx.x + j * NT, x = i % TW, y = i / TW;
            int s = ((f.y0 + y) & 1) * 2 + ((f.x0 + x) & 1);
            float o[3];
            if constexpr (METHOD == kBilinear)
                bilinear_px(v, x, y, s, o);
            else
                mhc_px(v, x, y, s, o);
            rgb[i] = o[0];
            rgb[P + i] = o[1];
            rgb[2 * P + i] = o[2];
        }
    }
    __syncthreads();
    epilogue<TW, TH, NT>(k, io, f.x0, f.y0, rgb);
}

} // namespace craw_dev
