/*
 * The fused develop kernel: prep + debayer + epilogue in one launch.
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
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace {

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
        uint16_t raw = __ldg((const uint16_t *)((const char *)io.src + (size_t)y * io.src_pitch) + x);
        v.p[i] = craw_prep(k, raw, (y & 1) * 2 + (x & 1));
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

/* ------------------------------------------------------------- kernel */

template <int METHOD, int TW, int TH, int NT> struct DevelopSmem {
    static constexpr int A = Apron<METHOD>::v;
    static constexpr int work = METHOD == kRcd ? RcdTile<TW, TH, NT>::floats
                                               : Tile<TW, TH, A, float>::N;
    static constexpr int floats = work + 3 * TW * TH;
};

template <int METHOD, int TW, int TH, int NT>
__global__ void __launch_bounds__(NT)
k_develop(const CRAWKDevelop k, const CRAWKDevelopIO io)
{
    constexpr int A = Apron<METHOD>::v;
    constexpr int PPT = TW * TH / NT;
    static_assert(TW * TH % NT == 0 && TW % 8 == 0 && TH % 8 == 0, "tile shape");
    __shared__ __align__(16) float smem[DevelopSmem<METHOD, TW, TH, NT>::floats];
    float *rgb_s = smem + DevelopSmem<METHOD, TW, TH, NT>::work;

    Frame f;
    f.x0 = blockIdx.x * TW;
    f.y0 = blockIdx.y * TH;
    f.w = k.width;
    f.h = k.height;
    f.interior = f.x0 >= A && f.y0 >= A && f.x0 + TW + A <= k.width && f.y0 + TH + A <= k.height;

    float out[PPT][3];
    if constexpr (METHOD == kRcd) {
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
            t.pixel(x, y, ((f.y0 + y) & 1) * 2 + ((f.x0 + x) & 1), out[j]);
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
            if constexpr (METHOD == kBilinear)
                bilinear_px(v, x, y, s, out[j]);
            else
                mhc_px(v, x, y, s, out[j]);
        }
    }

    /* Epilogue: the intermediate as it would be stored, then whatever the
     * frame needs of it. */
    const bool chroma = io.quarter != nullptr;
#pragma unroll
    for (int j = 0; j < PPT; j++) {
        int i = threadIdx.x + j * NT, x = f.x0 + i % TW, y = f.y0 + i / TW;
        if (k.fp16) {
#pragma unroll
            for (int c = 0; c < 3; c++)
                out[j][c] = craw_round_half(out[j][c]);
        }
        rgb_s[3 * i + 0] = out[j][0];
        rgb_s[3 * i + 1] = out[j][1];
        rgb_s[3 * i + 2] = out[j][2];
        if (x >= k.width || y >= k.height)
            continue;
        if (io.inter)
            craw_store_rgba(io.inter, io.inter_pitch, x, y, k.fp16, out[j][0], out[j][1], out[j][2]);
        if (!chroma && io.dst) {
            float o[3];
            craw_color(k.color, out[j], o);
            craw_store_rgba(io.dst, io.dst_pitch, x, y, io.dst_half, o[0], o[1], o[2]);
        }
    }
    if (!chroma && !io.awb.rec)
        return;
    __syncthreads();

    if (chroma) {
        /* 4x4 block means of (R - G, B - G, G), summed row by row over the
         * pixels inside the frame (reference lib/ref/ref_chroma.c:49-74). */
        constexpr int QB = (TW / 4) * (TH / 4);
        for (int b = threadIdx.x; b < QB; b += NT) {
            int bx = b % (TW / 4), by = b / (TW / 4);
            int qx = f.x0 / 4 + bx, qy = f.y0 / 4 + by;
            int qw = (k.width + 3) / 4, qh = (k.height + 3) / 4;
            if (qx >= qw || qy >= qh)
                continue;
            float s0 = 0.f, s1 = 0.f, s2 = 0.f, n = 0.f;
            for (int jj = 0; jj < 4; jj++)
                for (int ii = 0; ii < 4; ii++) {
                    int x = bx * 4 + ii, y = by * 4 + jj;
                    if (f.x0 + x >= k.width || f.y0 + y >= k.height)
                        continue;
                    const float *p = &rgb_s[3 * (y * TW + x)];
                    s0 = __fadd_rn(s0, __fsub_rn(p[0], p[1]));
                    s1 = __fadd_rn(s1, __fsub_rn(p[2], p[1]));
                    s2 = __fadd_rn(s2, p[1]);
                    n += 1.0f;
                }
            float m0 = __fdiv_rn(s0, n), m1 = __fdiv_rn(s1, n), m2 = __fdiv_rn(s2, n);
            craw_store_rgba(io.quarter, io.quarter_pitch, qx, qy, k.fp16, m0, m1, m2);
        }
        return;
    }

    /* 8x8 block means, row by row (reference lib/awb.c:239-253). */
    constexpr int AB = (TW / 8) * (TH / 8);
    const int blocks_x = (k.width + 7) / 8;
    for (int b = threadIdx.x; b < AB; b += NT) {
        int bx = b % (TW / 8), by = b / (TW / 8);
        if (f.x0 + bx * 8 >= k.width || f.y0 + by * 8 >= k.height)
            continue;
        int xe = min(8, k.width - (f.x0 + bx * 8)), ye = min(8, k.height - (f.y0 + by * 8));
        float s0 = 0.f, s1 = 0.f, s2 = 0.f;
        for (int jj = 0; jj < ye; jj++)
            for (int ii = 0; ii < xe; ii++) {
                const float *p = &rgb_s[3 * ((by * 8 + jj) * TW + bx * 8 + ii)];
                s0 = __fadd_rn(s0, p[0]);
                s1 = __fadd_rn(s1, p[1]);
                s2 = __fadd_rn(s2, p[2]);
            }
        float n = (float)(xe * ye);
        uint64_t rec = craw_awb_block(__fdiv_rn(s0, n), __fdiv_rn(s1, n), __fdiv_rn(s2, n),
                                      k.awb_wb, io.awb.deferred, io.awb.nb_deferred);
        io.awb.rec[(size_t)(f.y0 / 8 + by) * blocks_x + f.x0 / 8 + bx] = rec;
    }
}

template <int METHOD, int TW, int TH, int NT>
int launch(const CRAWKDevelop *k, const CRAWKDevelopIO *io, cudaStream_t s)
{
    dim3 grid((k->width + TW - 1) / TW, (k->height + TH - 1) / TH);
    k_develop<METHOD, TW, TH, NT><<<grid, NT, 0, s>>>(*k, *io);
    return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

} // namespace

extern "C" int craw_k_develop(const CRAWKDevelop *k, const CRAWKDevelopIO *io, int shape,
                              cudaStream_t s)
{
    (void)cudaGetLastError();   /* a stale error of an earlier call is not ours */
    (void)shape;
    switch (k->method) {
    case kBilinear: return launch<kBilinear, 64, 16, 256>(k, io, s);
    case kMhc:      return launch<kMhc, 64, 16, 256>(k, io, s);
    case kRcd:      return launch<kRcd, 32, 16, 256>(k, io, s);
    default:        return -22;
    }
}
