/*
 * The RCD of the frame's interior by strips (reference
 * lib/ref/ref_debayer.c:204-395; the passes of lib/shaders/rcd.comp.glsl).
 *
 * A CTA of SNT threads owns a strip of quad columns, one column a thread,
 * and walks down a segment of it one quad row (two pixel rows) a step.
 * Each pass of the RCD runs a fixed number of quad rows behind the one
 * before it, so a step does every pass once for every column:
 *
 *   stage A   D, L of quad row s (the four discriminations of the quad's
 *             pixels, the low pass at R and B);
 *             C of row s - 3 (the missing colour at R and B);
 *             the colour stage and stores of output row s - 5, and its
 *             AWB block sums (three threads a block, one a channel)
 *   barrier
 *   stage B   the 3-wide row sums of D of row s (a neighbour's edge pixel
 *             read from shared memory); W and G of row s - 1 (the weights
 *             from the 3x3 sums kept in registers down the column; green
 *             at R and B from the low passes of the column and its
 *             neighbours); the camera RGB of output row s - 4 into the
 *             output ring; the prepped mosaic of the rows step s + 1 needs
 *   barrier
 *
 * What a pass hands to the next lives in shared-memory rings a few quad
 * rows deep, so every value is computed once (the 64x16 tiles compute a
 * third to two thirds of their D, W and G twice, in their aprons) and
 * every thread has the same work in every pass. The arithmetic is the
 * tiles' (the rq_* helpers, explicit roundings), so both give the same
 * bits. Interior strips only: every pixel read, down to six outside the
 * strip's output, lies inside the frame.
 */
#pragma once

#include <type_traits>

#include "develop_tile.cuh"

namespace craw_dev {

constexpr int SNT = 128;                 /* threads: one quad column each */
constexpr int SOUT = SNT - 4;            /* output quad columns of a full strip */
constexpr int SVR = 16;                  /* pixel rows in the prepped-mosaic ring */
constexpr int SVS = 2 * SNT + 8;         /* its row stride, floats (260 used) */
constexpr int SQ = SNT + 2;              /* a quad ring's row: columns -1 .. SNT */
constexpr int SLR = 4, SGR = 8, SCR = 4, SWR = 4;   /* quad rows of the L, G, C, W rings */
constexpr int SAW = 2 * SOUT;            /* AWB ring row: the strip's output pixels */

/* Ring rows are indexed by the row (pixel or quad, relative to the
 * segment's first output row, >= -6) modulo their depth. Columns: the
 * mosaic ring holds frame pixel columns 2 ox - 6 .. 2 ox + 2 SOUT + 5
 * (ox: the strip's first output quad), thread j's own pixels at 2 j + 2
 * and 2 j + 3; the quad rings hold thread j's value at j + 1. */
struct StripSmem {
    float v[SVR * SVS];
    float4 d[2][2][SQ];       /* D of quad row s: [pixel row][even, odd pixel][j + 1] */
    float2 l[SLR][SQ];        /* low pass at (R, B) */
    float2 g[SGR][SQ];        /* green at (R, B) */
    float2 c[SCR][SQ];        /* B at R, R at B */
    float4 w[SWR][SNT];       /* (wp at R, wp at B, wv at Gr, wv at Gb), own column only */
    float a[3][2][SAW];       /* camera RGB of the last output quad row, planar: the
                               * colour stage and the AWB sums read it a step later */
};

/* The interior the strips cover, in quads: columns qx0 .. qx0 + nqx, rows
 * qy0 .. qy0 + nqy, in segments of seg rows a CTA (nqx, nqy and seg
 * multiples of 4, 2 qx0 and 2 qy0 multiples of 8, so that strips and
 * segments start on 8x8 AWB blocks). */
struct StripGrid {
    int qx0, nqx, qy0, nqy, seg;
};

struct Strip {
    const CRAWKDevelop &k;
    const CRAWKDevelopIO &io;
    StripSmem &S;
    int j, ox, oy, nout, nrows;

    CRAW_DEV float V(int yr, int cv) const { return S.v[(yr & (SVR - 1)) * SVS + cv]; }
    CRAW_DEV float2 V2(int yr, int cv) const
    {
        return *reinterpret_cast<const float2 *>(&S.v[(yr & (SVR - 1)) * SVS + cv]);
    }
    CRAW_DEV float2 G(int jj, int r) const { return S.g[r & (SGR - 1)][jj + 1]; }
    CRAW_DEV float2 C(int jj, int r) const { return S.c[r & (SCR - 1)][jj + 1]; }
    CRAW_DEV float2 L(int jj, int r) const { return S.l[r & (SLR - 1)][jj + 1]; }

    /* Mosaic quad column m of the ring (frame pixels 2 ox - 6 + 2 m, + 1),
     * pixel row yr, as its two raw samples. */
    CRAW_DEV uint32_t fetch(int yr, int m) const
    {
        const int y = 2 * oy + yr, x = 2 * (ox - 3 + m);
        if (!craw_in_bounds(y >= 0 && y < k.height && x >= 0 && x + 1 < k.width, io.err))
            return 0u;
        const char *row = (const char *)io.src + (size_t)y * io.src_pitch;
        return __ldg(reinterpret_cast<const uint32_t *>(row) + (ox - 3 + m));
    }
    CRAW_DEV void put(int yr, int m, uint32_t raw) const
    {
        float2 t;
        if (io.src_f16) {
            t = __half22float2(*reinterpret_cast<const __half2 *>(&raw));
        } else {
            const int s0 = (yr & 1) * 2;
            t = make_float2(craw_prep(k, (uint16_t)(raw & 0xffff), s0), craw_prep(k, (uint16_t)(raw >> 16), s0 + 1));
        }
        if (craw_in_bounds(m >= 0 && 2 * m + 1 < SVS, io.err))
            *reinterpret_cast<float2 *>(&S.v[(yr & (SVR - 1)) * SVS + 2 * m]) = t;
    }
};

template <int NT = SNT>
CRAW_DEV void rcd_strip(const CRAWKDevelop &k, const CRAWKDevelopIO &io, const StripGrid &g, int sx, int sy,
                        StripSmem &S)
{
    static_assert(NT == SNT, "one thread a quad column");
    Strip t{ k, io, S, (int)threadIdx.x, g.qx0 + sx * SOUT, g.qy0 + sy * g.seg,
             min(SOUT, g.nqx - sx * SOUT), min(g.seg, g.nqy - sy * g.seg) };
    const int j = t.j, nout = t.nout, nrows = t.nrows;
    const int X = 2 * j + 2;                      /* own left pixel's ring column */
    const bool p1 = j < nout + 4;                 /* D and L */
    const bool p2 = j >= 1 && j < nout + 3;       /* W, G and C */
    const bool po = j >= 2 && j < nout + 2;       /* output */
    const bool awb = io.awb.rec != nullptr;
    const bool fp16 = k.fp16 != 0;
    /* The mosaic columns this thread fills: its own, and the ring's two
     * edge columns on threads 0 and 1. */
    const int m0 = j + 1 <= nout + 5 ? j + 1 : -1;
    const int m1 = j == 0 ? 0 : (j == 1 && nout + 5 >= SNT + 1 ? SNT + 1 : -1);
    /* AWB: threads 4 b, 4 b + 1, 4 b + 2 (one warp) sum the R, G and B of
     * block b of the strip's output row of blocks. */
    const int ab = j >> 2, ac = j & 3;
    const bool folder = awb && ac < 3 && ab < nout / 4;
    float asum = 0.0f;

    /* The first six rows of the ring, then the next two in registers. */
    for (int yr = -6; yr < 0; yr++) {
        if (m0 >= 0)
            t.put(yr, m0, t.fetch(yr, m0));
        if (m1 >= 0)
            t.put(yr, m1, t.fetch(yr, m1));
    }
    uint32_t pf[2][2] = { { 0u, 0u }, { 0u, 0u } };
#pragma unroll
    for (int r = 0; r < 2; r++) {
        if (m0 >= 0)
            pf[r][0] = t.fetch(r, m0);
        if (m1 >= 0)
            pf[r][1] = t.fetch(r, m1);
    }
    __syncthreads();

    float4 hc[3][2];                      /* 3-wide row sums of D, pixel rows 2s - 3 .. 2s - 1 */
#pragma unroll
    for (int r = 0; r < 3; r++)
        hc[r][0] = hc[r][1] = make_float4(0.f, 0.f, 0.f, 0.f);

    /* The AWB sums of output quad row r (two pixel rows of the block, in
     * its row-major order, one channel a thread), and the block's record
     * once its eight rows are in (every thread of the CTA takes part: the
     * record gathers the three sums by warp shuffles). */
    auto awb_fold = [&](int r) {
        if (folder) {
#pragma unroll
            for (int jj = 0; jj < 2; jj++) {
                const float *pa = &S.a[ac][jj][8 * ab];
                const float4 q0 = *reinterpret_cast<const float4 *>(pa), q1 = *reinterpret_cast<const float4 *>(pa + 4);
                const float q[8] = { q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w };
#pragma unroll
                for (int ii = 0; ii < 8; ii++)
                    asum = __fadd_rn(asum, q[ii]);
            }
        }
        if ((r & 3) == 3) {
            const float sg = __shfl_down_sync(0xffffffffu, asum, 1), sb = __shfl_down_sync(0xffffffffu, asum, 2);
            if (folder && ac == 0) {
                const int bx = (2 * t.ox) / 8 + ab, by = (2 * t.oy + 2 * r - 6) / 8;
                const size_t ri = (size_t)by * ((k.width + 7) / 8) + bx;
                if (craw_in_bounds(bx >= 0 && by >= 0 && ri < craw_awb_blocks(k.width, k.height), io.err))
                    io.awb.rec[ri] = craw_awb_block(__fdiv_rn(asum, 64.0f), __fdiv_rn(sg, 64.0f),
                                                    __fdiv_rn(sb, 64.0f), k.awb_wb, io.awb.deferred,
                                                    io.awb.nb_deferred, craw_awb_blocks(k.width, k.height));
            }
            asum = 0.0f;
        }
    };

    /* The colour stage and the stores of output quad row r from the output
     * ring, pixel by pixel along its two rows (consecutive threads on
     * consecutive pixels, as the tiles' epilogue: coalesced stores, and the
     * gamut compression's branches taken alike by neighbours). */
    auto colour_rows = [&](int r) {
        const int rw = 2 * nout;
#pragma unroll 1
        for (int i = j; i < 2 * rw; i += SNT) {
            const int jj = i >= rw, c = i - jj * rw;
            const float v[3] = { S.a[0][jj][c], S.a[1][jj][c], S.a[2][jj][c] };
            const int px = 2 * t.ox + c, py = 2 * (t.oy + r) + jj;
            if (!craw_in_bounds(px >= 0 && px < k.width && py >= 0 && py < k.height && c < SAW, io.err))
                continue;
            if (io.inter)
                craw_store_rgba(io.inter, io.inter_pitch, px, py, k.fp16, v[0], v[1], v[2]);
            if (io.dst) {
                float q[3];
                craw_color(k.color, v, q);
                craw_store_rgba(io.dst, io.dst_pitch, px, py, io.dst_fmt, q[0], q[1], q[2]);
            }
        }
    };

    /* One step. ST: a step of the steady state (5 <= s <= nrows + 1),
     * where every pass has a row to do; there every thread runs every
     * pass, the threads outside a pass's columns on neighbouring (or
     * unfilled) ring entries whose results nothing reads, and only the
     * global stores and the AWB ring are kept to the output columns: one
     * basic block, so the passes' dependency chains interleave. */
    auto step = [&](const int s, auto steady) {
        constexpr bool ST = decltype(steady)::value;
        /* ---------------------------------------------------- stage A */
        float4 dd[2][2];                  /* own D of quad row s: [pixel row][pixel] */
        if (ST || (s <= nrows + 1 && p1)) {
            const int Y = 2 * s;
            float v[6][6];
#pragma unroll
            for (int r = 0; r < 6; r++)
#pragma unroll
                for (int c = 0; c < 6; c += 2) {
                    const float2 q = t.V2(Y - 2 + r, X - 2 + c);
                    v[r][c] = q.x;
                    v[r][c + 1] = q.y;
                }
            float lo[2];
#pragma unroll
            for (int e = 0; e < 2; e++) {
                const int cy = 2 + e, cx = 2 + e;
                lo[e] = rq_lowpass(v[cy][cx], v[cy - 1][cx], v[cy + 1][cx], v[cy][cx - 1], v[cy][cx + 1],
                                   v[cy - 1][cx - 1], v[cy - 1][cx + 1], v[cy + 1][cx - 1], v[cy + 1][cx + 1]);
            }
            S.l[s & (SLR - 1)][j + 1] = make_float2(lo[0], lo[1]);
#pragma unroll
            for (int b = 0; b < 2; b++)
#pragma unroll
                for (int a = 0; a < 2; a++) {
                    auto win = [&](int r, int c) { return v[b + r][a + c]; };
                    dd[b][a] = rq_disc4(win);
                    S.d[b][a][j + 1] = dd[b][a];
                }
        }
        if (ST || (s >= 2 && p2)) {
            /* C of quad row r (its R part is read by the output from row
             * 0 on, its B part down to row -1). */
            const int r = s - 3, Y = 2 * r;
            const float4 w4 = S.w[r & (SWR - 1)][j];
            const float2 g00 = t.G(j, r), gl = t.G(j - 1, r), gu = t.G(j, r - 1), gul = t.G(j - 1, r - 1);
            const float2 gd = t.G(j, r + 1), gr = t.G(j + 1, r), gdr = t.G(j + 1, r + 1);
            const float c_r = rq_cross(w4.x, g00.x, __fsub_rn(t.V(Y + 1, X - 1), gl.y),
                                       __fsub_rn(t.V(Y - 1, X + 1), gu.y), __fsub_rn(t.V(Y - 1, X - 1), gul.y),
                                       __fsub_rn(t.V(Y + 1, X + 1), g00.y));
            const float c_b = rq_cross(w4.y, g00.y, __fsub_rn(t.V(Y + 2, X), gd.x),
                                       __fsub_rn(t.V(Y, X + 2), gr.x), __fsub_rn(t.V(Y, X), g00.x),
                                       __fsub_rn(t.V(Y + 2, X + 2), gdr.x));
            S.c[r & (SCR - 1)][j + 1] = make_float2(c_r, c_b);
        }
        if (ST || s >= 5) {
            colour_rows(s - 5);
            if (awb)
                awb_fold(s - 5);
        }
        __syncthreads();

        /* ---------------------------------------------------- stage B */
        if (ST || (s <= nrows + 1 && p2)) {
            float4 hn[2][2];
#pragma unroll
            for (int b = 0; b < 2; b++) {
                const float4 mid = rq_add4(dd[b][0], dd[b][1]);
                hn[b][0] = rq_add4(S.d[b][1][j], mid);         /* D at 2 j - 1: the left quad's odd pixel */
                hn[b][1] = rq_add4(mid, S.d[b][0][j + 2]);     /* D at 2 j + 2: the right quad's even pixel */
            }
            if (ST || s >= 0) {
                /* W and G of quad row r = s - 1: the 3x3 sums of pixel rows
                 * 2r - 1 .. 2r + 2 are hc[0..2], hn[0]. */
                const int r = s - 1, Y = 2 * r;
                float4 sum[2][2];
#pragma unroll
                for (int a = 0; a < 2; a++) {
                    const float4 mid = rq_add4(hc[1][a], hc[2][a]);
                    sum[0][a] = rq_add4(hc[0][a], mid);
                    sum[1][a] = rq_add4(hn[0][a], mid);
                }
                const float wv_r = rq_wv(sum[0][0]), wv_b = rq_wv(sum[1][1]);
                S.w[r & (SWR - 1)][j] = make_float4(rq_wp(sum[0][0]), rq_wp(sum[1][1]), rq_wv(sum[0][1]),
                                                    rq_wv(sum[1][0]));
                const float2 l0 = t.L(j, r), lu = t.L(j, r - 1), ld = t.L(j, r + 1);
                const float2 ll = t.L(j - 1, r), lr = t.L(j + 1, r);
                const float g_r = rq_green(wv_r, l0.x, t.V(Y - 1, X), lu.x, t.V(Y + 1, X), ld.x, t.V(Y, X - 1), ll.x,
                                           t.V(Y, X + 1), lr.x);
                const float g_b = rq_green(wv_b, l0.y, t.V(Y, X + 1), lu.y, t.V(Y + 2, X + 1), ld.y, t.V(Y + 1, X),
                                           ll.y, t.V(Y + 1, X + 2), lr.y);
                S.g[r & (SGR - 1)][j + 1] = make_float2(g_r, g_b);
            }
#pragma unroll
            for (int a = 0; a < 2; a++) {
                hc[0][a] = hc[2][a];
                hc[1][a] = hn[0][a];
                hc[2][a] = hn[1][a];
            }
        }
        if (ST || (s >= 4 && po)) {
            /* The four pixels of output quad row r = s - 4. */
            const int r = s - 4, Y = 2 * r;
            const float4 w4 = S.w[r & (SWR - 1)][j];
            const float2 g0 = t.G(j, r), c0 = t.C(j, r);
            const float2 gr = t.G(j + 1, r), cr = t.C(j + 1, r);   /* R of the right quad */
            const float2 gd = t.G(j, r + 1), cd = t.C(j, r + 1);   /* R of the quad below */
            const float2 gl = t.G(j - 1, r), cl = t.C(j - 1, r);   /* B of the left quad */
            const float2 gu = t.G(j, r - 1), cu = t.C(j, r - 1);   /* B of the quad above */
            const float2 top = t.V2(Y, X), bot = t.V2(Y + 1, X);   /* R, Gr / Gb, B */
            float o[4][3];
            o[0][0] = top.x; o[0][1] = g0.x; o[0][2] = c0.x;
            o[3][0] = c0.y;  o[3][1] = g0.y; o[3][2] = bot.y;
            rq_green_site(w4.z, top.y,
                          __fsub_rn(top.x, g0.x), __fsub_rn(t.V(Y, X + 2), gr.x),
                          __fsub_rn(cu.y, gu.y), __fsub_rn(c0.y, g0.y),
                          __fsub_rn(t.V(Y - 1, X + 1), gu.y), __fsub_rn(bot.y, g0.y),
                          __fsub_rn(c0.x, g0.x), __fsub_rn(cr.x, gr.x), o[1][0], o[1][2]);
            o[1][1] = top.y;
            rq_green_site(w4.w, bot.x,
                          __fsub_rn(t.V(Y + 1, X - 1), gl.y), __fsub_rn(bot.y, g0.y),
                          __fsub_rn(c0.x, g0.x), __fsub_rn(cd.x, gd.x),
                          __fsub_rn(top.x, g0.x), __fsub_rn(t.V(Y + 2, X), gd.x),
                          __fsub_rn(cl.y, gl.y), __fsub_rn(c0.y, g0.y), o[2][2], o[2][0]);
            o[2][1] = bot.x;
            /* Camera RGB (rounded to half with FP16 storage) into the
             * output ring: the next step's colour stage and AWB sums read
             * it. */
            const int ax = 2 * (j - 2);
            if (fp16) {
#pragma unroll
                for (int p = 0; p < 4; p++)
#pragma unroll
                    for (int c = 0; c < 3; c++)
                        o[p][c] = craw_round_half(o[p][c]);
            }
            if (po) {
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    *reinterpret_cast<float2 *>(&S.a[c][0][ax]) = make_float2(o[0][c], o[1][c]);
                    *reinterpret_cast<float2 *>(&S.a[c][1][ax]) = make_float2(o[2][c], o[3][c]);
                }
            }
        }
        /* The mosaic rows of step s + 1, and the loads of the two after. */
        if (s <= nrows) {
#pragma unroll
            for (int r = 0; r < 2; r++) {
                if (m0 >= 0)
                    t.put(2 * s + 4 + r, m0, pf[r][0]);
                if (m1 >= 0)
                    t.put(2 * s + 4 + r, m1, pf[r][1]);
            }
            if (s < nrows) {
#pragma unroll
                for (int r = 0; r < 2; r++) {
                    if (m0 >= 0)
                        pf[r][0] = t.fetch(2 * s + 6 + r, m0);
                    if (m1 >= 0)
                        pf[r][1] = t.fetch(2 * s + 6 + r, m1);
                }
            }
        }
        __syncthreads();
    };
    int s = -2;
#pragma unroll 1
    for (; s < 5 && s <= nrows + 3; s++)
        step(s, std::false_type{});
#pragma unroll 1
    for (; s <= nrows + 1; s++)
        step(s, std::true_type{});
#pragma unroll 1
    for (; s <= nrows + 3; s++)
        step(s, std::false_type{});
    colour_rows(nrows - 1);
    if (awb)
        awb_fold(nrows - 1);
}

} // namespace craw_dev
