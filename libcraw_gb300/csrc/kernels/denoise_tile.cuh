/*
 * The raw-domain denoise, one tile: temporal recursive average + variance-
 * stabilising transform + non-local means on the four CFA planes, in one
 * launch (the reference's denoise_nlm pass; CPU definition
 * lib/ref/ref_denoise.c:168-336).
 *
 * One CTA filters the same OX x OY tile of all four planes, i.e. a
 * 2*OX x 2*OY region of the mosaic, so that the mosaic, the state and the
 * outputs move as whole 2x2 quads with 32-bit (mosaic) and 64-bit (state)
 * accesses. The stabilised planes of the tile and its search+patch apron
 * live in shared memory as FP32.
 *
 * The search: a thread owns BW columns x M rows of one plane. For a
 * search offset (dx, dy) it forms the squared differences of its own
 * (BW+2) x (M+2) window against the shifted one, sums them along x and
 * then along y in registers (sharing the middle pair of each three-sum),
 * and turns each of its BW*M patch distances into a weight with one ex2
 * on the MUFU. For one dy the shifted rows of all seven dx are a single
 * register block, read from shared memory once; dy is a runtime loop so
 * that the unrolled body of seven dx stays in the instruction cache.
 */
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "tma.cuh"

namespace craw_dn {


constexpr int S = 3;     /* search radius, reference lib/pipeline.c:261 */
constexpr int P = 1;     /* patch radius, reference lib/pipeline.c:262 */
constexpr float kLog2e = 1.4426950408889634f;
constexpr float kVarMin = 1.0e-4f;

CRAW_DEV float gat_fwd(const CRAWKDenoise &k, float u)
{
    if (u >= 0.0f)
        return k.gat_fwd * sqrtf(k.gat_a * u + k.gat_c);
    return k.gat_t0 + __fdiv_rn(u, k.gat_sc);
}

CRAW_DEV float gat_inv(const CRAWKDenoise &k, float t)
{
    if (t >= k.gat_t0)
        return k.gat_inv * t * t - k.gat_off;
    return (t - k.gat_t0) * k.gat_sc;
}

CRAW_DEV float pick4(const float a[4], int i)
{
    return i == 0 ? a[0] : (i == 1 ? a[1] : (i == 2 ? a[2] : a[3]));
}

CRAW_DEV float level(const CRAWKDenoise &k, uint32_t raw, int pl)
{
    return ((float)raw * (1.0f / 65535.0f) - k.black[pl]) * k.inv_range[pl];
}

/* The four plane samples of mosaic quad (qx, qy): R, Gr, Gb, B. */
/* The quad at plane position (qx, qy): its two mosaic rows as 32-bit
 * pairs (a: R, Gr; b: Gb, B) and the four samples. */
CRAW_DEV void load_quad_u16(const CRAWKDenoise &k, const CRAWKDenoiseIO &io, int qx, int qy, uint32_t q[4],
                           uint32_t &a, uint32_t &b, uint32_t *err)
{
    a = b = 0u;
    if (craw_in_bounds(qx >= 0 && qx < k.pw && qy >= 0 && qy < k.ph, err)) {
        const char *r0 = (const char *)io.src + (size_t)(2 * qy) * io.src_pitch;
        a = __ldg(reinterpret_cast<const uint32_t *>(r0) + qx);
        b = __ldg(reinterpret_cast<const uint32_t *>(r0 + io.src_pitch) + qx);
    }
    q[0] = a & 0xffffu; q[1] = a >> 16; q[2] = b & 0xffffu; q[3] = b >> 16;
}

/* Keeps the raw rows of a quad of the tile's own region (plane position
 * (cc, cr) within it) in the RW_W-wide raw array. */
template <int OX, int OY>
CRAW_DEV void keep_raw(uint32_t *rw, int cr, int cc, uint32_t a, uint32_t b)
{
    if (cr >= 0 && cr < OY && cc >= 0 && cc < OX) {
        rw[(2 * cr) * OX + cc] = a;
        rw[(2 * cr + 1) * OX + cc] = b;
    }
}

CRAW_DEV void load_quad_f32(const CRAWKDenoise &k, const float *base, size_t pitch, int qx, int qy, float q[4],
                           uint32_t *err)
{
    float2 a = make_float2(0.f, 0.f), b = a;
    if (craw_in_bounds(qx >= 0 && qx < k.pw && qy >= 0 && qy < k.ph, err)) {
        const char *r0 = (const char *)base + (size_t)(2 * qy) * pitch;
        a = __ldg(reinterpret_cast<const float2 *>(r0) + qx);
        b = __ldg(reinterpret_cast<const float2 *>(r0 + pitch) + qx);
    }
    q[0] = a.x; q[1] = a.y; q[2] = b.x; q[3] = b.y;
}

/* STAGED: the tile's raw mosaic and its output pass through shared memory
 * (below); the batch's persistent kernel leaves it off, whose shared
 * memory would otherwise cost it a CTA an SM. */
template <int BW, int M, int WP, bool SPATIAL, bool TEMPORAL, bool HISTORY, bool X2 = false, bool STAGED = true,
          bool TMA = false>
struct Cfg {
    static constexpr int R = SPATIAL ? S + P : 0;       /* apron of the tile */
    static constexpr int OX = 16 * BW, OY = 2 * M * WP;  /* plane samples per tile */
    static constexpr int TX = OX + 2 * R, TY = OY + 2 * R;
    static constexpr int TS = (TX + 1) & ~1;             /* row stride, even for float2 */
    static constexpr int TN = TY * TS;                   /* one plane's tile */
    static constexpr int EX = TX + 2, EY = TY + 2;       /* history: one more ring */
    static constexpr int EN = EX * EY;
    static constexpr int NT = 4 * WP * 32;
    /* The packed search (X2) keeps copies of the tile (and, with a
     * history, of the variance) shifted left by one sample, so that odd
     * column pairs load as aligned float2: TO and VO, after the rest.
     * (Placing them over the history's ring arrays, dead once the temporal
     * average is done, needs a separate copy pass after a barrier; at
     * 5760x3240 that cost more than the third CTA an SM it allows.) */
    static constexpr bool PACKED = X2 && SPATIAL;
    static constexpr int TO_OFF = HISTORY ? 8 * TN + 8 * EN : 4 * TN;
    static constexpr int VO_OFF = TO_OFF + 4 * TN;
    static constexpr int BASE_FLOATS = 4 * TN * (HISTORY ? 2 : 1) + (HISTORY ? 8 * EN : 0) +
                                       (PACKED ? 4 * TN * (HISTORY ? 2 : 1) : 0);
    /* The tile's own mosaic region, 2 OX x 2 OY 16-bit samples: the raw
     * samples the fill read (for the highlight guard), then the denoised
     * output until it is stored as whole 16-byte rows. */
    static constexpr int RW_W = 2 * OX, RW_H = 2 * OY;
    static constexpr int RW_OFF = BASE_FLOATS;
    static_assert(RW_OFF % 4 == 0 && RW_W % 8 == 0, "16-byte rows");
    /* TMA (spatial filtering only): the mosaic region of the tile and its
     * apron, 2 TX x 2 TY samples, as one tile copy leaves it, after the
     * rest (with room to align it to 128 bytes). */
    static constexpr int BOX_W = 2 * TX, BOX_H = 2 * TY;
    static constexpr uint32_t BOX_BYTES = BOX_W * BOX_H * 2;
    static constexpr int BOX_OFF = BASE_FLOATS + (STAGED ? RW_W * RW_H / 2 : 0);
    static constexpr int smem_floats = BOX_OFF + (TMA ? (int)BOX_BYTES / 4 + 32 : 0);
};

/* The NLM search of one thread: BW columns x M rows of one plane, at the
 * tile position (ox0, oy0), over the 7x7 offsets (reference
 * lib/ref/ref_denoise.c:109-154). Weights as exp2 on the MUFU:
 * exp(-max(d2/(9h^2) - 2, 0)) = 2^min(d2 * c1 + c0, 0) with
 * c1 = -log2(e)/(9h^2), c0 = 2 log2(e); with a history
 * exp(-max(d2/(9h^2) - (vc + vq), 0) / vc) = 2^min((vc + vq - d2/(9h^2)) * log2(e)/vc, 0),
 * expanded as 2^min(log2(e) + vq * lvc + d2 * nkl, 0) with the centre's
 * lvc = log2(e)/vc and nkl = -lvc/(9h^2) taken out of the search: two
 * multiply-adds an offset. */
template <int BW, int M, int R, int TS, bool HISTORY, bool CENTRE>
struct Search {
    static_assert(BW % 2 == 0 && M % 2 == 0, "pairs of columns and rows");
    float own[M + 2][BW + 2];
    float acc[M][BW], wsum[M][BW];
    float nkl[HISTORY ? M : 1][BW], lvc[HISTORY ? M : 1][BW];
    float kd, c1, c0;

    CRAW_DEV void init(const float *Tp, const float *Vp, int ox0, int oy0, float inv_h2)
    {
#pragma unroll
        for (int r = 0; r < M + 2; r++)
#pragma unroll
            for (int c = 0; c < BW + 2; c++)
                own[r][c] = Tp[(oy0 + R - 1 + r) * TS + ox0 + R - 1 + c];
        kd = (1.0f / 9.0f) * inv_h2;
        c1 = -kLog2e * kd;
        c0 = 2.0f * kLog2e;
#pragma unroll
        for (int m = 0; m < M; m++)
#pragma unroll
            for (int j = 0; j < BW; j++) {
                acc[m][j] = 0.0f;
                wsum[m][j] = 0.0f;
                if constexpr (HISTORY) {
                    lvc[m][j] = __fdiv_rn(kLog2e, Vp[(oy0 + R + m) * TS + ox0 + R + j]);
                    nkl[m][j] = -kd * lvc[m][j];
                }
            }
    }

    /* All seven dx of one dy. The shifted rows of this dy, every column any
     * dx reads, are one register block: rows oy0 + R - 1 + dy .. + M + 1,
     * columns ox0 .. ox0 + BW + 2S + 1 (ox0 is even and R - 1 = S, so every
     * float2 load is aligned), read once from shared memory for seven dx. */
    CRAW_DEV void step_dy(const float *Tp, const float *Vp, int ox0, int oy0, int dy)
    {
        constexpr int WC = BW + 2 + 2 * S;
        static_assert(R - 1 == S, "window origin");
        float win[M + 2][WC];
#pragma unroll
        for (int r = 0; r < M + 2; r++) {
            const float *row = Tp + (oy0 + R - 1 + dy + r) * TS + ox0;
#pragma unroll
            for (int c = 0; c < WC; c += 2) {
                float2 t = *reinterpret_cast<const float2 *>(row + c);
                win[r][c] = t.x;
                win[r][c + 1] = t.y;
            }
        }
        /* History: the variance of the shifted centres, columns
         * ox0 + 1 .. ox0 + BW + 2S (loaded from ox0 in pairs). */
        float vq[HISTORY ? M : 1][HISTORY ? BW + 2 * S + 2 : 1];
        if constexpr (HISTORY) {
#pragma unroll
            for (int m = 0; m < M; m++) {
                const float *row = Vp + (oy0 + R + dy + m) * TS + ox0;
#pragma unroll
                for (int c = 0; c < BW + 2 * S + 2; c += 2) {
                    float2 t = *reinterpret_cast<const float2 *>(row + c);
                    vq[m][c] = t.x;
                    vq[m][c + 1] = t.y;
                }
            }
        }
#pragma unroll
        for (int dx = -S; dx <= S; dx++) {
            float hs[M + 2][BW];
#pragma unroll
            for (int r = 0; r < M + 2; r++) {
                float e[BW + 2];
#pragma unroll
                for (int c = 0; c < BW + 2; c++) {
                    float d = own[r][c] - win[r][c + dx + S];
                    e[c] = d * d;
                }
                /* Row sums of three, the middle pair shared by two columns. */
#pragma unroll
                for (int j = 0; j < BW; j += 2) {
                    float mid = e[j + 1] + e[j + 2];
                    hs[r][j] = e[j] + mid;
                    hs[r][j + 1] = mid + e[j + 3];
                }
            }
#pragma unroll
            for (int m = 0; m < M; m += 2) {
#pragma unroll
                for (int j = 0; j < BW; j++) {
                    /* Column sums of three, the middle pair shared by two rows. */
                    float mid = hs[m + 1][j] + hs[m + 2][j];
                    float d2a = hs[m][j] + mid, d2b = mid + hs[m + 3][j];
                    float wa, wb;
                    if constexpr (HISTORY) {
                        wa = craw_ex2(fminf(fmaf(d2a, nkl[m][j], fmaf(vq[m][j + 1 + dx + S], lvc[m][j], kLog2e)), 0.0f));
                        wb = craw_ex2(fminf(fmaf(d2b, nkl[m + 1][j],
                                                 fmaf(vq[m + 1][j + 1 + dx + S], lvc[m + 1][j], kLog2e)), 0.0f));
                    } else {
                        wa = craw_ex2(fminf(fmaf(d2a, c1, c0), 0.0f));
                        wb = craw_ex2(fminf(fmaf(d2b, c1, c0), 0.0f));
                    }
                    wsum[m][j] += wa;
                    wsum[m + 1][j] += wb;
                    if constexpr (CENTRE) {
                        /* Centred on the sample's own value, so that the
                         * sum's rounding scales with the spread of the
                         * values around it rather than with their level. */
                        acc[m][j] = fmaf(wa, win[m + 1][j + 1 + dx + S] - own[m + 1][j + 1], acc[m][j]);
                        acc[m + 1][j] = fmaf(wb, win[m + 2][j + 1 + dx + S] - own[m + 2][j + 1], acc[m + 1][j]);
                    } else {
                        acc[m][j] = fmaf(wa, win[m + 1][j + 1 + dx + S], acc[m][j]);
                        acc[m + 1][j] = fmaf(wb, win[m + 2][j + 1 + dx + S], acc[m + 1][j]);
                    }
                }
            }
        }
    }
};

/* The search of a thread's 2 columns x M rows with the two columns in one
 * packed register: squared differences, the column sums of the patch, the
 * weight's affine steps, the weight sum and the weighted sum are f32x2
 * instructions; the row sums (which mix the columns), the clamp and the
 * exp2 stay scalar. `Tp` is the tile, `To` the same tile shifted left by
 * one sample; with a history `Vp` / `Vo` are the variance and its shifted
 * copy. Same arithmetic as Search (without fused multiply-adds in the
 * squared differences). */
template <int M, int R, int TS, bool HISTORY, bool CENTRE>
struct SearchX2 {
    static_assert(M % 2 == 0, "pairs of rows");
    static_assert(R - 1 == S, "window origin");
    f2x own[M + 2][2];            /* columns (0,1), (2,3) of the patch block */
    f2x acc[M], wsum[M];
    f2x nkl[HISTORY ? M : 1], lvc[HISTORY ? M : 1];
    f2x c1, c0;

    /* The centres of the two samples of patch-block row r (columns 1 and
     * 2) with CENTRE: the aligned pair of columns 0 and 1, each sample's
     * left neighbour. Any centre leaves the exact sum unchanged; a
     * neighbour's value lies as close to the window's values as the
     * sample's own, up to the noise, and needs no packing. */
    CRAW_DEV f2x centre(int r) const
    {
        return own[r][0];
    }

    CRAW_DEV void init(const float *To, const float *Vp, int ox0, int oy0, float inv_h2)
    {
        /* Patch block columns ox0 + S .. ox0 + S + 3: odd start, so they
         * are aligned pairs of the shifted copy at ox0 + S - 1. */
#pragma unroll
        for (int r = 0; r < M + 2; r++) {
            const float *row = To + (oy0 + R - 1 + r) * TS + ox0 + S - 1;
            own[r][0] = f2_ld(row);
            own[r][1] = f2_ld(row + 2);
        }
        const float kd = (1.0f / 9.0f) * inv_h2;
        c1 = f2_pack(-kLog2e * kd, -kLog2e * kd);
        /* With a history the constant term is log2(e) (Search's expansion). */
        c0 = HISTORY ? f2_pack(kLog2e, kLog2e) : f2_pack(2.0f * kLog2e, 2.0f * kLog2e);
#pragma unroll
        for (int m = 0; m < M; m++) {
            acc[m] = wsum[m] = f2_pack(0.0f, 0.0f);
            if constexpr (HISTORY) {
                /* The centres' variance: columns ox0 + R, + R + 1 (aligned). */
                const f2x vc = f2_ld(Vp + (oy0 + R + m) * TS + ox0 + R);
                const float l0 = __fdiv_rn(kLog2e, f2_lo(vc)), l1 = __fdiv_rn(kLog2e, f2_hi(vc));
                lvc[m] = f2_pack(l0, l1);
                nkl[m] = f2_pack(-kd * l0, -kd * l1);
            }
        }
    }

    CRAW_DEV void step_dy(const float *Tp, const float *To, const float *Vp, const float *Vo,
                          int ox0, int oy0, int dy)
    {
        /* The shifted rows of this dy: columns ox0 .. ox0 + 9 as aligned
         * pairs (even starts) and odd pairs (from the shifted copy). */
        f2x ev[M + 2][5], od[M + 2][4];
#pragma unroll
        for (int r = 0; r < M + 2; r++) {
            const int o = (oy0 + R - 1 + dy + r) * TS + ox0;
#pragma unroll
            for (int k = 0; k < 5; k++)
                ev[r][k] = f2_ld(Tp + o + 2 * k);
#pragma unroll
            for (int k = 0; k < 4; k++)
                od[r][k] = f2_ld(To + o + 2 * k);
        }
#pragma unroll
        for (int o = 0; o <= 2 * S; o++) {
            /* Patch-block columns c = 0..3 meet window columns c + o. */
            f2x h[M + 2];
#pragma unroll
            for (int r = 0; r < M + 2; r++) {
                const f2x w0 = (o & 1) ? od[r][o >> 1] : ev[r][o >> 1];
                const f2x w1 = (o & 1) ? od[r][(o >> 1) + 1] : ev[r][(o >> 1) + 1];
                const f2x d0 = f2_sub(own[r][0], w0), d1 = f2_sub(own[r][1], w1);
                const f2x e0 = f2_mul(d0, d0), e1 = f2_mul(d1, d1);
                /* Row sums of three, the middle pair shared. */
                const float mid = f2_hi(e0) + f2_lo(e1);
                h[r] = f2_pack(f2_lo(e0) + mid, mid + f2_hi(e1));
            }
#pragma unroll
            for (int m = 0; m < M; m += 2) {
                /* Column sums of three, the middle pair shared by two rows. */
                const f2x mid = f2_add(h[m + 1], h[m + 2]);
                const f2x d2a = f2_add(h[m], mid), d2b = f2_add(mid, h[m + 3]);
                f2x xa, xb;
                if constexpr (HISTORY) {
                    /* The shifted centres' variance, window columns 1 + o, 2 + o. */
                    const int vcol = (o & 1) ? ox0 + 1 + o : ox0 + o;
                    const float *vsrc = (o & 1) ? Vp : Vo;
                    const f2x vqa = f2_ld(vsrc + (oy0 + R + dy + m) * TS + vcol);
                    const f2x vqb = f2_ld(vsrc + (oy0 + R + dy + m + 1) * TS + vcol);
                    xa = f2_fma(d2a, nkl[m], f2_fma(vqa, lvc[m], c0));
                    xb = f2_fma(d2b, nkl[m + 1], f2_fma(vqb, lvc[m + 1], c0));
                } else {
                    xa = f2_fma(d2a, c1, c0);
                    xb = f2_fma(d2b, c1, c0);
                }
                const f2x wa = f2_pack(craw_ex2(fminf(f2_lo(xa), 0.0f)), craw_ex2(fminf(f2_hi(xa), 0.0f)));
                const f2x wb = f2_pack(craw_ex2(fminf(f2_lo(xb), 0.0f)), craw_ex2(fminf(f2_hi(xb), 0.0f)));
                /* The shifted centres: window columns 1 + o, 2 + o. */
                const f2x qa = (o & 1) ? ev[m + 1][(o + 1) >> 1] : od[m + 1][o >> 1];
                const f2x qb = (o & 1) ? ev[m + 2][(o + 1) >> 1] : od[m + 2][o >> 1];
                wsum[m] = f2_add(wsum[m], wa);
                wsum[m + 1] = f2_add(wsum[m + 1], wb);
                if constexpr (CENTRE) {
                    acc[m] = f2_fma(wa, f2_sub(qa, centre(m + 1)), acc[m]);
                    acc[m + 1] = f2_fma(wb, f2_sub(qb, centre(m + 2)), acc[m + 1]);
                } else {
                    acc[m] = f2_fma(wa, qa, acc[m]);
                    acc[m + 1] = f2_fma(wb, qb, acc[m + 1]);
                }
            }
        }
    }
};

/* One tile (tile column bx, tile row by) of all four planes; the whole
 * CTA takes part. `smem` holds Cfg::smem_floats floats. MARK (spatial
 * only): `rd` is the marking of samples whose code lies near a rounding
 * boundary (CRAWKRound), and the weighted sums are centred, which makes
 * their float error about 3x smaller at a boundary and the marked band
 * narrower, for about 6 % more time in the search. */
template <int BW, int M, int WP, bool SPATIAL, bool TEMPORAL, bool HISTORY, bool X2 = false, bool STAGED = true,
          bool MARK = false, bool TMA = false>
CRAW_DEV void denoise_tile(const CRAWKDenoise &k, const CRAWKDenoiseIO &io, int bx, int by, float *smem,
                           const CRAWKRound *rd = nullptr, const CUtensorMap *tmap = nullptr,
                           uint32_t *err = nullptr)
{
    using C = Cfg<BW, M, WP, SPATIAL, TEMPORAL, HISTORY, X2, STAGED, TMA>;
    static_assert(!C::PACKED || BW == 2, "the packed search pairs a thread's two columns");
    constexpr int R = C::R, OX = C::OX, OY = C::OY, TX = C::TX, TY = C::TY, TS = C::TS;
    constexpr int NT = C::NT;
    float *T = smem;                                 /* 4 planes of TN */
    float *V = smem + 4 * C::TN;                     /* history: variance left */
    float *TC = smem + 8 * C::TN;                    /* history: this frame, apron R+1 */
    float *TPv = TC + 4 * C::EN;                     /* history: last frame, apron R+1 */

    const int tx0 = bx * OX, ty0 = by * OY;
    const int tid = threadIdx.x;
    static_assert(!MARK || (SPATIAL && !TEMPORAL && BW == 2), "marks: spatial, a half-warp a word");
    if (MARK && rd->count2 && bx == 0 && by == 0 && tid == 0) {
        rd->count2[0] = 0;      /* this frame's list of undecided samples starts empty */
        rd->count2[1] = 0;      /* and so does the rounding's work counter */
        rd->count2[2] = 0;      /* and its list of marked samples */
    }

    /* ---- fill: the stabilised tile, temporally averaged when there is a
     * history (reference lib/ref/ref_denoise.c:244-296). */
    uint32_t *raw32 = reinterpret_cast<uint32_t *>(smem + C::RW_OFF);
    if constexpr (!HISTORY) {
        /* TMA: a tile whose apron lies inside the frame (plane columns
         * tx0 - R .. tx0 - R + TX, rows ty0 - R .. ty0 - R + TY) brings its
         * mosaic region in with one tile copy; the others, at the frame's
         * edges, mirror their plain loads. */
        const uint32_t *box = nullptr;
        if constexpr (TMA) {
            static_assert(SPATIAL && !TEMPORAL, "the spatial fill");
            static_assert((2 * OX) % 8 == 0 && (2 * R) % 8 == 0 && (C::BOX_W * 2) % 16 == 0,
                          "every box starts and ends on a 16-byte boundary");
            __shared__ __align__(8) uint64_t tma_bar;
            if (tx0 >= R && ty0 >= R && tx0 - R + TX <= k.pw && ty0 - R + TY <= k.ph) {
                box = reinterpret_cast<const uint32_t *>(((uintptr_t)(smem + C::BOX_OFF) + 127) &
                                                         ~(uintptr_t)127);
                craw_tma::bar_init(&tma_bar);
                if (tid == 0)
                    craw_tma::load_2d((void *)box, tmap, 2 * (tx0 - R), 2 * (ty0 - R), &tma_bar, C::BOX_BYTES);
                if (!__syncthreads_and(craw_tma::wait(&tma_bar, 0))) {
                    /* Never expected: record it, give the copy one more
                     * bound to land before the CTA leaves, and skip the
                     * tile. */
                    if (tid == 0 && err)
                        atomicOr(err, CRAW_K_ERR_TMA_WAIT);
                    (void)craw_tma::wait(&tma_bar, 0);
                    return;
                }
            }
        }
        for (int i = tid; i < TX * TY; i += NT) {
            int r = i / TX, c = i % TX;
            uint32_t q[4], qa, qb;
            if (TMA && box) {
                /* Plane row r is box rows 2r, 2r + 1; quad column c is the
                 * box's 32-bit word c of each. */
                qa = box[(2 * r) * TX + c];
                qb = box[(2 * r + 1) * TX + c];
                q[0] = qa & 0xffffu; q[1] = qa >> 16; q[2] = qb & 0xffffu; q[3] = qb >> 16;
            } else {
                int qy = craw_mirror(ty0 - R + r, k.ph), qx = craw_mirror(tx0 - R + c, k.pw);
                load_quad_u16(k, io, qx, qy, q, qa, qb, err);
            }
            if constexpr (STAGED)
                keep_raw<OX, OY>(raw32, r - R, c - R, qa, qb);
#pragma unroll
            for (int pl = 0; pl < 4; pl++) {
                const float t = gat_fwd(k, level(k, q[pl], pl));
                T[pl * C::TN + r * TS + c] = t;
                if constexpr (C::PACKED)
                    if (c > 0)
                        smem[C::TO_OFF + pl * C::TN + r * TS + c - 1] = t;
            }
        }
    } else {
        for (int i = tid; i < C::EN; i += NT) {
            int r = i / C::EX, c = i % C::EX;
            int qy = craw_mirror(ty0 - R - 1 + r, k.ph), qx = craw_mirror(tx0 - R - 1 + c, k.pw);
            uint32_t q[4], qa, qb;
            float lp[4];
            load_quad_u16(k, io, qx, qy, q, qa, qb, err);
            if constexpr (STAGED)
                keep_raw<OX, OY>(raw32, r - R - 1, c - R - 1, qa, qb);
            load_quad_f32(k, io.lvl_prev, io.lvl_pitch, qx, qy, lp, err);
#pragma unroll
            for (int pl = 0; pl < 4; pl++) {
                TC[pl * C::EN + i] = gat_fwd(k, level(k, q[pl], pl));
                TPv[pl * C::EN + i] = gat_fwd(k, lp[pl]);
            }
        }
        __syncthreads();
        /* A thread takes KR rows of one column, so that the 3x3 sums of
         * squared differences share their row sums: KR + 2 row sums of
         * three, then KR column sums of three (the same nine terms as the
         * reference's row-major sum, added in another order). */
        constexpr int KR = 4;
        static_assert(TY % KR == 0, "whole runs of rows");
        for (int i = tid; i < TX * (TY / KR); i += NT) {
            const int c = i % TX, r0 = (i / TX) * KR;
            const int qx = craw_mirror(tx0 - R + c, k.pw);
            uint32_t sv[KR][4];
#pragma unroll
            for (int j = 0; j < KR; j++) {
                const int qy = craw_mirror(ty0 - R + r0 + j, k.ph);
                const char *vr = (const char *)io.var_prev + (size_t)(2 * qy) * io.var_pitch;
                uint16_t v0 = 0, v1 = 0;
                if (craw_in_bounds(qx >= 0 && qx < k.pw && qy >= 0 && qy < k.ph, err)) {
                    v0 = __ldg(reinterpret_cast<const uint16_t *>(vr) + qx);
                    v1 = __ldg(reinterpret_cast<const uint16_t *>(vr + io.var_pitch) + qx);
                }
                sv[j][0] = v0 & 0xffu;
                sv[j][1] = (uint32_t)v0 >> 8;
                sv[j][2] = v1 & 0xffu;
                sv[j][3] = (uint32_t)v1 >> 8;
            }
#pragma unroll
            for (int pl = 0; pl < 4; pl++) {
                const float *cp = TC + pl * C::EN, *pp = TPv + pl * C::EN;
                /* Ring rows r0 .. r0 + KR + 1, columns c .. c + 2: the 3x3
                 * windows of tile rows r0 .. r0 + KR - 1 at column c. */
                float hs[KR + 2];
#pragma unroll
                for (int j = 0; j < KR + 2; j++) {
                    const int e = (r0 + j) * C::EX + c;
                    const float a0 = pp[e] - cp[e], a1 = pp[e + 1] - cp[e + 1], a2 = pp[e + 2] - cp[e + 2];
                    hs[j] = __fadd_rn(__fadd_rn(__fmul_rn(a0, a0), __fmul_rn(a1, a1)), __fmul_rn(a2, a2));
                }
#pragma unroll
                for (int j = 0; j < KR; j++) {
                    const int r = r0 + j, e0 = (r + 1) * C::EX + c + 1;
                    const float d2 = __fadd_rn(__fadd_rn(hs[j], hs[j + 1]), hs[j + 2]);
                    float x = d2 * (1.0f / 9.0f) * k.t_inv_h2 - 2.0f;
                    float a = k.t_alpha * expf(-fmaxf(x, 0.0f));
                    float sp = (float)sv[j][pl] * (1.0f / 255.0f);
                    float vv = __fadd_rn(__fmul_rn(1.0f - a, 1.0f - a), __fmul_rn(a * a, sp * sp));
                    const float t = __fadd_rn(__fmul_rn(cp[e0], 1.0f - a), __fmul_rn(pp[e0], a));
                    T[pl * C::TN + r * TS + c] = t;
                    V[pl * C::TN + r * TS + c] = fmaxf(vv, kVarMin);
                    if constexpr (C::PACKED)
                        if (c > 0) {
                            smem[C::TO_OFF + pl * C::TN + r * TS + c - 1] = t;
                            smem[C::VO_OFF + pl * C::TN + r * TS + c - 1] = fmaxf(vv, kVarMin);
                        }
                }
            }
        }
    }
    __syncthreads();

    /* ---- the search */
    const int warp = tid >> 5, lane = tid & 31;
    const int pl = warp / WP, band = warp % WP;
    const int ox0 = (lane & 15) * BW, oy0 = ((band << 1) | (lane >> 4)) * M;
    const float *Tp = T + pl * C::TN;
    float res[M][BW];

    if constexpr (C::PACKED) {
        const float *To = smem + C::TO_OFF + pl * C::TN;
        const float *Vp = V + pl * C::TN, *Vo = smem + C::VO_OFF + pl * C::TN;
        SearchX2<M, R, TS, HISTORY, MARK> st;
        st.init(To, Vp, ox0, oy0, k.inv_h2);
#pragma unroll 1
        for (int dy = -S; dy <= S; dy++)
            st.step_dy(Tp, To, Vp, Vo, ox0, oy0, dy);
#pragma unroll
        for (int m = 0; m < M; m++) {
            res[m][0] = __fdiv_rn(f2_lo(st.acc[m]), f2_lo(st.wsum[m]));
            res[m][1] = __fdiv_rn(f2_hi(st.acc[m]), f2_hi(st.wsum[m]));
            if constexpr (MARK) {
                const f2x c = st.centre(m + 1);
                res[m][0] += f2_lo(c);
                res[m][1] += f2_hi(c);
            }
        }
    } else if constexpr (SPATIAL) {
        const float *Vp = V + pl * C::TN;
        Search<BW, M, R, TS, HISTORY, MARK> st;
        st.init(Tp, Vp, ox0, oy0, k.inv_h2);
        /* dy is a runtime loop and only the seven dx of one dy are
         * unrolled, so that the loop body stays in the instruction cache. */
#pragma unroll 1
        for (int dy = -S; dy <= S; dy++)
            st.step_dy(Tp, Vp, ox0, oy0, dy);
#pragma unroll
        for (int m = 0; m < M; m++)
#pragma unroll
            for (int j = 0; j < BW; j++)
                res[m][j] = MARK ? st.own[m + 1][j + 1] + __fdiv_rn(st.acc[m][j], st.wsum[m][j])
                                 : __fdiv_rn(st.acc[m][j], st.wsum[m][j]);
    }

    /* ---- outputs: the next state, and the denoised mosaic in its raw
     * encoding after the highlight guard (reference
     * lib/ref/ref_denoise.c:285-324). */
    const int px = pl & 1, py = pl >> 1;
    /* This warp's plane constants, selected once (indexing the parameter
     * arrays with the warp's plane would copy them to local memory). */
    const float blk = pick4(k.black, pl), irng = pick4(k.inv_range, pl), rng = pick4(k.range, pl);
    /* The marks need a half-warp's 16 lanes x BW columns to be one word. */
    const bool mark = MARK && rd->flags;
#pragma unroll
    for (int m = 0; m < M; m++) {
        const int qy = ty0 + oy0 + m;
        bool near[BW];
#pragma unroll
        for (int j = 0; j < BW; j++) {
            const int qx = tx0 + ox0 + j;
            near[j] = false;
            if (qy >= k.ph || qx >= k.pw || !craw_in_bounds(qx >= 0 && qy >= 0, err))
                continue;
            const int my = 2 * qy + py, mx = 2 * qx + px;
            const float tc = Tp[(oy0 + R + m) * TS + ox0 + R + j];
            if constexpr (TEMPORAL) {
                float *lr = (float *)((char *)io.lvl_next + (size_t)my * io.lvl_pitch);
                uint8_t *vr = io.var_next + (size_t)my * io.var_pitch;
                lr[mx] = gat_inv(k, tc);
                if constexpr (HISTORY) {
                    float vv = V[pl * C::TN + (oy0 + R + m) * TS + ox0 + R + j];
                    vr[mx] = (uint8_t)rintf(sqrtf(fminf(fmaxf(vv, 0.0f), 1.0f)) * 255.0f);
                } else {
                    vr[mx] = 255;
                }
            }
            float u = gat_inv(k, SPATIAL ? res[m][j] : tc);
            /* The sample's raw value (kept by the fill when STAGED), and in
             * its place the output. */
            uint16_t *cell = reinterpret_cast<uint16_t *>(raw32) + (2 * (oy0 + m) + py) * C::RW_W +
                             2 * (ox0 + j) + px;
            uint16_t raw0;
            if constexpr (STAGED)
                raw0 = *cell;
            else
                raw0 = __ldg((const uint16_t *)((const char *)io.src + (size_t)my * io.src_pitch) + mx);
            float u0 = ((float)raw0 * (1.0f / 65535.0f) - blk) * irng;
            float gr = fminf(fmaxf((u0 - k.guard_lo) * k.guard_inv, 0.0f), 1.0f);
            u = u + (u0 - u) * gr;
            float ro = fminf(fmaxf(blk + u * rng, 0.0f), 1.0f);
            const float xv = ro * 65535.0f;
            const uint16_t code = (uint16_t)rintf(xv);
            if (mark) {
                /* Within the float error of a rounding boundary: the exact
                 * rounding decides this code. */
                const float tm = SPATIAL ? res[m][j] : tc;
                near[j] = fabsf(xv - rintf(xv)) > 0.5f - fmaf(tm * tm, rd->c2, rd->c0);
            }
            if constexpr (STAGED)
                *cell = code;
            else
                ((uint16_t *)((char *)io.dst + (size_t)my * io.dst_pitch))[mx] = code;
        }
        if constexpr (BW == 2) {
            if (mark) {
                /* A half-warp holds one plane row's 32 columns tx0 .. tx0 + 31:
                 * lane l's two columns are bits l and 16 + l of its word. */
                const uint32_t b0 = __ballot_sync(0xffffffffu, near[0]);
                const uint32_t b1 = __ballot_sync(0xffffffffu, near[1]);
                const uint32_t sh = lane & 16;
                const uint32_t word = ((b0 >> sh) & 0xffffu) | (((b1 >> sh) & 0xffffu) << 16);
                const size_t wi = ((size_t)pl * k.ph + qy) * CRAW_K_ROUND_WW(k.pw) + (tx0 >> 5);
                if ((lane & 15) == 0 && qy < k.ph &&
                    craw_in_bounds(wi < (size_t)CRAW_K_ROUND_WORDS(k.pw, k.ph), err))
                    rd->flags[wi] = word;
            }
        }
    }
    if constexpr (!STAGED)
        return;

    /* The tile's mosaic region out, 16 bytes a thread (element by element
     * at the frame's right edge, or if the rows are not 16-byte aligned). */
    __syncthreads();
    constexpr int CH = C::RW_W / 8;
    const int mx0 = 2 * tx0, my0 = 2 * ty0, W = 2 * k.pw, H = 2 * k.ph;
    const bool a16 = !(((uintptr_t)io.dst | io.dst_pitch) & 15);
    const uint16_t *raw16 = reinterpret_cast<const uint16_t *>(raw32);
    for (int i = tid; i < C::RW_H * CH; i += NT) {
        const int yy = i / CH, xx = (i % CH) * 8, my = my0 + yy, mx = mx0 + xx;
        if (my >= H || mx >= W || !craw_in_bounds(my >= 0 && mx >= 0 && yy < C::RW_H, err))
            continue;
        uint16_t *dr = (uint16_t *)((char *)io.dst + (size_t)my * io.dst_pitch) + mx;
        if (a16 && mx + 8 <= W) {
            *reinterpret_cast<uint4 *>(dr) = reinterpret_cast<const uint4 *>(raw32)[i];
        } else {
            for (int e = 0; e < 8 && mx + e < W; e++)
                dr[e] = raw16[yy * C::RW_W + xx + e];
        }
    }
}

} // namespace craw_dn
