/*
 * Exact rounding of the denoised mosaic.
 *
 * The denoise ends by re-encoding each filtered sample as a 16-bit code,
 * rint(clamp(black + u * range) * 65535) (reference
 * lib/ref/ref_denoise.c:318-323). The float evaluation of the filter is
 * within about 1e-6 relative of the exact value, so wherever the exact
 * code position x lies within that error of a half-integer, float and
 * double evaluations round to neighbouring codes; one code is up to 1e-2
 * of a dark pixel, far beyond a 1e-3 bound on the developed output.
 *
 * The denoise kernel marks the samples whose float x lies within a band
 * around a boundary (CRAWKRound). Two kernels here settle them:
 *
 * k_round_decide  takes the marked samples off the bit map (a warp queues
 *   the set bits of 32 KW words at a time, GA lanes a sample) and evaluates
 *   each again in float, GA lanes a sample, in a form whose error it can
 *   bound: every stabilised value of the 9x9 window as its difference from
 *   the value m_c of the code the float path chose, computed without
 *   cancellation from the exact integer difference of the codes,
 *     t_k - m_c = (t_k^2 - m_c^2) / (t_k + m_c),
 *     t_k^2 - m_c^2 = 4 (r_k - code) / (65535 range a),
 *   the weights from these differences, and the code offset
 *     y = x - code = (65535 range a / 4) m' (2 m_c + m'),  m' = m - m_c,
 *   with a bound on the error of y from the unit roundoff of each step.
 *   When y +- bound rounds the same way, that is the code a double
 *   evaluation gives; otherwise (and for every sample near the white
 *   guard, at or below black, or at the ends of the code range) the sample
 *   goes to a list;
 * k_round_exact  evaluates each listed sample in double-float arithmetic
 *   (dfloat.cuh, about 1e-13 relative; the double evaluation's own error
 *   is about 1e-15), G lanes a sample: the window stabilised
 *   (ref_denoise.c:30-58), the 49 patch distances and weights
 *   exp(-max(d2/(9 h^2) - 2, 0)) (ref_denoise.c:109-154), the weighted
 *   mean, the inverse transform, the highlight guard and the re-encoding
 *   (ref_denoise.c:298-324).
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "dfloat.cuh"

namespace {

constexpr int NT = 128;                /* threads per CTA */
constexpr int WIN = 9;                 /* search 3 + patch 1, both sides */
constexpr int KW = 1;                  /* bit-map words a lane scans a step */
constexpr int GA = 4;                  /* lanes of the decision stage a sample */
constexpr int G = 16;                  /* lanes of the exact stage a sample */
constexpr int GPL = (WIN * WIN + GA - 1) / GA;   /* window samples a decision lane loads */
constexpr int XPL = (WIN * WIN + G - 1) / G;     /* and an exact-stage lane */
constexpr int DECIDE_CTAS = 7;         /* resident decision CTAs an SM (72 registers) */
constexpr float U = 0x1p-24f;          /* float unit roundoff */

/* ------------------------------------------------------------ helpers */

CRAW_DEV const uint16_t *row16(const void *base, size_t pitch, int y)
{
    return (const uint16_t *)((const char *)base + (size_t)y * pitch);
}

CRAW_DEV void record_change(uint32_t *stats, float t, float x, float dist, int pl)
{
    atomicAdd(&stats[1], 1u);
    const uint32_t r = atomicAdd(&stats[2], 1u);
    if (r < CRAW_K_ROUND_RECORDS) {
        float4 rec;
        rec.x = t;
        rec.y = x;
        rec.z = dist;
        rec.w = (float)pl;
        reinterpret_cast<float4 *>(stats + 4)[r] = rec;
    }
}

/* ------------------------------------------- the float decision stage */

/* The stabilised value of a code above black, sqrt(q raw + beta), the
 * root's argument formed in double-float (it cancels near black) and
 * rounded once: within 1 ulp. */
CRAW_DEV float stab(const CRAWKDenoiseExact &e, int pl, uint32_t raw)
{
    const float r = (float)raw;
    const float p = e.qq[pl][0] * r;
    float lo = fmaf(e.qq[pl][0], r, -p);
    lo = fmaf(e.qq[pl][1], r, lo);
    const dfl sm = df_two_sum(p, e.beta[pl][0]);
    return sqrtf(sm.hi + (sm.lo + (lo + e.beta[pl][1])));
}

/* Settles sample (pl, qx, qy) with the GA lanes of a group (g = 0 .. GA-1,
 * D the group's 81 floats of shared memory): true on every lane of the
 * group when the code in io.dst is now the double evaluation's. Every
 * lane of the warp calls it (valid false where there is no sample), so
 * that the warp's synchronisations match.
 *
 * Error bound (u = 2^-24): each window value is the stabilised value t_k
 * less m_c, d_k = (r_k - code) q / (t_k + m_c), within 5u of itself (q
 * and the product 1u; t_k and m_c within 1u, so the denominator 1.5u; the
 * correctly rounded reciprocal and its product 1u). A patch distance's
 * error is then at most 10u sum |e| (|a| + |b|) + 12u d2 (e = a - b per
 * tap: its own rounding, the square's and the sum's), and
 * sum |e| (|a| + |b|) <= sqrt(2 d2 (P_c + P_i)) (Cauchy-Schwarz; P: a
 * patch's sum of d^2); a weight's relative error is 1/(9h^2) times that,
 * plus its argument's rounding (0.7u |log2 w|) and the exponential's (8u).
 * The weighted sum's rounding is bounded as it runs (u times the sum of
 * the partial sums' magnitudes); the weight sum's is at most 16u of it. */
CRAW_DEV bool decide(const CRAWKDenoise &k, const CRAWKDenoiseExact &e, const CRAWKDenoiseIO &io, int pl,
                     int qx, int qy, bool valid, int g, int lane, float *D, uint32_t *stats)
{
    const int px = pl & 1, py = pl >> 1;
    const int my = 2 * qy + py, mx = 2 * qx + px;
    bool ok = valid && e.decide;
    int code = 0;
    if (ok) {
        const uint32_t raw0 = row16(io.src, io.src_pitch, my)[mx];
        if (fmaf((float)raw0, e.k1[pl], -e.k0[pl]) >= k.guard_lo - 1e-3f)
            ok = false;                     /* the white guard blends: exact stage */
        code = row16(io.dst, io.dst_pitch, my)[mx];
        if (code <= (int)e.dark_code + 2 || code >= 65534)
            ok = false;                     /* near black (the linear branch) or the clamp */
    }
    const float mc = stab(e, pl, (uint32_t)code);
    const float q = e.q[pl];
    if (ok) {
        /* The lane's window samples, every GA-th: all loads issued before
         * any is used, so that their latencies overlap. */
        const bool inner = qy >= 4 && qy + 4 < k.ph && qx >= 4 && qx + 4 < k.pw;
        uint32_t raw[(GPL + 1) / 2];        /* two codes a register */
#pragma unroll
        for (int i = 0; i < GPL; i++) {
            const int s = g + i * GA;
            uint32_t r = 0u;
            if (s < WIN * WIN) {
                int yy = qy + s / WIN - 4, xx = qx + s % WIN - 4;
                if (!inner) {
                    yy = craw_mirror(yy, k.ph);
                    xx = craw_mirror(xx, k.pw);
                }
                r = __ldg(row16(io.src, io.src_pitch, 2 * yy + py) + 2 * xx + px);
            }
            raw[i >> 1] = (i & 1) ? raw[i >> 1] | (r << 16) : r;
        }
#pragma unroll
        for (int i = 0; i < GPL; i++) {
            const int s = g + i * GA;
            const uint32_t r = (raw[i >> 1] >> (16 * (i & 1))) & 0xffffu;
            if (s < WIN * WIN) {
                if (r <= e.dark_code)
                    ok = false;             /* a sample at or below black: exact stage */
                D[s] = (float)((int)r - code) * q * __frcp_rn(stab(e, pl, r) + mc);
            }
        }
    }
    /* The group goes on only if all its lanes may. */
    const uint32_t gmask = ((1u << GA) - 1u) << (lane & ~(GA - 1));
    ok = (__ballot_sync(0xffffffffu, ok) & gmask) == gmask;
    __syncwarp();

    float s = 0.0f, es = 0.0f, wt = 0.0f, a = 0.0f, b = 0.0f, r = 0.0f;
    if (ok) {
        float pc = 0.0f;
#pragma unroll
        for (int ky = -1; ky <= 1; ky++)
#pragma unroll
            for (int kx = -1; kx <= 1; kx++) {
                const float d = D[(4 + ky) * WIN + 4 + kx];
                pc = fmaf(d, d, pc);
            }
        for (int o = g; o < 49; o += GA) {
            const int dy = o / 7 - 3, dx = o % 7 - 3;
            float d2 = 0.0f, pi = 0.0f;
#pragma unroll
            for (int ky = -1; ky <= 1; ky++)
#pragma unroll
                for (int kx = -1; kx <= 1; kx++) {
                    const float bb = D[(4 + dy + ky) * WIN + 4 + dx + kx];
                    const float df = D[(4 + ky) * WIN + 4 + kx] - bb;
                    d2 = fmaf(df, df, d2);
                    pi = fmaf(bb, bb, pi);
                }
            const float xa = fmaf(d2, e.c1, e.c0);
            const float w = craw_ex2(fminf(xa, 0.0f));
            const float cs = sqrtf(2.0f * d2 * (pc + pi));
            const float rho = U * fmaf(e.kn, fmaf(10.0f, cs, 12.0f * d2), fmaf(0.7f, fabsf(xa), 8.0f));
            const float dc = D[(4 + dy) * WIN + 4 + dx];
            const float wr = w * rho;
            s = fmaf(w, dc, s);
            es += fabsf(s);
            wt += w;
            a = fmaf(w, fabsf(dc), a);
            b = fmaf(wr, fabsf(dc), b);
            r += wr;
        }
    }
#pragma unroll
    for (int m = 1; m < GA; m <<= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, m);
        es += __shfl_xor_sync(0xffffffffu, es, m) + fabsf(s);
        wt += __shfl_xor_sync(0xffffffffu, wt, m);
        a += __shfl_xor_sync(0xffffffffu, a, m);
        b += __shfl_xor_sync(0xffffffffu, b, m);
        r += __shfl_xor_sync(0xffffffffu, r, m);
    }
    __syncwarp();
    if (!ok)
        return false;
    const float mp = s / wt;
    const float em = (5.0f * U * a + U * es + b) / wt + fabsf(mp) * (16.0f * U + r / wt);
    const float k2 = e.k2[pl];
    const float y = k2 * mp * (2.0f * mc + mp);
    const float ey = k2 * (2.0f * mc + 2.0f * fabsf(mp)) * em + 10.0f * U * fabsf(y);
    const float n = rintf(y);
    const float dist = 0.5f - fabsf(y - n);
    if (!(dist > ey * 1.25f + 1e-7f))
        return false;
    if (n != 0.0f && g == 0) {
        const int nc = code + (int)n;
        ((uint16_t *)((char *)io.dst + (size_t)my * io.dst_pitch))[mx] = (uint16_t)nc;
        record_change(stats, mc + mp, (float)nc + (y - n), dist, pl);
    }
    return true;
}

/* Samples a warp's decision stage takes at once: one per group of GA lanes. */
constexpr int BATCH = 32 / GA;
/* A warp's queue of marked samples: one step's marks (32 KW words of 32
 * bits) on top of a partial batch. */
constexpr int QCAP = 32 * KW * 32 + BATCH;

/* Appends the marked samples of the 32 * KW bit-map words from `first` to
 * the warp's queue Q (which holds qn) as packed indices
 * (pl * ph + qy) * pw + qx, the list's form; returns the new length. */
CRAW_DEV int enqueue_marks(const uint32_t *flags, long long nwords, int ww, int pw, int ph, long long first,
                           int lane, uint32_t *Q, int qn)
{
    uint32_t w[KW];
    int cnt = 0;
#pragma unroll
    for (int j = 0; j < KW; j++) {
        const long long i = first + (long long)lane * KW + j;
        w[j] = i < nwords ? __ldg(flags + i) : 0u;
        cnt += __popc(w[j]);
    }
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o)
            incl += v;
    }
    const int tot = __shfl_sync(0xffffffffu, incl, 31);
    int at = qn + incl - cnt;
#pragma unroll
    for (int j = 0; j < KW; j++) {
        const long long wi = first + (long long)lane * KW + j;
        const uint32_t row = (uint32_t)(wi / ww), base = row * (uint32_t)pw + (uint32_t)(wi % ww) * 32u;
        for (uint32_t m = w[j]; m; m &= m - 1) {
            const int bit = __ffs(m) - 1;
            Q[at++] = base + (uint32_t)(bit < 16 ? 2 * bit : 2 * (bit - 16) + 1);
        }
    }
    __syncwarp();
    return qn + tot;
}

/* The marked samples as a list (rd.count2[2] counts them; entries past
 * `cap` are not written): each warp counts the marks of its own run of
 * bit-map steps, takes its place in the list with one atomic and writes
 * them in bit-map order, so that a batch's samples are neighbours. */
__global__ void __launch_bounds__(NT)
k_round_compact(const CRAWKRound rd, int pw, int ph, uint32_t *marked, uint32_t cap)
{
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (NT / 32);
    const long long wid = (long long)blockIdx.x * (NT / 32) + threadIdx.x / 32;
    const int ww = CRAW_K_ROUND_WW(pw);
    const long long nwords = (long long)CRAW_K_ROUND_WORDS(pw, ph);
    const long long steps = (nwords + 31) / 32, per = (steps + warps - 1) / warps;
    const long long s0 = wid * per, s1 = s0 + per < steps ? s0 + per : steps;
    int tot = 0;
    for (long long st = s0; st < s1; st++) {
        const long long i = st * 32 + lane;
        tot += __popc(i < nwords ? __ldg(rd.flags + i) : 0u);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        tot += __shfl_xor_sync(0xffffffffu, tot, o);
    if (tot == 0)
        return;
    uint32_t base = 0;
    if (lane == 0)
        base = atomicAdd(rd.count2 + 2, (uint32_t)tot);
    base = __shfl_sync(0xffffffffu, base, 0);
    for (long long st = s0; st < s1; st++) {
        const long long i = st * 32 + lane;
        const uint32_t w = i < nwords ? __ldg(rd.flags + i) : 0u;
        const int cnt = __popc(w);
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o)
                incl += v;
        }
        uint32_t at = base + (uint32_t)(incl - cnt);
        const uint32_t row = (uint32_t)(i / ww), first = row * (uint32_t)pw + (uint32_t)(i % ww) * 32u;
        for (uint32_t m = w; m; m &= m - 1) {
            const int bit = __ffs(m) - 1;
            if (at < cap)
                marked[at] = first + (uint32_t)(bit < 16 ? 2 * bit : 2 * (bit - 16) + 1);
            at++;
        }
        base += (uint32_t)__shfl_sync(0xffffffffu, incl, 31);
    }
}

/* Decides the samples of a batch (packed indices v, one per group of GA
 * lanes, `take` of them) and lists the undecided ones. */
CRAW_DEV void decide_batch(const CRAWKDenoise &k, const CRAWKDenoiseExact &e, const CRAWKDenoiseIO &io,
                           const CRAWKRound &rd, uint32_t v, int take, int g, int lane, float *D,
                           uint32_t *list, uint32_t list_cap, uint32_t *stats)
{
    const bool valid = lane / GA < take;
    const uint32_t qx = v % (uint32_t)k.pw, r = v / (uint32_t)k.pw;
    const int qy = (int)(r % (uint32_t)k.ph), pl = (int)(r / (uint32_t)k.ph);
    const bool done = decide(k, e, io, pl, (int)qx, qy, valid, g, lane, D, stats);
    /* The batch's undecided samples take their places in the list with
     * one atomic. */
    const bool put = valid && !done && g == 0;
    const uint32_t bal = __ballot_sync(0xffffffffu, put);
    if (!bal)
        return;
    uint32_t base = 0;
    if (lane == 0)
        base = atomicAdd(rd.count2, (uint32_t)__popc(bal));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (put) {
        const uint32_t slot = base + (uint32_t)__popc(bal & ((1u << lane) - 1u));
        if (slot < list_cap)
            list[slot] = v;
    }
}

/* The decision stage over the list of marked samples: a batch of BATCH
 * list entries a warp at a time, batches in turn over the grid's warps
 * (their costs hardly differ). If the list overflowed (more than
 * `marked_cap` marks), the warps walk the bit map instead: they take
 * steps of 32 KW words off a shared counter (the marks gather where the
 * image is bright, so fixed shares would leave a few warps with most of
 * the work) and queue each step's marked samples, so that every batch but
 * a warp's last fills all its groups. */
__global__ void __launch_bounds__(NT, DECIDE_CTAS)
k_round_decide(const CRAWKDenoise k, const CRAWKDenoiseExact e, const CRAWKDenoiseIO io, const CRAWKRound rd,
               const uint32_t *marked, uint32_t marked_cap, uint32_t *list, uint32_t list_cap,
               uint32_t *stats)
{
    __shared__ float Dw[NT / GA][WIN * WIN];
    __shared__ uint32_t Qw[NT / 32][QCAP];
    const int lane = threadIdx.x & 31, g = lane % GA;
    float *D = Dw[threadIdx.x / GA];
    const uint32_t nm = *(volatile const uint32_t *)(rd.count2 + 2);
    if (nm <= marked_cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0)
            atomicAdd(&stats[0], nm);
        const long long warps = (long long)gridDim.x * (NT / 32);
        const long long wid = (long long)blockIdx.x * (NT / 32) + threadIdx.x / 32;
        for (long long b = wid * BATCH; b < nm; b += warps * BATCH) {
            const int take = nm - b < BATCH ? (int)(nm - b) : BATCH;
            const uint32_t v = lane / GA < take ? __ldg(marked + b + lane / GA) : 0u;
            decide_batch(k, e, io, rd, v, take, g, lane, D, list, list_cap, stats);
        }
        return;
    }
    uint32_t *Q = Qw[threadIdx.x / 32];
    const int ww = CRAW_K_ROUND_WW(k.pw);
    const long long nwords = (long long)CRAW_K_ROUND_WORDS(k.pw, k.ph);
    int qn = 0;               /* the same on every lane, as is `more` */
    uint32_t taken = 0;
    bool more = true;
    while (more || qn > 0) {
        if (more) {
            uint32_t c = 0;
            if (lane == 0)
                c = atomicAdd(rd.count2 + 1, 1u);
            const long long first = (long long)__shfl_sync(0xffffffffu, c, 0) * 32 * KW;
            if (first >= nwords)
                more = false;
            else
                qn = enqueue_marks(rd.flags, nwords, ww, k.pw, k.ph, first, lane, Q, qn);
        }
        while (qn >= BATCH || (!more && qn > 0)) {
            const int take = qn < BATCH ? qn : BATCH;
            const uint32_t v = lane / GA < take ? Q[qn - take + lane / GA] : 0u;
            __syncwarp();   /* read before the next steps write over it */
            qn -= take;
            taken += (uint32_t)take;
            decide_batch(k, e, io, rd, v, take, g, lane, D, list, list_cap, stats);
        }
    }
    if (lane == 0 && taken)
        atomicAdd(&stats[0], taken);
}

/* ------------------------------------------------ the double-float stage */

CRAW_DEV dfl ld(const float v[2])
{
    return df_make(v[0], v[1]);
}

CRAW_DEV dfl shfl_df(dfl a, int m)
{
    return df_make(__shfl_xor_sync(0xffffffffu, a.hi, m), __shfl_xor_sync(0xffffffffu, a.lo, m));
}

/* The stabilised value of a raw code at quad site pl (reference
 * lib/ref/ref_denoise.c:30-40 after the normalisation of 268-270). */
CRAW_DEV dfl gat_fwd_x(const CRAWKDenoiseExact &e, uint32_t raw, int pl)
{
    const dfl r = df_mul_f(ld(e.inv65535), (float)raw);
    const dfl u = df_mul(df_sub(r, ld(e.black[pl])), ld(e.inv_range[pl]));
    if (u.hi >= 0.0f && !(u.hi == 0.0f && u.lo < 0.0f))
        return df_mul(ld(e.gat_fwd), df_sqrt(df_add(df_mul_f(u, e.gat_a), ld(e.gat_c))));
    return df_add(ld(e.gat_t0), df_mul(u, ld(e.gat_isc)));
}

/* The inverse (reference lib/ref/ref_denoise.c:44-58). */
CRAW_DEV dfl gat_inv_x(const CRAWKDenoiseExact &e, dfl t)
{
    if (df_cmp(t, ld(e.gat_t0)) >= 0)
        return df_sub(df_mul(df_mul(ld(e.gat_inv), t), t), ld(e.gat_off));
    return df_mul(df_sub(t, ld(e.gat_t0)), ld(e.gat_sc));
}

/* The double evaluation's code of sample (pl, qx, qy), written to io.dst,
 * by a group of G lanes (g = 0 .. G-1): each stabilises every G-th value
 * of the window into the group's scratch (Th/Tl, 81 double-floats) and
 * takes every G-th search offset; shuffles add the group's partial sums,
 * and lane 0 of the group finishes. `valid` false: the lanes only take
 * part in the synchronisation. */
CRAW_DEV void exact_sample(const CRAWKDenoiseExact &e, const CRAWKDenoiseIO &io, int pl, int qx, int qy,
                           bool valid, int g, float *Th, float *Tl, uint32_t *stats)
{
    const int px = pl & 1, py = pl >> 1;
    if (valid) {
        /* Every G-th window sample, the loads issued first. */
        uint32_t raw[XPL];
#pragma unroll
        for (int i = 0; i < XPL; i++) {
            const int s = g + i * G;
            raw[i] = 0u;
            if (s < WIN * WIN) {
                const int yy = craw_mirror(qy + s / WIN - 4, e.ph), xx = craw_mirror(qx + s % WIN - 4, e.pw);
                raw[i] = __ldg(row16(io.src, io.src_pitch, 2 * yy + py) + 2 * xx + px);
            }
        }
#pragma unroll
        for (int i = 0; i < XPL; i++) {
            const int s = g + i * G;
            if (s < WIN * WIN) {
                const dfl t = gat_fwd_x(e, raw[i], pl);
                Th[s] = t.hi;
                Tl[s] = t.lo;
            }
        }
    }
    __syncwarp();
    dfl acc = df_from(0.0f), wsum = df_from(0.0f);
    if (valid) {
        for (int o = g; o < 49; o += G) {
            const int dy = o / 7 - 3, dx = o % 7 - 3;
            dfl d2 = df_from(0.0f);
#pragma unroll
            for (int ky = -1; ky <= 1; ky++)
#pragma unroll
                for (int kx = -1; kx <= 1; kx++) {
                    const int a = (4 + ky) * WIN + 4 + kx, b = (4 + dy + ky) * WIN + 4 + dx + kx;
                    const dfl d = df_sub(df_make(Th[a], Tl[a]), df_make(Th[b], Tl[b]));
                    d2 = df_add_same(d2, df_sqr(d));
                }
            const dfl x = df_add_f(df_mul(d2, ld(e.k_nlm)), -2.0f);
            const bool pos = x.hi > 0.0f || (x.hi == 0.0f && x.lo > 0.0f);
            const dfl w = pos ? df_exp_neg(x) : df_from(1.0f);
            const int c = (4 + dy) * WIN + 4 + dx;
            acc = df_add(acc, df_mul(w, df_make(Th[c], Tl[c])));
            wsum = df_add_same(wsum, w);
        }
    }
#pragma unroll
    for (int m = 1; m < G; m <<= 1) {
        acc = df_add(acc, shfl_df(acc, m));
        wsum = df_add_same(wsum, shfl_df(wsum, m));
    }
    __syncwarp();
    if (!valid || g != 0)
        return;
    const dfl tm = df_div(acc, wsum);
    dfl u = gat_inv_x(e, tm);
    const int my = 2 * qy + py, mx = 2 * qx + px;
    const uint16_t raw0 = row16(io.src, io.src_pitch, my)[mx];
    const dfl u0 = df_mul(df_sub(df_mul_f(ld(e.inv65535), (float)raw0), ld(e.black[pl])), ld(e.inv_range[pl]));
    const dfl gr = df_clamp01(df_mul(df_sub(u0, ld(e.guard_lo)), ld(e.guard_inv)));
    u = df_add(u, df_mul(df_sub(u0, u), gr));
    const dfl ro = df_clamp01(df_add(ld(e.black[pl]), df_mul(u, ld(e.range[pl]))));
    const dfl xe = df_mul_f(ro, 65535.0f);
    const float n = df_rint(xe);
    const uint16_t code = (uint16_t)n;
    uint16_t *cell = (uint16_t *)((char *)io.dst + (size_t)my * io.dst_pitch) + mx;
    if (*cell != code) {
        *cell = code;
        record_change(stats, tm.hi, xe.hi, 0.5f - fabsf((xe.hi - n) + xe.lo), pl);
    }
}

/* One group of G lanes a listed sample. */
__global__ void __launch_bounds__(NT)
k_round_exact(const CRAWKDenoiseExact e, const CRAWKDenoiseIO io, const CRAWKRound rd, const uint32_t *list,
              uint32_t list_cap, uint32_t *stats)
{
    __shared__ float Th[NT / G][WIN * WIN], Tl[NT / G][WIN * WIN];
    const uint32_t listed = *rd.count2, n = min(listed, list_cap);
    if (blockIdx.x == 0 && threadIdx.x == 0)
        atomicAdd(&stats[3], listed);
    const int grp = threadIdx.x / G, g = threadIdx.x % G;
    const uint32_t groups = gridDim.x * (NT / G);
    /* Every lane runs the same number of rounds, so that the warp's
     * synchronisations match. */
    for (uint32_t base = blockIdx.x * (NT / G); base < n; base += groups) {
        const uint32_t i = base + grp;
        const bool valid = i < n;
        const uint32_t v = valid ? list[i] : 0u;
        const uint32_t qx = v % (uint32_t)e.pw, r = v / (uint32_t)e.pw;
        exact_sample(e, io, (int)(r / (uint32_t)e.ph), (int)qx, (int)(r % (uint32_t)e.ph), valid, g, Th[grp],
                     Tl[grp], stats);
    }
}

} // namespace

extern "C" int craw_k_denoise_round(const CRAWKDenoise *k, const CRAWKDenoiseExact *e, const CRAWKDenoiseIO *io,
                                    const CRAWKRound *rd, uint32_t *list, uint32_t *stats, int sm_count,
                                    cudaStream_t s)
{
    if (!k || !e || !io || !rd || !rd->flags || !rd->count2 || !list || !stats)
        return -22;
    if ((e->mode & (CRAW_K_DN_SPATIAL | CRAW_K_DN_TEMPORAL)) != CRAW_K_DN_SPATIAL)
        return -22;
    if (craw_launch_ready() < 0)
        return -5;
    const int sms = sm_count > 0 ? sm_count : 152;
    const size_t cap = CRAW_K_ROUND_LIST(k->pw, k->ph);
    uint32_t *marked = list, *undecided = list + cap;
    const long long steps = ((long long)CRAW_K_ROUND_WORDS(k->pw, k->ph) + 31) / 32;
    long long ctas_c = (steps / 4 + NT / 32 - 1) / (NT / 32);
    ctas_c = ctas_c < (long long)sms * 8 ? ctas_c : (long long)sms * 8;
    k_round_compact<<<(unsigned)(ctas_c > 0 ? ctas_c : 1), NT, 0, s>>>(*rd, k->pw, k->ph, marked, (uint32_t)cap);
    if (cudaGetLastError() != cudaSuccess)
        return -5;
    k_round_decide<<<(unsigned)sms * DECIDE_CTAS, NT, 0, s>>>(*k, *e, *io, *rd, marked, (uint32_t)cap, undecided,
                                                    (uint32_t)cap, stats);
    if (cudaGetLastError() != cudaSuccess)
        return -5;
    k_round_exact<<<(unsigned)sms * 8, NT, 0, s>>>(*e, *io, *rd, undecided, (uint32_t)cap, stats);
    return cudaGetLastError() == cudaSuccess ? 0 : -5;
}
