/*
 * Highlight reconstruction (reference lib/ref/ref_highlight.c, the stage
 * the reference's tools run by default): the clipped sites of a mosaic are
 * rebuilt from their unclipped neighbours and a smooth field of the
 * scene's colour, before the debayer.
 *
 *   k_hl_level0    one texel per 2x2 quads: weighted log chroma (ln R/G,
 *                  ln B/G) of the quads, and the weight, which falls to 0
 *                  within 3 quads of a clip (the quads' clip ramps and
 *                  their 7x7 max are made in shared memory on the way)
 *   k_hl_pull      each coarser level the sum of its four children, to 1x1
 *   k_hl_coarse    the levels of at most kCoarseTexels, pulled and pushed
 *                  in one CTA
 *   k_hl_push      back down: each texel blended from the coarser level's
 *                  bilinear colour toward its own mean by its weight
 *   k_hl_fill      per site: u * gain, lifted where a > 0 toward the level
 *                  its neighbours' channels and the field predict; fp16
 *
 * The mosaic is read twice and the fp16 mosaic written once; the field is
 * 1/16 size. Operation order follows the reference and this file is built
 * without multiply-add contraction (the oracle's -ffp-contract=off), so
 * the only differences are the device's logf/expf against the host's.
 */
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace {

constexpr float kULo = 0.92f, kUHi = 0.98f, kEps = 1e-4f, kLogMax = 2.0f, kWSat = 1.0f;
constexpr int kDilate = 3;

CRAW_DEV int site_chan(int s) { return s == 0 ? 0 : (s == 3 ? 2 : 1); }

/* smoothstep(kULo, kUHi, v); below kULo the quotient is <= 0 and clamps
 * to 0, which the early return gives without the division. */
CRAW_DEV float smooth(float v)
{
    if (v <= kULo)
        return 0.0f;
    float t = __fdiv_rn(v - kULo, kUHi - kULo);
    t = t < 0.0f ? 0.0f : (t > 1.0f ? 1.0f : t);
    return t * t * (3.0f - 2.0f * t);
}

CRAW_DEV float site_u(const CRAWKHighlight &k, uint16_t raw, int s)
{
    return ((float)raw * (1.0f / 65535.0f) - k.black[s]) * k.inv_range[s];
}

CRAW_DEV float fmax0(float m, float v) { return m > v ? m : v; }   /* the reference's MAX(m, v) */

CRAW_DEV float clampf(float v, float lo, float hi)
{
    return fminf(fmaxf(v, lo), hi);
}

/* Level 0 of the colour field, straight from the mosaic. A CTA makes
 * kF0W x kF0H texels (2x2 quads each, so a kQW x kQH quad region):
 *   1. the clip ramp qa (the largest of the quad's four) of every quad of
 *      the region and kDilate quads around it (0 outside the grid, which
 *      is what skipping those quads gives, all ramps being >= 0), and the
 *      balanced channel sums and largest u of the region's own quads;
 *   2. the largest qa over +-kDilate along x, then along y: the 7x7 max;
 *   3. each quad's weight (1 - amax) * min(umax, 1)^2 and log chroma;
 *   4. per texel, the weighted sums over its quads in the reference's order.
 * The two 16-bit samples of a quad row are one 32-bit load (rows are
 * 16-byte aligned, a quad starts at an even column). */
constexpr int kF0W = 16, kF0H = 8, kF0Threads = 256;
constexpr int kQW = 2 * kF0W, kQH = 2 * kF0H;
constexpr int kAW = kQW + 2 * kDilate, kAH = kQH + 2 * kDilate;

__global__ void __launch_bounds__(kF0Threads) k_hl_level0(const CRAWKHighlight k, const CRAWKHighlightIO io)
{
    __shared__ float qa_s[kAH][kAW];
    __shared__ float hx_s[kAH][kQW];
    __shared__ float4 q_s[kQH][kQW];
    const int qw = k.width / 2, qh = k.height / 2;
    const int qx0 = blockIdx.x * kQW, qy0 = blockIdx.y * kQH;

    /* Every load of the thread first, then their use. */
    constexpr int kIt = (kAW * kAH + kF0Threads - 1) / kF0Threads;
    uint32_t p0s[kIt], p1s[kIt];
#pragma unroll
    for (int it = 0; it < kIt; it++) {
        const int i = threadIdx.x + it * kF0Threads, ay = i / kAW, ax = i - ay * kAW;
        const int qx = qx0 - kDilate + ax, qy = qy0 - kDilate + ay;
        if (i < kAW * kAH && qx >= 0 && qy >= 0 && qx < qw && qy < qh) {
            const char *row = (const char *)io.src + (size_t)(2 * qy) * io.src_pitch + (size_t)qx * 4;
            p0s[it] = __ldg(reinterpret_cast<const uint32_t *>(row));
            p1s[it] = __ldg(reinterpret_cast<const uint32_t *>(row + io.src_pitch));
        }
    }
#pragma unroll
    for (int it = 0; it < kIt; it++) {
        const int i = threadIdx.x + it * kF0Threads, ay = i / kAW, ax = i - ay * kAW;
        const int qx = qx0 - kDilate + ax, qy = qy0 - kDilate + ay;
        if (i >= kAW * kAH)
            break;
        float m = 0.0f;
        if (qx >= 0 && qy >= 0 && qx < qw && qy < qh) {
            const uint32_t p0 = p0s[it], p1 = p1s[it];
            const float u[4] = { site_u(k, (uint16_t)(p0 & 0xffffu), 0), site_u(k, (uint16_t)(p0 >> 16), 1),
                                 site_u(k, (uint16_t)(p1 & 0xffffu), 2), site_u(k, (uint16_t)(p1 >> 16), 3) };
#pragma unroll
            for (int s = 0; s < 4; s++)
                m = fmax0(m, smooth(u[s]));
            const int cx = ax - kDilate, cy = ay - kDilate;
            if (cx >= 0 && cy >= 0 && cx < kQW && cy < kQH) {
                float rgb[3] = { 0.0f, 0.0f, 0.0f }, umax = 0.0f;
#pragma unroll
                for (int s = 0; s < 4; s++) {
                    const int c = site_chan(s);
                    rgb[c] += u[s] * k.wb[c];
                    umax = fmax0(umax, u[s]);
                }
                q_s[cy][cx] = make_float4(rgb[0], rgb[1], rgb[2], umax);
            }
        }
        qa_s[ay][ax] = m;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kAH * kQW; i += kF0Threads) {
        const int r = i / kQW, c = i - r * kQW;
        float m = 0.0f;
#pragma unroll
        for (int d = 0; d <= 2 * kDilate; d++)
            m = fmax0(m, qa_s[r][c + d]);
        hx_s[r][c] = m;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kQH * kQW; i += kF0Threads) {
        const int r = i / kQW, c = i - r * kQW;
        float4 t = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (qx0 + c < qw && qy0 + r < qh) {
            float amax = 0.0f;
#pragma unroll
            for (int d = 0; d <= 2 * kDilate; d++)
                amax = fmax0(amax, hx_s[r + d][c]);
            const float4 q = q_s[r][c];
            const float g0 = q.y * 0.5f, umax = q.w;
            const float m = umax < 1.0f ? umax : 1.0f;
            const float wq = (1.0f - amax) * m * m;
            /* At weight 0 the products are +-0 (the logs are clamped, so
             * finite) and add nothing to a sum that is never -0. */
            if (wq != 0.0f) {
                const float g = fmax0(g0, kEps);
                const float lr = clampf(logf(__fdiv_rn(fmax0(q.x, kEps), g)), -kLogMax, kLogMax);
                const float lb = clampf(logf(__fdiv_rn(fmax0(q.z, kEps), g)), -kLogMax, kLogMax);
                t = make_float4(wq * lr, wq * lb, wq, 0.0f);
            }
        }
        q_s[r][c] = t;
    }
    __syncthreads();
    if (threadIdx.x < kF0W * kF0H) {
        const int tx = threadIdx.x % kF0W, ty = threadIdx.x / kF0W;
        const int bx = blockIdx.x * kF0W + tx, by = blockIdx.y * kF0H + ty;
        if (bx < k.lw[0] && by < k.lh[0]) {
            float acc0 = 0.0f, acc1 = 0.0f, acc2 = 0.0f;
#pragma unroll
            for (int j = 0; j < 2; j++)
#pragma unroll
                for (int i = 0; i < 2; i++) {
                    const float4 q = q_s[2 * ty + j][2 * tx + i];
                    acc0 += q.x;
                    acc1 += q.y;
                    acc2 += q.z;
                }
            float4 *l0 = reinterpret_cast<float4 *>(io.levels) + k.off[0];
            l0[(size_t)by * k.lw[0] + bx] = make_float4(acc0, acc1, acc2, 0.0f);
        }
    }
}

/* Texel (x, y) of level l + 1 as the sum of its children in level l. */
CRAW_DEV void pull_texel(const CRAWKHighlight &k, const CRAWKHighlightIO &io, int l, int x, int y)
{
    const int fw = k.lw[l], fh = k.lh[l];
    const float4 *f = reinterpret_cast<const float4 *>(io.levels) + k.off[l];
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
    for (int dy = 0; dy < 2; dy++)
        for (int dx = 0; dx < 2; dx++) {
            const int fx = 2 * x + dx, fy = 2 * y + dy;
            if (fx >= fw || fy >= fh)
                continue;
            const float4 t = f[(size_t)fy * fw + fx];
            a0 += t.x;
            a1 += t.y;
            a2 += t.z;
        }
    reinterpret_cast<float4 *>(io.levels)[k.off[l + 1] + (size_t)y * k.lw[l + 1] + x] =
        make_float4(a0, a1, a2, 0.0f);
}

__global__ void k_hl_pull(const CRAWKHighlight k, const CRAWKHighlightIO io, int l)
{
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x < k.lw[l + 1] && y < k.lh[l + 1])
        pull_texel(k, io, l, x, y);
}

/* A level's colour at a texel clamped to its edge; the top level still
 * holds sums (reference ref_highlight.c:57-70). */
CRAW_DEV void texel(const float4 *t, int w, int h, int x, int y, bool top, float out[2])
{
    x = x < 0 ? 0 : (x >= w ? w - 1 : x);
    y = y < 0 ? 0 : (y >= h ? h - 1 : y);
    const float4 v = t[(size_t)y * w + x];
    if (top) {
        out[0] = v.z > 0.0f ? __fdiv_rn(v.x, v.z) : 0.0f;
        out[1] = v.z > 0.0f ? __fdiv_rn(v.y, v.z) : 0.0f;
    } else {
        out[0] = v.x;
        out[1] = v.y;
    }
}

/* Bilinear at (px, py), mixed along x first (ref_highlight.c:74-93). */
CRAW_DEV void bilinear(const float4 *t, int w, int h, float px, float py, bool top, float out[2])
{
    const float fx0 = floorf(px), fy0 = floorf(py), fx = px - fx0, fy = py - fy0;
    const int x0 = (int)fx0, y0 = (int)fy0;
    float c00[2], c10[2], c01[2], c11[2];
    texel(t, w, h, x0, y0, top, c00);
    texel(t, w, h, x0 + 1, y0, top, c10);
    texel(t, w, h, x0, y0 + 1, top, c01);
    texel(t, w, h, x0 + 1, y0 + 1, top, c11);
#pragma unroll
    for (int i = 0; i < 2; i++) {
        const float a = __fadd_rn(__fmul_rn(c00[i], 1.0f - fx), __fmul_rn(c10[i], fx));
        const float b = __fadd_rn(__fmul_rn(c01[i], 1.0f - fx), __fmul_rn(c11[i], fx));
        out[i] = __fadd_rn(__fmul_rn(a, 1.0f - fy), __fmul_rn(b, fy));
    }
}

/* Texel (x, y) of level l pushed from level l + 1, in place. */
CRAW_DEV void push_texel(const CRAWKHighlight &k, const CRAWKHighlightIO &io, int l, int x, int y)
{
    const int w = k.lw[l];
    const float4 *c = reinterpret_cast<const float4 *>(io.levels) + k.off[l + 1];
    float4 *f = reinterpret_cast<float4 *>(io.levels) + k.off[l];
    float up[2];
    bilinear(c, k.lw[l + 1], k.lh[l + 1], ((float)x + 0.5f) * 0.5f - 0.5f,
             ((float)y + 0.5f) * 0.5f - 0.5f, l + 2 == k.nb_levels, up);
    float4 t = f[(size_t)y * w + x];
    if (t.z > 0.0f) {
        const float q = __fdiv_rn(t.z, kWSat), s = q < 1.0f ? q : 1.0f;
        t.x = up[0] + s * (__fdiv_rn(t.x, t.z) - up[0]);
        t.y = up[1] + s * (__fdiv_rn(t.y, t.z) - up[1]);
    } else {
        t.x = up[0];
        t.y = up[1];
    }
    f[(size_t)y * w + x] = t;
}

__global__ void k_hl_push(const CRAWKHighlight k, const CRAWKHighlightIO io, int l)
{
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x < k.lw[l] && y < k.lh[l])
        push_texel(k, io, l, x, y);
}

/* The coarse end of the pyramid in one CTA: pull from level l0 to the top,
 * then push back down to l0, a barrier between levels (a dozen tiny
 * launches otherwise). */
constexpr int kCoarseThreads = 1024, kCoarseTexels = 8192;

__global__ void __launch_bounds__(kCoarseThreads) k_hl_coarse(const CRAWKHighlight k, const CRAWKHighlightIO io, int l0)
{
    for (int l = l0; l + 1 < k.nb_levels; l++) {
        const int w = k.lw[l + 1], n = w * k.lh[l + 1];
        for (int i = threadIdx.x; i < n; i += kCoarseThreads)
            pull_texel(k, io, l, i % w, i / w);
        __syncthreads();
    }
    for (int l = k.nb_levels - 2; l >= l0; l--) {
        const int w = k.lw[l], n = w * k.lh[l];
        for (int i = threadIdx.x; i < n; i += kCoarseThreads)
            push_texel(k, io, l, i % w, i / w);
        __syncthreads();
    }
}

/* The lift of one site (reference ref_highlight.c:286-327): `xc` its
 * balanced value, `a` its ramp; (s1, n1, m1) and (s2, n2, m2) the sum,
 * count and largest ramp of its neighbours of the other two channels
 * k1 < k2, `rho1`, `rho2`, `rhoc` their and its own log chroma. The
 * counts are 2 or 4, so the means are products with 1/n, which round as
 * the quotients do. */
CRAW_DEV float lift(float xc, float a, float s1, float inv_n1, float m1, float s2, float inv_n2, float m2,
                    float rho1, float rho2, float rhoc)
{
    const float a1 = 1.0f - m1, a2 = 1.0f - m2;
    const float l1 = logf(fmax0(s1 * inv_n1, kEps)) - rho1;
    const float l2 = logf(fmax0(s2 * inv_n2, kEps)) - rho2;
    const float lc = logf(fmax0(xc, kEps)) - rhoc;
    const float A = a1 + a2;
    const float lfull = expf(fmax0(lc, fmax0(l1, l2)));
    const float lpart = A > 0.0f ? expf(__fdiv_rn(a1 * l1 + a2 * l2, A)) : lfull;
    const float L = lfull + (A < 1.0f ? A : 1.0f) * (lpart - lfull);
    return xc + a * fmax0(L * expf(rhoc) - xc, 0.0f);
}

/* A CTA rebuilds kFillW x kFillH quads, one a thread. The u and ramp of
 * its samples and a one-sample apron (mirrored at the frame's edge;
 * mirroring keeps parity) are staged in shared memory once; staged
 * column j holds frame column X0 - 2 + j, so a quad's own pair is an
 * aligned float2. A quad none of whose sites is near the clip only scales
 * its four samples; otherwise its 4x4 window (cell (r, c) = frame position
 * (x0 - 1 + c, y0 - 1 + r), CFA site ((r + 1) & 1) * 2 + ((c + 1) & 1),
 * known at compile time) is read and each site whose ramp is above 0 is
 * lifted. Neighbours of each channel are summed in the reference's scan
 * order (rows, then columns). */
/* The mirror of a staged position: one reflection, which is exact for
 * the positions a window reads (at most one sample outside the frame),
 * then a clamp that keeps the positions no window reads (a tile hanging
 * past a small frame) inside it. */
CRAW_DEV int edge(int v, int n)
{
    v = v < 0 ? -v : v;
    v = v >= n ? 2 * n - 2 - v : v;
    return v < 0 ? 0 : v;
}

constexpr int kFillW = 32, kFillH = 8, kFillThreads = kFillW * kFillH;
constexpr int kStH = 2 * kFillH + 2, kStPitch = 2 * kFillW + 4, kStPairs = kStPitch / 2;
constexpr int kStN = kStPairs * kStH, kStIt = (kStN + kFillThreads - 1) / kFillThreads;

__global__ void __launch_bounds__(kFillThreads) k_hl_fill(const CRAWKHighlight k, const CRAWKHighlightIO io)
{
    __shared__ __align__(16) float u_s[kStH][kStPitch];
    __shared__ __align__(16) float a_s[kStH][kStPitch];
    const int X0 = blockIdx.x * 2 * kFillW, Y0 = blockIdx.y * 2 * kFillH;
    const int tid = threadIdx.y * kFillW + threadIdx.x;
    /* Staged in pairs of samples (an even frame column and the next: one
     * 32-bit load inside the frame, two mirrored loads past its edge), all
     * of a thread's loads first, then their use. X0 and Y0 are even, so a
     * staged sample's CFA site follows from its staged row and column. */
    uint32_t raw[kStIt];
#pragma unroll
    for (int it = 0; it < kStIt; it++) {
        const int i = tid + it * kFillThreads, r = i / kStPairs, xa = X0 - 2 + 2 * (i - r * kStPairs);
        if (i < kStN) {
            const int yr = edge(Y0 - 1 + r, k.height);
            const uint16_t *row = reinterpret_cast<const uint16_t *>(
                (const char *)io.src + (size_t)yr * io.src_pitch);
            if (!craw_in_bounds(yr >= 0 && yr < k.height, io.err))
                raw[it] = 0u;
            else if (xa >= 0 && xa + 1 < k.width)
                raw[it] = __ldg(reinterpret_cast<const uint32_t *>(row + xa));
            else
                raw[it] = (uint32_t)__ldg(row + edge(xa, k.width)) |
                          ((uint32_t)__ldg(row + edge(xa + 1, k.width)) << 16);
        }
    }
#pragma unroll
    for (int it = 0; it < kStIt; it++) {
        const int i = tid + it * kFillThreads, r = i / kStPairs, j = 2 * (i - r * kStPairs);
        if (i < kStN) {
            /* The sites' constants by selects, not a runtime index into
             * the parameter block. */
            const bool odd_row = !(r & 1);
            const float b0 = odd_row ? k.black[2] : k.black[0], b1 = odd_row ? k.black[3] : k.black[1];
            const float i0 = odd_row ? k.inv_range[2] : k.inv_range[0];
            const float i1 = odd_row ? k.inv_range[3] : k.inv_range[1];
            const float v0 = ((float)(raw[it] & 0xffffu) * (1.0f / 65535.0f) - b0) * i0;
            const float v1 = ((float)(raw[it] >> 16) * (1.0f / 65535.0f) - b1) * i1;
            *reinterpret_cast<float2 *>(&u_s[r][j]) = make_float2(v0, v1);
            *reinterpret_cast<float2 *>(&a_s[r][j]) = make_float2(smooth(v0), smooth(v1));
        }
    }
    __syncthreads();
    const int qw = k.width / 2, qh = k.height / 2;
    const int qx = blockIdx.x * kFillW + threadIdx.x, qy = blockIdx.y * kFillH + threadIdx.y;
    if (qx >= qw || qy >= qh)
        return;
    const int x0 = 2 * qx, y0 = 2 * qy;
    const int sr = 2 * threadIdx.y, sc = 2 * threadIdx.x + 1;   /* window cell (0, 0) */
    const float2 uc0 = *reinterpret_cast<const float2 *>(&u_s[sr + 1][sc + 1]);
    const float2 uc1 = *reinterpret_cast<const float2 *>(&u_s[sr + 2][sc + 1]);
    const float2 ac0 = *reinterpret_cast<const float2 *>(&a_s[sr + 1][sc + 1]);
    const float2 ac1 = *reinterpret_cast<const float2 *>(&a_s[sr + 2][sc + 1]);
    const float wr = k.wb[0], wg = k.wb[1], wbl = k.wb[2];
    float out[2][2];
    out[0][0] = uc0.x * wr;
    out[0][1] = uc0.y * wg;
    out[1][0] = uc1.x * wg;
    out[1][1] = uc1.y * wbl;
    if (ac0.x > 0.0f || ac0.y > 0.0f || ac1.x > 0.0f || ac1.y > 0.0f) {
        float u[4][4], ar[4][4];
#pragma unroll
        for (int r = 0; r < 4; r++)
#pragma unroll
            for (int c = 0; c < 4; c++) {
                u[r][c] = u_s[sr + r][sc + c];
                ar[r][c] = a_s[sr + r][sc + c];
            }
        float lf[2];
        bilinear(reinterpret_cast<const float4 *>(io.levels) + k.off[0], k.lw[0], k.lh[0],
                 (float)qx * 0.5f - 0.25f, (float)qy * 0.5f - 0.25f, false, lf);
        /* R at cell (1, 1): G on the cross, B on the diagonals. */
        if (ar[1][1] > 0.0f) {
            float sg = 0.0f, mg = 0.0f, sb = 0.0f, mb = 0.0f;
            sb += u[0][0] * wbl; mb = fmax0(mb, ar[0][0]);
            sg += u[0][1] * wg;  mg = fmax0(mg, ar[0][1]);
            sb += u[0][2] * wbl; mb = fmax0(mb, ar[0][2]);
            sg += u[1][0] * wg;  mg = fmax0(mg, ar[1][0]);
            sg += u[1][2] * wg;  mg = fmax0(mg, ar[1][2]);
            sb += u[2][0] * wbl; mb = fmax0(mb, ar[2][0]);
            sg += u[2][1] * wg;  mg = fmax0(mg, ar[2][1]);
            sb += u[2][2] * wbl; mb = fmax0(mb, ar[2][2]);
            out[0][0] = lift(out[0][0], ar[1][1], sg, 0.25f, mg, sb, 0.25f, mb, 0.0f, lf[1], lf[0]);
        }
        /* Gr at cell (1, 2): R left and right, B above and below. */
        if (ar[1][2] > 0.0f) {
            float sr = 0.0f, mr = 0.0f, sb = 0.0f, mb = 0.0f;
            sb += u[0][2] * wbl; mb = fmax0(mb, ar[0][2]);
            sr += u[1][1] * wr;  mr = fmax0(mr, ar[1][1]);
            sr += u[1][3] * wr;  mr = fmax0(mr, ar[1][3]);
            sb += u[2][2] * wbl; mb = fmax0(mb, ar[2][2]);
            out[0][1] = lift(out[0][1], ar[1][2], sr, 0.5f, mr, sb, 0.5f, mb, lf[0], lf[1], 0.0f);
        }
        /* Gb at cell (2, 1): R above and below, B left and right. */
        if (ar[2][1] > 0.0f) {
            float sr = 0.0f, mr = 0.0f, sb = 0.0f, mb = 0.0f;
            sr += u[1][1] * wr;  mr = fmax0(mr, ar[1][1]);
            sb += u[2][0] * wbl; mb = fmax0(mb, ar[2][0]);
            sb += u[2][2] * wbl; mb = fmax0(mb, ar[2][2]);
            sr += u[3][1] * wr;  mr = fmax0(mr, ar[3][1]);
            out[1][0] = lift(out[1][0], ar[2][1], sr, 0.5f, mr, sb, 0.5f, mb, lf[0], lf[1], 0.0f);
        }
        /* B at cell (2, 2): R on the diagonals, G on the cross. */
        if (ar[2][2] > 0.0f) {
            float sr = 0.0f, mr = 0.0f, sg = 0.0f, mg = 0.0f;
            sr += u[1][1] * wr;  mr = fmax0(mr, ar[1][1]);
            sg += u[1][2] * wg;  mg = fmax0(mg, ar[1][2]);
            sr += u[1][3] * wr;  mr = fmax0(mr, ar[1][3]);
            sg += u[2][1] * wg;  mg = fmax0(mg, ar[2][1]);
            sg += u[2][3] * wg;  mg = fmax0(mg, ar[2][3]);
            sr += u[3][1] * wr;  mr = fmax0(mr, ar[3][1]);
            sg += u[3][2] * wg;  mg = fmax0(mg, ar[3][2]);
            sr += u[3][3] * wr;  mr = fmax0(mr, ar[3][3]);
            out[1][1] = lift(out[1][1], ar[2][2], sr, 0.25f, mr, sg, 0.25f, mg, lf[0], 0.0f, lf[1]);
        }
    }
#pragma unroll
    for (int r = 0; r < 2; r++) {
        __half2 hv = __floats2half2_rn(out[r][0], out[r][1]);
        if (craw_in_bounds(x0 >= 0 && x0 + 1 < k.width && y0 + r >= 0 && y0 + r < k.height, io.err))
            *reinterpret_cast<__half2 *>((char *)io.dst + (size_t)(y0 + r) * io.dst_pitch + (size_t)x0 * 2) = hv;
    }
}

dim3 grid2(int w, int h) { return dim3((w + 31) / 32, (h + 7) / 8); }

} // namespace

extern "C" int64_t craw_k_highlight_levels(int32_t width, int32_t height, CRAWKHighlight *k)
{
    int64_t total = 0;
    int n = 0;
    for (int lw = (width + 3) / 4, lh = (height + 3) / 4;; lw = (lw + 1) / 2, lh = (lh + 1) / 2) {
        if (n == CRAW_K_HL_LEVELS)
            return -1;
        k->lw[n] = lw;
        k->lh[n] = lh;
        k->off[n] = total;
        total += (int64_t)lw * lh;
        n++;
        if (lw == 1 && lh == 1)
            break;
    }
    k->nb_levels = n;
    return total;
}

extern "C" int craw_k_highlights(const CRAWKHighlight *k, const CRAWKHighlightIO *io, cudaStream_t s)
{
    if (craw_launch_ready() < 0)
        return -5;
    const int qw = k->width / 2, qh = k->height / 2;
    const dim3 blk(32, 8);
    k_hl_level0<<<dim3((k->lw[0] + kF0W - 1) / kF0W, (k->lh[0] + kF0H - 1) / kF0H), kF0Threads, 0, s>>>(
        *k, *io);
    /* The levels from lc up are small enough for one CTA. */
    int lc = 0;
    while (lc + 1 < k->nb_levels && (int64_t)k->lw[lc] * k->lh[lc] > kCoarseTexels)
        lc++;
    for (int l = 0; l < lc; l++)
        k_hl_pull<<<grid2(k->lw[l + 1], k->lh[l + 1]), blk, 0, s>>>(*k, *io, l);
    if (k->nb_levels > 1)
        k_hl_coarse<<<1, kCoarseThreads, 0, s>>>(*k, *io, lc);
    for (int l = lc - 1; l >= 0; l--)
        k_hl_push<<<grid2(k->lw[l], k->lh[l]), blk, 0, s>>>(*k, *io, l);
    k_hl_fill<<<grid2(qw, qh), blk, 0, s>>>(*k, *io);
    return cudaGetLastError() == cudaSuccess ? 0 : -5;
}
