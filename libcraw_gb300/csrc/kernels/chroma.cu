/*
 * Chroma denoise on the quarter-resolution colour differences (reference
 * lib/ref/ref_chroma.c:22-158; the block means of its pass 1 are formed in
 * the develop kernel's epilogue). Pass 2 is a 9x9 joint bilateral on the
 * quarter grid; pass 3 puts the smoothed band back into every pixel and is
 * fused here with the AWB block statistic and the colour stage, so the
 * updated intermediate never goes to memory unless it is asked for.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace {

constexpr int kR = 4;                       /* reference ref_chroma.c:15 */
constexpr float kInv2s2 = 1.0f / 8.0f;      /* 1 / (2 sigma_s^2), sigma_s = 2 */
constexpr float kRangeK = 0.35f, kChromaK = 0.35f, kRangeEps = 0.02f;

constexpr int BX = 32, BY = 8;              /* quarter texels per CTA */

__global__ void __launch_bounds__(BX * BY)
k_chroma_blur(const CRAWKChroma c, const void *q, size_t q_pitch, void *qf, size_t qf_pitch)
{
    __shared__ float4 t[(BY + 2 * kR) * (BX + 2 * kR)];
    constexpr int SX = BX + 2 * kR;
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    for (int i = threadIdx.x; i < (BY + 2 * kR) * SX; i += BX * BY) {
        int x = craw_mirror(x0 - kR + i % SX, c.qw), y = craw_mirror(y0 - kR + i / SX, c.qh);
        float v[3] = { 0.0f, 0.0f, 0.0f };
        if (craw_in_bounds(x >= 0 && x < c.qw && y >= 0 && y < c.qh, c.err))
            craw_load_rgb(q, q_pitch, x, y, c.fp16, v);
        t[i] = make_float4(v[0], v[1], v[2], 0.0f);
    }
    __syncthreads();
    const int lx = threadIdx.x % BX, ly = threadIdx.x / BX;
    const int x = x0 + lx, y = y0 + ly;
    if (x >= c.qw || y >= c.qh || !craw_in_bounds(x >= 0 && y >= 0, c.err))
        return;
    const float4 ctr = t[(ly + kR) * SX + lx + kR];
    const float level = fmaxf(ctr.z, 0.0f) + kRangeEps;
    const float inv_range = 1.0f / (kRangeK * level), inv_chroma = 1.0f / (kChromaK * level);
    float a0 = 0.0f, a1 = 0.0f, ws = 0.0f;
#pragma unroll
    for (int dy = -kR; dy <= kR; dy++) {
#pragma unroll
        for (int dx = -kR; dx <= kR; dx++) {
            float4 s = t[(ly + kR + dy) * SX + lx + kR + dx];
            float dg = (s.z - ctr.z) * inv_range;
            float d0 = (s.x - ctr.x) * inv_chroma, d1 = (s.y - ctr.y) * inv_chroma;
            /* The fast exponential: CUDA documents its error as at most
             * 2 + floor(|1.16 x|) ulp, i.e. under 1e-6 relative for the
             * weights that matter (|x| < 10, w > 4.5e-5 of the centre's
             * 1) and larger only for weights too small to move the
             * normalised weighted mean; the stage is held to 2e-4 against
             * the oracle (tests/test_gpu_parity.py, saturated rectangles
             * and zone plates, so large chroma differences). */
            float w = __expf(-(float)(dx * dx + dy * dy) * kInv2s2 - dg * dg - d0 * d0 - d1 * d1);
            a0 += w * s.x;
            a1 += w * s.y;
            ws += w;
        }
    }
    craw_store_rgba(qf, qf_pitch, x, y, c.fp16, a0 / ws, a1 / ws, ctr.z);
}

/* 64x32 pixels a CTA, 8 a thread: the AWB block sums at the end are
 * sequential chains on a few threads (32 blocks here), and a larger tile
 * keeps that tail a small part of a CTA's life (at 5760x3240: 32x16 tiles
 * 0.172 ms, 64x32 0.134 ms, 64x48 0.147 ms with fewer CTAs an SM). */
constexpr int TW = 64, TH = 32, NT = 256;

__global__ void __launch_bounds__(NT)
k_chroma_up_color(const CRAWKDevelop k, const CRAWKChroma c, const void *inter, size_t inter_pitch,
                  const void *q, const void *qf, size_t q_pitch, void *dst, size_t dst_pitch,
                  int dst_fmt, void *inter_out, const CRAWKAwbOut awb)
{
    __shared__ __align__(16) float rgb_s[3 * TW * TH];
    static_assert(TW % 8 == 0, "block rows are whole float4s");
    const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
#pragma unroll
    for (int j = 0; j < TW * TH / NT; j++) {
        int i = threadIdx.x + j * NT, x = x0 + i % TW, y = y0 + i / TW;
        if (x >= c.width || y >= c.height)
            continue;
        float fy = ((float)y + 0.5f) * 0.25f - 0.5f, fly = floorf(fy), ty = fy - fly;
        float fx = ((float)x + 0.5f) * 0.25f - 0.5f, flx = floorf(fx), tx = fx - flx;
        int ya = min(max((int)fly, 0), c.qh - 1), yb = min(max((int)fly + 1, 0), c.qh - 1);
        int xa = min(max((int)flx, 0), c.qw - 1), xb = min(max((int)flx + 1, 0), c.qw - 1);
        if (!craw_in_bounds(x >= 0 && y >= 0 && xa >= 0 && ya >= 0 && xb < c.qw && yb < c.qh, c.err))
            continue;
        float w00 = (1.0f - tx) * (1.0f - ty), w10 = tx * (1.0f - ty);
        float w01 = (1.0f - tx) * ty, w11 = tx * ty;
        float d00[3], d10[3], d01[3], d11[3], b00[3], b10[3], b01[3], b11[3], px[3];
        craw_load_rgb(q, q_pitch, xa, ya, c.fp16, d00);
        craw_load_rgb(q, q_pitch, xb, ya, c.fp16, d10);
        craw_load_rgb(q, q_pitch, xa, yb, c.fp16, d01);
        craw_load_rgb(q, q_pitch, xb, yb, c.fp16, d11);
        craw_load_rgb(qf, q_pitch, xa, ya, c.fp16, b00);
        craw_load_rgb(qf, q_pitch, xb, ya, c.fp16, b10);
        craw_load_rgb(qf, q_pitch, xa, yb, c.fp16, b01);
        craw_load_rgb(qf, q_pitch, xb, yb, c.fp16, b11);
        craw_load_rgb(inter, inter_pitch, x, y, c.fp16, px);
        float g = px[1], d[2] = { px[0] - g, px[2] - g };
#pragma unroll
        for (int ch = 0; ch < 2; ch++) {
            float lo = w00 * d00[ch] + w10 * d10[ch] + w01 * d01[ch] + w11 * d11[ch];
            float lf = w00 * b00[ch] + w10 * b10[ch] + w01 * b01[ch] + w11 * b11[ch];
            d[ch] += c.strength * (lf - lo);
        }
        float o[3] = { g + d[0], g, g + d[1] };
        if (c.fp16) {
            o[0] = craw_round_half(o[0]);
            o[2] = craw_round_half(o[2]);
        }
        rgb_s[3 * i + 0] = o[0];
        rgb_s[3 * i + 1] = o[1];
        rgb_s[3 * i + 2] = o[2];
        if (inter_out)
            craw_store_rgba(inter_out, inter_pitch, x, y, c.fp16, o[0], o[1], o[2]);
        float co[3];
        craw_color(k.color, o, co);
        craw_store_rgba(dst, dst_pitch, x, y, dst_fmt, co[0], co[1], co[2]);
    }
    if (!awb.rec)
        return;
    __syncthreads();
    const int blocks_x = (c.width + 7) / 8;
    for (int b = threadIdx.x; b < (TW / 8) * (TH / 8); b += NT) {
        int bx = b % (TW / 8), by = b / (TW / 8);
        if (x0 + bx * 8 >= c.width || y0 + by * 8 >= c.height)
            continue;
        int xe = min(8, c.width - (x0 + bx * 8)), ye = min(8, c.height - (y0 + by * 8));
        float s0 = 0.f, s1 = 0.f, s2 = 0.f;
        if (xe == 8 && ye == 8) {
            /* A whole block: the same order, unrolled, a row's 24 values
             * read as six 16-byte loads ahead of the dependent adds. */
#pragma unroll
            for (int jj = 0; jj < 8; jj++) {
                const float4 *row = reinterpret_cast<const float4 *>(
                    &rgb_s[3 * ((by * 8 + jj) * TW + bx * 8)]);
                float v[24];
#pragma unroll
                for (int u = 0; u < 6; u++) {
                    const float4 t = row[u];
                    v[4 * u] = t.x; v[4 * u + 1] = t.y; v[4 * u + 2] = t.z; v[4 * u + 3] = t.w;
                }
#pragma unroll
                for (int ii = 0; ii < 8; ii++) {
                    s0 = __fadd_rn(s0, v[3 * ii]);
                    s1 = __fadd_rn(s1, v[3 * ii + 1]);
                    s2 = __fadd_rn(s2, v[3 * ii + 2]);
                }
            }
        } else {
            for (int jj = 0; jj < ye; jj++)
                for (int ii = 0; ii < xe; ii++) {
                    const float *p = &rgb_s[3 * ((by * 8 + jj) * TW + bx * 8 + ii)];
                    s0 = __fadd_rn(s0, p[0]);
                    s1 = __fadd_rn(s1, p[1]);
                    s2 = __fadd_rn(s2, p[2]);
                }
        }
        float n = (float)(xe * ye);
        const size_t ri = (size_t)(y0 / 8 + by) * blocks_x + x0 / 8 + bx;
        if (!craw_in_bounds(ri < craw_awb_blocks(k.width, k.height), c.err))
            continue;
        awb.rec[ri] =
            craw_awb_block(__fdiv_rn(s0, n), __fdiv_rn(s1, n), __fdiv_rn(s2, n), k.awb_wb,
                           awb.deferred, awb.nb_deferred, craw_awb_blocks(k.width, k.height));
    }
}

} // namespace

extern "C" int craw_k_chroma_blur(const CRAWKChroma *c, const void *q, size_t q_pitch,
                                  void *qf, size_t qf_pitch, cudaStream_t s)
{
    if (craw_launch_ready() < 0)
        return -5;
    dim3 grid((c->qw + BX - 1) / BX, (c->qh + BY - 1) / BY);
    k_chroma_blur<<<grid, BX * BY, 0, s>>>(*c, q, q_pitch, qf, qf_pitch);
    return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

extern "C" int craw_k_chroma_up_color(const CRAWKDevelop *k, const CRAWKChroma *c,
                                      const void *inter, size_t inter_pitch,
                                      const void *q, const void *qf, size_t q_pitch,
                                      void *dst, size_t dst_pitch, int dst_fmt,
                                      void *inter_out, const CRAWKAwbOut *awb, cudaStream_t s)
{
    if (craw_launch_ready() < 0)
        return -5;
    dim3 grid((c->width + TW - 1) / TW, (c->height + TH - 1) / TH);
    k_chroma_up_color<<<grid, NT, 0, s>>>(*k, *c, inter, inter_pitch, q, qf, q_pitch, dst,
                                          dst_pitch, dst_fmt, inter_out, *awb);
    return cudaGetLastError() == cudaSuccess ? 0 : -5;
}
