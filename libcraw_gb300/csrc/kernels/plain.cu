/*
 * The plain FP32 pipeline: the same algorithm as the fused kernels, as one
 * straightforward kernel per stage, one thread per output value, every
 * intermediate a full-resolution FP32 image in device memory and every
 * stencil read through the cache (mirrored per tap, except that the NLM
 * reads directly where its whole window lies inside the plane). It is
 * the baseline the fused pipeline is measured against, and a second,
 * independent GPU formulation of the reference's sweeps
 * (lib/ref/ref_denoise.c:168-336, lib/ref/ref_debayer.c:42-395,
 * lib/ref/ref_chroma.c, lib/awb.c:213-296, lib/ref/ref_color.c:10-76).
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace {

constexpr int S = 3, P = 1;
constexpr int B2 = 16;   /* 16 x 16 thread blocks */

CRAW_DEV float at(const float *p, int w, int h, int x, int y)
{
    return p[(size_t)craw_mirror(y, h) * w + craw_mirror(x, w)];
}

#define GRID2(w, h) dim3(((w) + B2 - 1) / B2, ((h) + B2 - 1) / B2), dim3(B2, B2)
#define XY                                                  \
    const int x = blockIdx.x * B2 + threadIdx.x;            \
    const int y = blockIdx.y * B2 + threadIdx.y;

/* ---------------------------------------------------------------- denoise */

CRAW_DEV float gat_fwd(const CRAWKDenoise &k, float u)
{
    return u >= 0.0f ? k.gat_fwd * sqrtf(k.gat_a * u + k.gat_c) : k.gat_t0 + u / k.gat_sc;
}

CRAW_DEV float gat_inv(const CRAWKDenoise &k, float t)
{
    return t >= k.gat_t0 ? k.gat_inv * t * t - k.gat_off : (t - k.gat_t0) * k.gat_sc;
}

CRAW_DEV float dn_level(const CRAWKDenoise &k, const CRAWKDenoiseIO &io, int mx, int my, int pl)
{
    const uint16_t *r = (const uint16_t *)((const char *)io.src + (size_t)my * io.src_pitch);
    return ((float)r[mx] * (1.0f / 65535.0f) - k.black[pl]) * k.inv_range[pl];
}

/* Stabilised planes (4 x pw x ph), and with a history the temporal
 * average and the variance it leaves. */
__global__ void p_dn_vst(const CRAWKDenoise k, const CRAWKDenoiseIO io, float *t, float *cur,
                         float *prv)
{
    XY
    const int pl = blockIdx.z;
    if (x >= k.pw || y >= k.ph)
        return;
    const int mx = 2 * x + (pl & 1), my = 2 * y + (pl >> 1);
    const size_t i = ((size_t)pl * k.ph + y) * k.pw + x;
    float tc = gat_fwd(k, dn_level(k, io, mx, my, pl));
    if (k.mode & CRAW_K_DN_HISTORY) {
        const float *lr = (const float *)((const char *)io.lvl_prev + (size_t)my * io.lvl_pitch);
        cur[i] = tc;
        prv[i] = gat_fwd(k, lr[mx]);
    } else {
        t[i] = tc;
    }
}

__global__ void p_dn_temporal(const CRAWKDenoise k, const CRAWKDenoiseIO io, float *t,
                              const float *cur, const float *prv, float *var)
{
    XY
    const int pl = blockIdx.z;
    if (x >= k.pw || y >= k.ph)
        return;
    const size_t o = (size_t)pl * k.ph * k.pw;
    float d2 = 0.0f;
    for (int ky = -1; ky <= 1; ky++)
        for (int kx = -1; kx <= 1; kx++) {
            float e = at(prv + o, k.pw, k.ph, x + kx, y + ky) - at(cur + o, k.pw, k.ph, x + kx, y + ky);
            d2 += e * e;
        }
    float a = k.t_alpha * expf(-fmaxf(d2 * (1.0f / 9.0f) * k.t_inv_h2 - 2.0f, 0.0f));
    const int mx = 2 * x + (pl & 1), my = 2 * y + (pl >> 1);
    const uint8_t *vr = io.var_prev + (size_t)my * io.var_pitch;
    float sp = (float)vr[mx] * (1.0f / 255.0f);
    const size_t i = o + (size_t)y * k.pw + x;
    t[i] = cur[i] * (1.0f - a) + prv[i] * a;
    var[i] = fmaxf((1.0f - a) * (1.0f - a) + a * a * (sp * sp), 1.0e-4f);
}

__global__ void p_dn_nlm(const CRAWKDenoise k, const CRAWKDenoiseIO io, const float *t,
                         const float *var)
{
    XY
    const int pl = blockIdx.z;
    if (x >= k.pw || y >= k.ph)
        return;
    const size_t o = (size_t)pl * k.ph * k.pw;
    const float *tp = t + o;
    const bool hist = (k.mode & CRAW_K_DN_HISTORY) != 0;
    const float *vp = hist ? var + o : nullptr;
    const int mx = 2 * x + (pl & 1), my = 2 * y + (pl >> 1);
    const float tc = tp[(size_t)y * k.pw + x];
    float u;
    if (k.mode & CRAW_K_DN_SPATIAL) {
        float acc = 0.0f, wsum = 0.0f;
        const float vc = hist ? vp[(size_t)y * k.pw + x] : 1.0f;
        /* The plane value at (x + a, y + b): read directly where the whole
         * 9x9 window lies inside the plane (nearly every sample), mirrored
         * at the edges. The centre's own patch is read once. */
        const bool inner = x >= S + P && y >= S + P && x + S + P < k.pw && y + S + P < k.ph;
        auto val = [&](const float *pp, int a, int b) {
            return inner ? __ldg(pp + (size_t)(y + b) * k.pw + x + a) : at(pp, k.pw, k.ph, x + a, y + b);
        };
        float c[2 * P + 1][2 * P + 1];
        for (int ky = -P; ky <= P; ky++)
            for (int kx = -P; kx <= P; kx++)
                c[ky + P][kx + P] = val(tp, kx, ky);
        for (int dy = -S; dy <= S; dy++) {
            for (int dx = -S; dx <= S; dx++) {
                float d2 = 0.0f;
#pragma unroll
                for (int ky = -P; ky <= P; ky++)
#pragma unroll
                    for (int kx = -P; kx <= P; kx++) {
                        float e = c[ky + P][kx + P] - val(tp, dx + kx, dy + ky);
                        d2 += e * e;
                    }
                float w;
                if (hist) {
                    float v2 = vc + val(vp, dx, dy);
                    w = expf(-fmaxf(d2 * (1.0f / 9.0f) * k.inv_h2 - v2, 0.0f) / vc);
                } else {
                    w = expf(-fmaxf(d2 * (1.0f / 9.0f) * k.inv_h2 - 2.0f, 0.0f));
                }
                wsum += w;
                acc += w * val(tp, dx, dy);
            }
        }
        u = gat_inv(k, acc / wsum);
    } else {
        u = gat_inv(k, tc);
    }
    if (k.mode & CRAW_K_DN_TEMPORAL) {
        float *lr = (float *)((char *)io.lvl_next + (size_t)my * io.lvl_pitch);
        lr[mx] = gat_inv(k, tc);
        io.var_next[(size_t)my * io.var_pitch + mx] =
            hist ? (uint8_t)rintf(sqrtf(fminf(fmaxf(var[o + (size_t)y * k.pw + x], 0.0f), 1.0f)) * 255.0f)
                 : (uint8_t)255;
    }
    float u0 = dn_level(k, io, mx, my, pl);
    float gr = fminf(fmaxf((u0 - k.guard_lo) * k.guard_inv, 0.0f), 1.0f);
    u = u + (u0 - u) * gr;
    float ro = fminf(fmaxf(k.black[pl] + u * k.range[pl], 0.0f), 1.0f);
    ((uint16_t *)((char *)io.dst + (size_t)my * io.dst_pitch))[mx] = (uint16_t)rintf(ro * 65535.0f);
}

/* ---------------------------------------------------------------- develop */

__global__ void p_prep(const CRAWKDevelop k, const uint16_t *src, size_t pitch, float *v)
{
    XY
    if (x >= k.width || y >= k.height)
        return;
    uint16_t raw = ((const uint16_t *)((const char *)src + (size_t)y * pitch))[x];
    v[(size_t)y * k.width + x] = craw_prep(k, raw, (y & 1) * 2 + (x & 1));
}

CRAW_DEV void put(float *inter, size_t pitch, int x, int y, float r, float g, float b)
{
    reinterpret_cast<float4 *>((char *)inter + (size_t)y * pitch)[x] = make_float4(r, g, b, 1.0f);
}

#define V(dx, dy) at(v, w, h, x + (dx), y + (dy))

__global__ void p_bilinear(int w, int h, const float *v, float *inter, size_t ip)
{
    XY
    if (x >= w || y >= h)
        return;
    int s = (y & 1) * 2 + (x & 1);
    float edge = 0.25f * (V(0, -1) + V(0, 1) + V(-1, 0) + V(1, 0));
    float corner = 0.25f * (V(-1, -1) + V(1, -1) + V(-1, 1) + V(1, 1));
    float horiz = 0.5f * (V(-1, 0) + V(1, 0)), vert = 0.5f * (V(0, -1) + V(0, 1));
    float c = V(0, 0);
    if (s == 0)      put(inter, ip, x, y, c, edge, corner);
    else if (s == 1) put(inter, ip, x, y, horiz, c, vert);
    else if (s == 2) put(inter, ip, x, y, vert, c, horiz);
    else             put(inter, ip, x, y, corner, edge, c);
}

__global__ void p_mhc(int w, int h, const float *v, float *inter, size_t ip)
{
    XY
    if (x >= w || y >= h)
        return;
    int s = (y & 1) * 2 + (x & 1);
    float c = V(0, 0);
    float g = (4.0f * c + 2.0f * (V(0, -1) + V(0, 1) + V(-1, 0) + V(1, 0))
               - (V(0, -2) + V(0, 2) + V(-2, 0) + V(2, 0))) * 0.125f;
    float hz = (5.0f * c + 4.0f * (V(-1, 0) + V(1, 0))
                - (V(-1, -1) + V(1, -1) + V(-1, 1) + V(1, 1) + V(-2, 0) + V(2, 0))
                + 0.5f * (V(0, -2) + V(0, 2))) * 0.125f;
    float vt = (5.0f * c + 4.0f * (V(0, -1) + V(0, 1))
                - (V(-1, -1) + V(1, -1) + V(-1, 1) + V(1, 1) + V(0, -2) + V(0, 2))
                + 0.5f * (V(-2, 0) + V(2, 0))) * 0.125f;
    float d = (6.0f * c + 2.0f * (V(-1, -1) + V(1, -1) + V(-1, 1) + V(1, 1))
               - 1.5f * (V(0, -2) + V(0, 2) + V(-2, 0) + V(2, 0))) * 0.125f;
    if (s == 0)      put(inter, ip, x, y, c, g, d);
    else if (s == 1) put(inter, ip, x, y, hz, c, vt);
    else if (s == 2) put(inter, ip, x, y, vt, c, hz);
    else             put(inter, ip, x, y, d, g, c);
}

/* RCD, one kernel per sweep of reference lib/ref/ref_debayer.c:234-378. */
__global__ void p_rcd_lp(int w, int h, const float *v, float *lp)
{
    XY
    if (x >= w || y >= h)
        return;
    lp[(size_t)y * w + x] = (4.0f * V(0, 0) + 2.0f * (V(0, -1) + V(0, 1) + V(-1, 0) + V(1, 0))
                             + V(-1, -1) + V(1, -1) + V(-1, 1) + V(1, 1)) * (1.0f / 16.0f);
}

__global__ void p_rcd_dir(int w, int h, const float *v, float *ga, float *gb, int diag)
{
    XY
    if (x >= w || y >= h)
        return;
    size_t i = (size_t)y * w + x;
    float c2 = 2.0f * V(0, 0);
    if (!diag) {
        ga[i] = fabsf(V(0, -1) - V(0, 1)) + fabsf(c2 - V(0, -2) - V(0, 2));
        gb[i] = fabsf(V(-1, 0) - V(1, 0)) + fabsf(c2 - V(-2, 0) - V(2, 0));
    } else {
        ga[i] = fabsf(V(-1, 1) - V(1, -1)) + fabsf(c2 - V(-2, 2) - V(2, -2));
        gb[i] = fabsf(V(-1, -1) - V(1, 1)) + fabsf(c2 - V(-2, -2) - V(2, 2));
    }
}
#undef V

CRAW_DEV float box3(const float *s, int w, int h, int x, int y)
{
    float a = 0.0f;
    for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++)
            a += at(s, w, h, x + dx, y + dy);
    return a * (1.0f / 9.0f);
}

/* wv = hs / (hs + vs + eps) from (ga, gb) = (V, H); wp = qs / (ps + qs + eps)
 * from (ga, gb) = (P, Q). */
__global__ void p_rcd_weight(int w, int h, const float *ga, const float *gb, float *out, int diag)
{
    XY
    if (x >= w || y >= h)
        return;
    float a = box3(ga, w, h, x, y), b = box3(gb, w, h, x, y);
    out[(size_t)y * w + x] = diag ? b / (a + b + 1e-5f) : b / (b + a + 1e-5f);
}

CRAW_DEV float ratio(float a, float b)
{
    a = fmaxf(a, 0.0f);
    b = fmaxf(b, 0.0f);
    return (a - b) / (a + b + 1e-5f);
}

#define V(dx, dy) at(v, w, h, x + (dx), y + (dy))
#define L(dx, dy) at(lp, w, h, x + (dx), y + (dy))
#define G(dx, dy) at(gp, w, h, x + (dx), y + (dy))
#define C(dx, dy) at(cp, w, h, x + (dx), y + (dy))

__global__ void p_rcd_green(int w, int h, const float *v, const float *lp, const float *wv, float *gp)
{
    XY
    if (x >= w || y >= h)
        return;
    size_t i = (size_t)y * w + x;
    int s = (y & 1) * 2 + (x & 1);
    if (s == 1 || s == 2) {
        gp[i] = v[i];
        return;
    }
    float l00 = L(0, 0);
    float gv = 0.5f * (V(0, -1) * (1.0f + ratio(l00, L(0, -2))) + V(0, 1) * (1.0f + ratio(l00, L(0, 2))));
    float gh = 0.5f * (V(-1, 0) * (1.0f + ratio(l00, L(-2, 0))) + V(1, 0) * (1.0f + ratio(l00, L(2, 0))));
    gp[i] = wv[i] * gv + (1.0f - wv[i]) * gh;
}

__global__ void p_rcd_rb(int w, int h, const float *v, const float *gp, const float *wp,
                         float *cp, float *inter, size_t ip)
{
    XY
    if (x >= w || y >= h)
        return;
    size_t i = (size_t)y * w + x;
    int s = (y & 1) * 2 + (x & 1);
    if (s == 1 || s == 2)
        return;
    float g00 = gp[i], wt = wp[i];
    float c = wt * (g00 + 0.5f * ((V(-1, 1) - G(-1, 1)) + (V(1, -1) - G(1, -1))))
            + (1.0f - wt) * (g00 + 0.5f * ((V(-1, -1) - G(-1, -1)) + (V(1, 1) - G(1, 1))));
    cp[i] = c;
    if (s == 0) put(inter, ip, x, y, v[i], g00, c);
    else        put(inter, ip, x, y, c, g00, v[i]);
}

__global__ void p_rcd_g(int w, int h, const float *v, const float *gp, const float *cp,
                        const float *wv, float *inter, size_t ip)
{
    XY
    if (x >= w || y >= h)
        return;
    size_t i = (size_t)y * w + x;
    int s = (y & 1) * 2 + (x & 1);
    if (s == 0 || s == 3)
        return;
    float g00 = gp[i], wt = wv[i];
    float dh = 0.5f * ((V(-1, 0) - G(-1, 0)) + (V(1, 0) - G(1, 0)));
    float ev = 0.5f * ((C(0, -1) - G(0, -1)) + (C(0, 1) - G(0, 1)));
    float ch = wt * (g00 + ev) + (1.0f - wt) * (g00 + dh);
    float dv = 0.5f * ((V(0, -1) - G(0, -1)) + (V(0, 1) - G(0, 1)));
    float eh = 0.5f * ((C(-1, 0) - G(-1, 0)) + (C(1, 0) - G(1, 0)));
    float cv = wt * (g00 + dv) + (1.0f - wt) * (g00 + eh);
    if (s == 1) put(inter, ip, x, y, ch, v[i], cv);
    else        put(inter, ip, x, y, cv, v[i], ch);
}
#undef V
#undef L
#undef G
#undef C

/* ----------------------------------------------------------------- chroma */

__global__ void p_chroma_down(int w, int h, int qw, int qh, const float *inter, size_t ip, float *q)
{
    XY
    if (x >= qw || y >= qh)
        return;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, n = 0.f;
    for (int j = 0; j < 4; j++)
        for (int i = 0; i < 4; i++) {
            int px = 4 * x + i, py = 4 * y + j;
            if (px >= w || py >= h)
                continue;
            float4 p = reinterpret_cast<const float4 *>((const char *)inter + (size_t)py * ip)[px];
            s0 += p.x - p.y;
            s1 += p.z - p.y;
            s2 += p.y;
            n += 1.0f;
        }
    reinterpret_cast<float4 *>(q)[(size_t)y * qw + x] = make_float4(s0 / n, s1 / n, s2 / n, 0.f);
}

__global__ void p_chroma_blur(int qw, int qh, const float *q, float *qf)
{
    XY
    if (x >= qw || y >= qh)
        return;
    const float4 *Q = reinterpret_cast<const float4 *>(q);
    float4 c = Q[(size_t)y * qw + x];
    float level = fmaxf(c.z, 0.0f) + 0.02f;
    float ir = 1.0f / (0.35f * level), ic = 1.0f / (0.35f * level);
    float a0 = 0.f, a1 = 0.f, ws = 0.f;
    for (int dy = -4; dy <= 4; dy++)
        for (int dx = -4; dx <= 4; dx++) {
            float4 s = Q[(size_t)craw_mirror(y + dy, qh) * qw + craw_mirror(x + dx, qw)];
            float dg = (s.z - c.z) * ir, d0 = (s.x - c.x) * ic, d1 = (s.y - c.y) * ic;
            float wt = expf(-(float)(dx * dx + dy * dy) * 0.125f - dg * dg - d0 * d0 - d1 * d1);
            a0 += wt * s.x;
            a1 += wt * s.y;
            ws += wt;
        }
    reinterpret_cast<float4 *>(qf)[(size_t)y * qw + x] = make_float4(a0 / ws, a1 / ws, c.z, 0.f);
}

__global__ void p_chroma_up(int w, int h, int qw, int qh, float s, float *inter, size_t ip,
                            const float *q, const float *qf)
{
    XY
    if (x >= w || y >= h)
        return;
    const float4 *Q = reinterpret_cast<const float4 *>(q), *F = reinterpret_cast<const float4 *>(qf);
    float fy = ((float)y + 0.5f) * 0.25f - 0.5f, fly = floorf(fy), ty = fy - fly;
    float fx = ((float)x + 0.5f) * 0.25f - 0.5f, flx = floorf(fx), tx = fx - flx;
    int ya = min(max((int)fly, 0), qh - 1), yb = min(max((int)fly + 1, 0), qh - 1);
    int xa = min(max((int)flx, 0), qw - 1), xb = min(max((int)flx + 1, 0), qw - 1);
    float w00 = (1.0f - tx) * (1.0f - ty), w10 = tx * (1.0f - ty), w01 = (1.0f - tx) * ty, w11 = tx * ty;
    float4 d00 = Q[(size_t)ya * qw + xa], d10 = Q[(size_t)ya * qw + xb];
    float4 d01 = Q[(size_t)yb * qw + xa], d11 = Q[(size_t)yb * qw + xb];
    float4 b00 = F[(size_t)ya * qw + xa], b10 = F[(size_t)ya * qw + xb];
    float4 b01 = F[(size_t)yb * qw + xa], b11 = F[(size_t)yb * qw + xb];
    float4 *row = reinterpret_cast<float4 *>((char *)inter + (size_t)y * ip);
    float4 p = row[x];
    float g = p.y;
    float dr = p.x - g, db = p.z - g;
    dr += s * ((w00 * b00.x + w10 * b10.x + w01 * b01.x + w11 * b11.x) -
               (w00 * d00.x + w10 * d10.x + w01 * d01.x + w11 * d11.x));
    db += s * ((w00 * b00.y + w10 * b10.y + w01 * b01.y + w11 * b11.y) -
               (w00 * d00.y + w10 * d10.y + w01 * d01.y + w11 * d11.y));
    row[x] = make_float4(g + dr, g, g + db, 1.0f);
}

/* ----------------------------------------------------------- awb, colour */

__global__ void p_awb(const CRAWKDevelop k, const float *inter, size_t ip, uint32_t *hist,
                      const CRAWKAwbOut awb)
{
    XY
    const int bw = (k.width + 7) / 8, bh = (k.height + 7) / 8;
    if (x >= bw || y >= bh)
        return;
    const int xe = min(8, k.width - 8 * x), ye = min(8, k.height - 8 * y);
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
    for (int j = 0; j < ye; j++) {
        const float4 *row = reinterpret_cast<const float4 *>((const char *)inter + (size_t)(8 * y + j) * ip);
        for (int i = 0; i < xe; i++) {
            float4 p = row[8 * x + i];
            s0 = __fadd_rn(s0, p.x);
            s1 = __fadd_rn(s1, p.y);
            s2 = __fadd_rn(s2, p.z);
        }
    }
    float n = (float)(xe * ye);
    uint64_t r = craw_awb_block(__fdiv_rn(s0, n), __fdiv_rn(s1, n), __fdiv_rn(s2, n), k.awb_wb,
                                awb.deferred, awb.nb_deferred, craw_awb_blocks(k.width, k.height));
    if (r & CRAW_K_AWB_VALID) {
        uint32_t bin = (uint32_t)(r & 0x3fffu);
        atomicAdd(&hist[bin], 1u);
        atomicAdd(&hist[16384 + bin], (uint32_t)((r >> 14) & 0xffffu));
        atomicAdd(&hist[32768 + bin], (uint32_t)((r >> 30) & 0xffffu));
    }
}

__global__ void p_color(const CRAWKDevelop k, const float *inter, size_t ip, void *dst,
                        size_t dp, int half_fmt)
{
    XY
    if (x >= k.width || y >= k.height)
        return;
    float4 p = reinterpret_cast<const float4 *>((const char *)inter + (size_t)y * ip)[x];
    float in[3] = { p.x, p.y, p.z }, o[3];
    craw_color(k.color, in, o);
    craw_store_rgba(dst, dp, x, y, half_fmt, o[0], o[1], o[2]);
}

#define LAUNCH_OK (cudaGetLastError() == cudaSuccess ? 0 : -5)

} // namespace

extern "C" int craw_k_plain_denoise(const CRAWKDenoise *k, const CRAWKDenoiseIO *io,
                                    float *t, float *var, cudaStream_t s)
{
    if (craw_launch_ready() < 0)
        return -5;
    dim3 g(((k->pw + B2 - 1) / B2), (k->ph + B2 - 1) / B2, 4), b(B2, B2);
    const size_t plane = (size_t)4 * k->pw * k->ph;
    if (k->mode & CRAW_K_DN_HISTORY) {
        /* `var` holds 3 planes' worth: the variance, this frame, last frame. */
        float *cur = var + plane, *prv = var + 2 * plane;
        p_dn_vst<<<g, b, 0, s>>>(*k, *io, t, cur, prv);
        p_dn_temporal<<<g, b, 0, s>>>(*k, *io, t, cur, prv, var);
    } else {
        p_dn_vst<<<g, b, 0, s>>>(*k, *io, t, nullptr, nullptr);
    }
    p_dn_nlm<<<g, b, 0, s>>>(*k, *io, t, var);
    return LAUNCH_OK;
}

extern "C" int craw_k_plain_develop(const CRAWKDevelop *k, const CRAWKDevelopIO *io,
                                    const CRAWKChroma *chroma, float *v, float *inter,
                                    size_t ip, float *scratch, float *q, float *qf,
                                    uint32_t *hist, cudaStream_t s)
{
    if (craw_launch_ready() < 0)
        return -5;
    const int w = k->width, h = k->height;
    const size_t n = (size_t)w * h;
    p_prep<<<GRID2(w, h), 0, s>>>(*k, io->src, io->src_pitch, v);
    if (k->method == 0) {
        p_bilinear<<<GRID2(w, h), 0, s>>>(w, h, v, inter, ip);
    } else if (k->method == 1) {
        p_mhc<<<GRID2(w, h), 0, s>>>(w, h, v, inter, ip);
    } else {
        float *lp = scratch, *wv = scratch + n, *wp = scratch + 2 * n, *gp = scratch + 3 * n;
        float *cp = scratch + 4 * n, *ga = scratch + 5 * n, *gb = scratch + 6 * n;
        p_rcd_lp<<<GRID2(w, h), 0, s>>>(w, h, v, lp);
        p_rcd_dir<<<GRID2(w, h), 0, s>>>(w, h, v, ga, gb, 0);
        p_rcd_weight<<<GRID2(w, h), 0, s>>>(w, h, ga, gb, wv, 0);
        p_rcd_dir<<<GRID2(w, h), 0, s>>>(w, h, v, ga, gb, 1);
        p_rcd_weight<<<GRID2(w, h), 0, s>>>(w, h, ga, gb, wp, 1);
        p_rcd_green<<<GRID2(w, h), 0, s>>>(w, h, v, lp, wv, gp);
        p_rcd_rb<<<GRID2(w, h), 0, s>>>(w, h, v, gp, wp, cp, inter, ip);
        p_rcd_g<<<GRID2(w, h), 0, s>>>(w, h, v, gp, cp, wv, inter, ip);
    }
    if (chroma) {
        p_chroma_down<<<GRID2(chroma->qw, chroma->qh), 0, s>>>(w, h, chroma->qw, chroma->qh, inter, ip, q);
        p_chroma_blur<<<GRID2(chroma->qw, chroma->qh), 0, s>>>(chroma->qw, chroma->qh, q, qf);
        p_chroma_up<<<GRID2(w, h), 0, s>>>(w, h, chroma->qw, chroma->qh, chroma->strength, inter, ip, q, qf);
    }
    if (hist)
        p_awb<<<GRID2((w + 7) / 8, (h + 7) / 8), 0, s>>>(*k, inter, ip, hist, io->awb);
    if (io->dst)
        p_color<<<GRID2(w, h), 0, s>>>(*k, inter, ip, io->dst, io->dst_pitch, io->dst_fmt);
    return LAUNCH_OK;
}
