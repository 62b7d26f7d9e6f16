/*
 * Device helpers shared by the sm_103a kernels: borders, the prep, the
 * colour stage, the AWB block statistic and image stores.
 */
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

#include <atomic>

#include "../kabi.h"

#define CRAW_DEV __device__ __forceinline__

/* Index checks of the CRAW_DEBUG_BOUNDS build (the library built with
 * -DCRAW_DEBUG_BOUNDS=1 as _lib/libcraw_bounds.so): `ok` is the check of
 * an index against its buffer; a failed one sets CRAW_K_ERR_BOUNDS in the
 * kernel's error word `err` (when there is one) and the caller skips the
 * access, so that no fault, trap or hang follows. In the product build
 * the check is true and costs nothing. */
#if defined(CRAW_DEBUG_BOUNDS) && CRAW_DEBUG_BOUNDS
CRAW_DEV bool craw_in_bounds(bool ok, uint32_t *err)
{
    if (!ok && err)
        atomicOr(err, CRAW_K_ERR_BOUNDS);
    return ok;
}
#else
CRAW_DEV constexpr bool craw_in_bounds(bool, uint32_t *)
{
    return true;
}
#endif

/* 0, or -5 (EIO) when a CUDA error of an earlier call is pending on this
 * thread: it is the caller's to read, not ours to clear, and a launch now
 * could not tell its own error from it. Every launcher checks this first,
 * then reads (and so clears) only the error of its own launches. */
inline int craw_launch_ready()
{
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -5;
}

/* Lets `fn` take `bytes` of dynamic shared memory, once per device (the
 * attribute belongs to the function in each device's context); `done`
 * holds a bit per device ordinal below 64, above which it is set every
 * time. 0, or -5 when the runtime refuses. */
template <typename F>
inline int craw_smem_attr(F fn, size_t bytes, std::atomic<uint64_t> &done)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return -5;
    const uint64_t bit = dev >= 0 && dev < 64 ? (uint64_t)1 << dev : 0;
    if (bit && (done.load(std::memory_order_acquire) & bit))
        return 0;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
        return -5;
    done.fetch_or(bit, std::memory_order_release);
    return 0;
}

/* Item i of a W x H grid as (x, y). With W > 32 the first 32 H items take
 * 32 consecutive columns of one row each and the rest the W - 32 columns
 * left over, so that the items of a warp (block sizes a multiple of 32)
 * never wrap from one row to the next: a wrap lands the second row's
 * shared-memory words on banks the first row's half-warp already uses. */
template <int W, int H>
CRAW_DEV void craw_row_item(int i, int &x, int &y)
{
    if constexpr (W > 32) {
        if (i < 32 * H) {
            x = i & 31;
            y = i >> 5;
            return;
        }
        const int e = i - 32 * H;
        x = 32 + e % (W - 32);
        y = e / (W - 32);
    } else {
        x = i % W;
        y = i / W;
    }
}

/* Mirror without repeating the edge sample (reference common.glsl:49-55,
 * lib/ref/ref_debayer.c:21-34), looping for tiles that hang further past
 * a small frame than one reflection reaches. n >= 2. */
CRAW_DEV int craw_mirror(int v, int n)
{
    while (v < 0 || v >= n) {
        if (v < 0)
            v = -v;
        if (v >= n)
            v = 2 * n - 2 - v;
    }
    return v;
}

/* The prep of one raw sample at quad site s (reference
 * lib/ref/ref_debayer.c:42-63): UNORM, above black in units of the
 * site's range, times the gain of its channel, clipped at 1.0. */
CRAW_DEV float craw_prep(const CRAWKDevelop &k, uint16_t raw, int s)
{
    float r = (float)raw * (1.0f / 65535.0f);
    float t = (r - k.black[s]) * k.inv_range[s] * k.wbs[s];
    return t < k.clip ? t : k.clip;
}

/* 2^x on the MUFU. */
CRAW_DEV float craw_ex2(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

/* Two fp32 lanes in one 64-bit register, for the sm_100 family's packed
 * f32x2 add / sub / mul / fma (one instruction for two columns, the same
 * IEEE rounding per lane as the scalar forms). */
typedef unsigned long long f2x;

CRAW_DEV f2x f2_pack(float lo, float hi)
{
    f2x r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
CRAW_DEV float f2_lo(f2x a)
{
    return __uint_as_float((uint32_t)a);
}
CRAW_DEV float f2_hi(f2x a)
{
    return __uint_as_float((uint32_t)(a >> 32));
}
CRAW_DEV f2x f2_add(f2x a, f2x b)
{
    f2x d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
CRAW_DEV f2x f2_sub(f2x a, f2x b)
{
    f2x d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
CRAW_DEV f2x f2_mul(f2x a, f2x b)
{
    f2x d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
CRAW_DEV f2x f2_fma(f2x a, f2x b, f2x c)
{
    f2x d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
CRAW_DEV f2x f2_ld(const float *p)   /* p 8-byte aligned */
{
    return *reinterpret_cast<const f2x *>(p);
}

CRAW_DEV float craw_round_half(float x)
{
    return __half2float(__float2half_rn(x));
}

/* ACES 1.3 reference gamut compression of one AP1 triple (reference
 * lib/gamut.c:61-92; a channel below its threshold is left untouched). */
CRAW_DEV void craw_gamut_compress(const CRAWKColor &c, float o[3])
{
    float ach = fmaxf(o[0], fmaxf(o[1], o[2]));
    if (ach == 0.0f)
        return;
    float mag = fabsf(ach), inv_mag = 1.0f / mag;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float d = (ach - o[i]) * inv_mag;
        if (d < c.gc_thr[i])
            continue;
        float nd = (d - c.gc_thr[i]) / c.gc_scl[i];
        float p = __powf(nd, c.gc_pwr);
        d = c.gc_thr[i] + c.gc_scl[i] * nd * __powf(1.0f + p, -c.gc_inv_pwr);
        o[i] = ach - d * mag;
    }
}

/* Matrix, gain and exposure to the output space, then the optional
 * compression and clamp (reference lib/shaders/color.comp.glsl:72-91). */
CRAW_DEV void craw_color(const CRAWKColor &c, const float in[3], float o[3])
{
#pragma unroll
    for (int r = 0; r < 3; r++)
        o[r] = c.m[r][0] * in[0] + c.m[r][1] * in[1] + c.m[r][2] * in[2];
    if (c.flags & CRAW_K_COLOR_RGC)
        craw_gamut_compress(c, o);
    if (c.flags & CRAW_K_COLOR_CLAMP) {
#pragma unroll
        for (int r = 0; r < 3; r++)
            o[r] = fmaxf(o[r], 0.0f);
    }
}

/* Pixel (x, y) of an RGB image of layout `fmt` (CRAW_K_OUT_*: 0 four
 * floats, 1 four half floats, 2 three floats). */
CRAW_DEV void craw_store_rgba(void *base, size_t pitch, int x, int y, int fmt,
                              float r, float g, float b)
{
    char *row = (char *)base + (size_t)y * pitch;
    if (fmt == CRAW_K_OUT_RGB32F) {
        float *p = reinterpret_cast<float *>(row) + 3 * (size_t)x;
        p[0] = r;
        p[1] = g;
        p[2] = b;
    } else if (fmt == CRAW_K_OUT_RGBA16F) {
        __half2 lo = __floats2half2_rn(r, g), hi = __floats2half2_rn(b, 1.0f);
        uint2 v;
        v.x = *reinterpret_cast<uint32_t *>(&lo);
        v.y = *reinterpret_cast<uint32_t *>(&hi);
        reinterpret_cast<uint2 *>(row)[x] = v;
    } else {
        reinterpret_cast<float4 *>(row)[x] = make_float4(r, g, b, 1.0f);
    }
}

CRAW_DEV void craw_load_rgb(const void *base, size_t pitch, int x, int y, int half_fmt,
                            float o[3])
{
    const char *row = (const char *)base + (size_t)y * pitch;
    if (half_fmt) {
        uint2 v = reinterpret_cast<const uint2 *>(row)[x];
        __half2 lo = *reinterpret_cast<__half2 *>(&v.x), hi = *reinterpret_cast<__half2 *>(&v.y);
        float2 a = __half22float2(lo), b = __half22float2(hi);
        o[0] = a.x; o[1] = a.y; o[2] = b.x;
    } else {
        float4 v = reinterpret_cast<const float4 *>(row)[x];
        o[0] = v.x; o[1] = v.y; o[2] = v.z;
    }
}

/* The frame's 8x8 blocks: a deferred-block list this long never fills. */
CRAW_DEV uint32_t craw_awb_blocks(int w, int h)
{
    return (uint32_t)((w + 7) / 8) * (uint32_t)((h + 7) / 8);
}

/* The AWB statistic of one block from its mean (reference
 * lib/awb.c:255-291, whose operation order is kept so that the bins and
 * weights are the CPU builder's bit for bit): skip clipped and near-black
 * blocks, divide the gains back out, bin ln(R/G), ln(B/G) over
 * [-2.5, 1] in 128 bins, weights min(g, 0.5) and g^4 in 16.16.
 *
 * The logarithm is CUDA's logf (within 1 ulp, as the host's is): the two
 * can differ by 2 ulp of ln(R/G), i.e. at most 2e-5 of a bin, so a block
 * whose bin position lies within 2e-4 of a bin edge, where the two could
 * choose different bins, is deferred to the host instead; every other
 * block lands in the host's bin. (GB300's FP64 rate is a small fraction
 * of its FP32 rate, so a double-precision log would cost more than the
 * whole block sum.) */
CRAW_DEV uint64_t craw_awb_block(float r, float g, float b, const float wb[3],
                                 CRAWKAwbDeferred *deferred, uint32_t *nb_deferred, uint32_t cap)
{
    const float lmin = -2.5f, lmax = 1.0f, span = lmax - lmin;
    if (fmaxf(fmaxf(r, g), b) >= 0.98f || g < 0.002f)
        return 0;
    float rr = __fdiv_rn(__fdiv_rn(r, wb[0]), g);
    float bb = __fdiv_rn(__fdiv_rn(b, wb[2]), g);
    float x = logf(rr), y = logf(bb);
    x = x > lmin ? (x < lmax ? x : lmax) : lmin;
    y = y > lmin ? (y < lmax ? y : lmax) : lmin;
    float fx = __fmul_rn(__fdiv_rn(__fsub_rn(x, lmin), span), 128.0f);
    float fy = __fmul_rn(__fdiv_rn(__fsub_rn(y, lmin), span), 128.0f);
    /* Edges at 0 and 128 cannot flip: the bin index is clamped there. */
    const float rx = rintf(fx), ry = rintf(fy);
    const bool near_x = rx >= 1.0f && rx <= 127.0f && fabsf(fx - rx) < 2e-4f;
    const bool near_y = ry >= 1.0f && ry <= 127.0f && fabsf(fy - ry) < 2e-4f;
    if (deferred && (near_x || near_y)) {
        uint32_t i = atomicAdd(nb_deferred, 1u);
        if (i < cap) {
            CRAWKAwbDeferred d;
            d.rr = rr; d.bb = bb; d.g = g; d.pad = 0;
            deferred[i] = d;
            return 0;
        }
    }
    int ix = (int)floorf(fx), iy = (int)floorf(fy);
    ix = ix < 0 ? 0 : (ix > 127 ? 127 : ix);
    iy = iy < 0 ? 0 : (iy > 127 ? 127 : iy);
    float w = g < 0.5f ? g : 0.5f;
    uint32_t wq = (uint32_t)roundf(__fmul_rn(w, 65536.0f));
    uint32_t bq = (uint32_t)roundf(__fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(g, g), g), g), 65536.0f));
    return CRAW_K_AWB_VALID | (uint64_t)(iy * 128 + ix) | ((uint64_t)wq << 14) | ((uint64_t)bq << 30);
}
