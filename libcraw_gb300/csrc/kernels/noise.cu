/*
 * Noise-model estimation, the device half (reference lib/noise.c:338-504,
 * binning 396-450; the least-trimmed-squares seed 187-250).
 *
 *   k_noise_lut     the four sites' plane values of every 16-bit code, in
 *                   double and rounded once, as the reference converts
 *   k_noise_bin     per CTA a 32x8 patch of interior plane positions of
 *                   all four planes: the 3x3 high-pass and the 9x9 mean
 *                   (81 float additions in the reference's order), the
 *                   bin, per-bin counts and exact sums of the means, and
 *                   a first histogram of |high-pass| per bin (its top 11
 *                   bits)
 *   k_noise_select  per bin, which bucket holds the (count / 2)-th
 *                   smallest |high-pass|; two more rounds over the next
 *                   10 and last 10 bits (k_noise_refine) leave its bits
 *   k_noise_lts     the trimmed cost of every pair of bins, one warp each
 *
 * The median is an order statistic, so it is the reference's value
 * exactly; so are the counts. A bin's sum of means is kept as an integer
 * (each float mean times 2^64, exact for means >= 2^-40, in three 32-bit
 * words) so that it does not depend on the order the atomics land in;
 * the reference adds the same floats into a double one by one. Built
 * without multiply-add contraction, as the reference's host code is.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "common.cuh"

namespace {

constexpr int kR = 4;                                   /* radius of the plane mean */
constexpr int kTX = 32, kTY = 8, kThreads = kTX * kTY;  /* outputs of a CTA, per plane */
constexpr int kSX = kTX + 2 * kR, kSY = kTY + 2 * kR;   /* staged plane patch: 40 x 16 */
constexpr int kSP = kSX + 1;                            /* its row pitch */
constexpr int kB1 = 2048, kB2 = 1024, kB3 = 1024;       /* buckets: key bits 30-20, 19-10, 9-0 */
constexpr uint16_t kNoBin = 0xffff;

struct Layout {
    size_t lut, h1, h2, h3, sel, keys, bidx, total;
};

Layout layout(int32_t w, int32_t h, int32_t nb)
{
    const size_t n = (size_t)4 * (size_t)(w / 2 - 2 * kR) * (size_t)(h / 2 - 2 * kR);
    Layout L;
    size_t o = 0;
    auto take = [&o](size_t bytes) {
        const size_t at = o;
        o = (o + bytes + 255) / 256 * 256;
        return at;
    };
    L.lut = take((size_t)4 * 65536 * sizeof(float));
    L.h1 = take((size_t)nb * kB1 * 4);
    L.h2 = take((size_t)nb * kB2 * 4);
    L.h3 = take((size_t)nb * kB3 * 4);
    L.sel = take((size_t)nb * 8);
    L.keys = take(n * 4);
    L.bidx = take(n * 2);
    L.total = o;
    return L;
}

__global__ void k_noise_lut(CRAWKNoise k, float *lut)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 4 * 65536)
        return;
    const int s = t >> 16, raw = t & 0xffff;
    const float range = k.white[s] - k.black[s];          /* float, as the reference */
    const double v = ((double)raw * (1.0 / 65535.0) - (double)k.black[s]) / (double)range;
    lut[t] = (float)v;
}

/* A positive float (below 2^31) times 2^64 as a 96-bit integer, in three
 * 32-bit words, truncated below 2^-64. f = m 2^(e - 150), m < 2^24. */
__device__ __forceinline__ void fixed96(float f, uint32_t w[3])
{
    const uint32_t b = __float_as_uint(f);
    const int e = (int)(b >> 23);
    const uint64_t m = (uint64_t)((b & 0x7fffffu) | 0x800000u);
    const int sh = e - 86;
    uint64_t lo = 0;
    uint32_t hi = 0;
    if (e == 0 || sh <= -24) {
    } else if (sh < 0) {
        lo = m >> -sh;
    } else if (sh <= 40) {
        lo = m << sh;
    } else if (sh < 64) {
        lo = m << sh;
        hi = (uint32_t)(m >> (64 - sh));
    } else {
        hi = (uint32_t)(m << (sh - 64));
    }
    w[0] = (uint32_t)lo;
    w[1] = (uint32_t)(lo >> 32);
    w[2] = hi;
}

/* One sample, p its staged plane value, of a warp all of whose lanes call
 * this together: the 3x3 high-pass, the bin, the record (keys, bidx at o
 * when inside), the CTA's per-bin tallies and the first histogram. */
__device__ __forceinline__ void bin_sample(const CRAWKNoise &k, const float *p, float mean, bool inside, size_t o,
                                           uint32_t *cnt_s, unsigned long long (*sum_s)[CRAW_K_NOISE_MAX_BINS],
                                           uint32_t *h1, uint32_t *keys, uint16_t *bidx)
{
    /* [1 -2 1; -2 4 -2; 1 -2 1] / 6, in the reference's order. */
    const float hp = (p[-kSP - 1] + p[-kSP + 1] + p[kSP - 1] + p[kSP + 1] -
                      2.0f * (p[-kSP] + p[kSP] + p[-1] + p[1]) + 4.0f * p[0]) * (1.0f / 6.0f);
    int bin = -1;
    uint32_t key = 0, f[3] = { 0, 0, 0 };
    if (inside && mean > 0.0f && !(mean > k.max_level)) {
        bin = (int)(sqrtf(mean) * (float)k.nb_bins);
        bin = bin < 0 ? 0 : (bin > k.nb_bins - 1 ? k.nb_bins - 1 : bin);
        key = __float_as_uint(fabsf(hp));
        fixed96(mean, f);
    }
    /* Neighbouring samples mostly share a bin: the lanes of a bin add
     * their counts and sums first (each 32-bit word as two 16-bit halves,
     * which cannot overflow over 32 lanes), then one lane adds them into
     * the CTA's tallies. */
    const unsigned grp = __match_any_sync(0xffffffffu, bin);
    uint64_t tot[3];
#pragma unroll
    for (int q = 0; q < 3; q++)
        tot[q] = (uint64_t)__reduce_add_sync(grp, f[q] & 0xffffu) +
                 ((uint64_t)__reduce_add_sync(grp, f[q] >> 16) << 16);
    if (bin >= 0 && (threadIdx.x & 31) == __ffs(grp) - 1) {
        atomicAdd(&cnt_s[bin], (uint32_t)__popc(grp));
#pragma unroll
        for (int q = 0; q < 3; q++)
            if (tot[q])
                atomicAdd(&sum_s[q][bin], (unsigned long long)tot[q]);
    }
    if (inside) {
        keys[o] = key;
        bidx[o] = bin < 0 ? kNoBin : (uint16_t)bin;
    }
    /* One atomic per distinct bucket of the warp. */
    const uint32_t addr = bin < 0 ? 0xffffffffu : (uint32_t)bin * kB1 + (key >> 20);
    const unsigned same = __match_any_sync(0xffffffffu, addr);
    if (addr != 0xffffffffu && (threadIdx.x & 31) == __ffs(same) - 1)
        atomicAdd(&h1[addr], (uint32_t)__popc(same));
}

__global__ void __launch_bounds__(kThreads)
k_noise_bin(const CRAWKNoise k, const uint16_t *src, size_t pitch, const float *lut, uint32_t *h1,
            uint32_t *keys, uint16_t *bidx, CRAWKNoiseBin *bins)
{
    __shared__ __align__(16) float P[4][kSY][kSP];
    __shared__ uint32_t cnt_s[CRAW_K_NOISE_MAX_BINS];
    __shared__ unsigned long long sum_s[3][CRAW_K_NOISE_MAX_BINS];
    const int w2 = k.width / 2, h2 = k.height / 2;
    const int ww = w2 - 2 * kR, hh = h2 - 2 * kR;
    const int i0 = blockIdx.x * kTX, k0 = blockIdx.y * kTY;   /* first output; plane (k0 + kR, i0 + kR) */
    const int tid = threadIdx.x;

    for (int b = tid; b < k.nb_bins; b += kThreads) {
        cnt_s[b] = 0;
        sum_s[0][b] = sum_s[1][b] = sum_s[2][b] = 0;
    }
    /* The patch: plane rows k0 .. k0 + kSY, columns i0 .. i0 + kSX, i.e.
     * mosaic rows 2 kp + py and the 32-bit pair at column 2 ip of each. */
    constexpr int kLoads = kSY * kSX * 2, kIt = (kLoads + kThreads - 1) / kThreads;
    uint32_t pr[kIt];
#pragma unroll
    for (int it = 0; it < kIt; it++) {
        const int t = tid + it * kThreads, py = t / (kSY * kSX), rem = t - py * (kSY * kSX);
        const int r = rem / kSX, c = rem - r * kSX;
        pr[it] = 0;
        if (t < kLoads && k0 + r < h2 && i0 + c < w2)
            pr[it] = __ldg(reinterpret_cast<const uint32_t *>(
                (const char *)src + (size_t)(2 * (k0 + r) + py) * pitch) + i0 + c);
    }
#pragma unroll
    for (int it = 0; it < kIt; it++) {
        const int t = tid + it * kThreads, py = t / (kSY * kSX), rem = t - py * (kSY * kSX);
        const int r = rem / kSX, c = rem - r * kSX;
        if (t < kLoads) {
            P[2 * py][r][c] = __ldg(lut + (2 * py) * 65536 + (pr[it] & 0xffffu));
            P[2 * py + 1][r][c] = __ldg(lut + (2 * py + 1) * 65536 + (pr[it] >> 16));
        }
    }
    __syncthreads();

    /* One output a thread a plane; the 81-term mean in the reference's
     * order (rows, then columns). A variant with two columns a thread in
     * f32x2 adds ran slower (more registers, fewer CTAs a SM). */
    const int tx = tid % kTX, ty = tid / kTX;
    const int io = i0 + tx, ko = k0 + ty;
#pragma unroll 1
    for (int s = 0; s < 4; s++) {
        float mean = 0.0f;
#pragma unroll
        for (int dy = 0; dy <= 2 * kR; dy++)
#pragma unroll
            for (int dx = 0; dx <= 2 * kR; dx++)
                mean += P[s][ty + dy][tx + dx];
        bin_sample(k, &P[s][ty + kR][tx + kR], mean * (1.0f / 81), io < ww && ko < hh,
                   ((size_t)s * hh + ko) * ww + io, cnt_s, sum_s, h1, keys, bidx);
    }
    __syncthreads();
    for (int b = tid; b < k.nb_bins; b += kThreads)
        if (cnt_s[b]) {
            atomicAdd(&bins[b].count, cnt_s[b]);
#pragma unroll
            for (int q = 0; q < 3; q++)
                atomicAdd(reinterpret_cast<unsigned long long *>(&bins[b].sum[q]), sum_s[q][b]);
        }
}

/* Level 2 or 3: the samples whose key agrees with their bin's prefix so
 * far, counted by their next 10 bits. Four samples a thread a step. */
template <int LEVEL>
__global__ void __launch_bounds__(256)
k_noise_refine(const uint32_t *keys, const uint16_t *bidx, size_t n, const uint2 *sel, uint32_t *hist)
{
    const size_t n4 = n / 4;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    auto one = [&](uint32_t key, uint32_t b) {
        if (b == kNoBin)
            return;
        const uint32_t pre = sel[b].x;
        if (LEVEL == 2 ? (key >> 20) == pre : (key >> 10) == pre)
            atomicAdd(&hist[b * 1024 + (LEVEL == 2 ? (key >> 10) & 1023 : key & 1023)], 1u);
    };
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += stride) {
        const uint4 kk = __ldg(reinterpret_cast<const uint4 *>(keys) + q);
        const uint2 bb = __ldg(reinterpret_cast<const uint2 *>(bidx) + q);
        one(kk.x, bb.x & 0xffffu);
        one(kk.y, bb.x >> 16);
        one(kk.z, bb.y & 0xffffu);
        one(kk.w, bb.y >> 16);
    }
    for (size_t o = n4 * 4 + (size_t)blockIdx.x * blockDim.x + threadIdx.x; o < n; o += stride)
        one(keys[o], bidx[o]);
}

/* One warp per bin: the bucket of `hist` holding the bin's rank-th
 * smallest key (rank = count / 2 at level 1, then what is left of it
 * inside the chosen bucket); sel = (key prefix, remaining rank). */
__global__ void k_noise_select(int level, const uint32_t *hist, int nbuckets, uint2 *sel,
                               CRAWKNoiseBin *bins)
{
    const int b = blockIdx.x, lane = threadIdx.x;
    const uint32_t cnt = bins[b].count;
    if (cnt == 0) {
        if (lane == 0 && level == 3)
            bins[b].median = 0;
        return;
    }
    const uint32_t rank = level == 1 ? cnt / 2 : sel[b].y;
    const uint32_t *h = hist + (size_t)b * nbuckets;
    const int per = nbuckets / 32;
    uint32_t sum = 0;
    for (int j = 0; j < per; j++)
        sum += h[lane * per + j];
    uint32_t incl = sum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d)
            incl += o;
    }
    const unsigned past = __ballot_sync(0xffffffffu, incl > rank);
    if (lane != __ffs(past) - 1)
        return;
    uint32_t r = rank - (incl - sum);
    int j = 0;
    for (; j < per - 1 && r >= h[lane * per + j]; j++)
        r -= h[lane * per + j];
    const uint32_t bucket = (uint32_t)(lane * per + j);
    const uint32_t prefix = level == 1 ? bucket : (sel[b].x << 10) | bucket;
    sel[b] = make_uint2(prefix, r);
    if (level == 3)
        bins[b].median = prefix;
}

/* One warp per pair (i = blockIdx.x, j = blockIdx.y * 8 + warp): the
 * residuals of the line through bins i and j, sorted ascending in shared
 * memory (bitonic), the `keep` smallest added in order by one lane. */
constexpr int kLtsWarps = 8;

__global__ void __launch_bounds__(32 * kLtsWarps)
k_noise_lts(const double *m, const double *v, const double *lv, int nb, int np2, int keep, double *cost)
{
    __shared__ double d2[kLtsWarps][CRAW_K_NOISE_MAX_BINS];
    const int warp = threadIdx.x / 32, lane = threadIdx.x & 31;
    const int i = blockIdx.x, j = blockIdx.y * kLtsWarps + warp;
    if (j <= i || j >= nb)
        return;                                      /* whole warps only */
    double *w = d2[warp];
    const double dm = m[j] - m[i];
    double a = 0.0, b = 0.0;
    bool ok = !(dm < 1e-5);
    if (ok) {
        a = (v[j] - v[i]) / dm;
        b = v[i] - a * m[i];
        ok = a > 0.0 && !(b < 0.0);
    }
    if (!ok) {
        if (lane == 0)
            cost[(size_t)i * nb + j] = INFINITY;
        return;
    }
    for (int t = lane; t < np2; t += 32) {
        double d = INFINITY;
        if (t < nb) {
            d = lv[t] - log(a * m[t] + b);
            d = d * d;
        }
        w[t] = d;
    }
    __syncwarp();
    for (int size = 2; size <= np2; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = lane; t < np2 / 2; t += 32) {
                const int lo = 2 * t - (t & (stride - 1)), hi = lo + stride;
                const bool up = (lo & size) == 0;
                const double x = w[lo], y = w[hi];
                if ((x > y) == up) {
                    w[lo] = y;
                    w[hi] = x;
                }
            }
            __syncwarp();
        }
    if (lane == 0) {
        double c = 0.0;
        for (int t = 0; t < keep; t++)
            c += w[t];
        cost[(size_t)i * nb + j] = c;
    }
}

} // namespace

extern "C" size_t craw_k_noise_scratch(int32_t width, int32_t height, int32_t nb_bins)
{
    return layout(width, height, nb_bins).total;
}

extern "C" int craw_k_noise_bins(const CRAWKNoise *k, const uint16_t *src, size_t src_pitch, void *scratch,
                                 CRAWKNoiseBin *bins, cudaStream_t s)
{
    if (craw_launch_ready() < 0)
        return -5;
    const Layout L = layout(k->width, k->height, k->nb_bins);
    char *base = static_cast<char *>(scratch);
    float *lut = reinterpret_cast<float *>(base + L.lut);
    uint32_t *h1 = reinterpret_cast<uint32_t *>(base + L.h1);
    uint32_t *h2 = reinterpret_cast<uint32_t *>(base + L.h2);
    uint32_t *h3 = reinterpret_cast<uint32_t *>(base + L.h3);
    uint2 *sel = reinterpret_cast<uint2 *>(base + L.sel);
    uint32_t *keys = reinterpret_cast<uint32_t *>(base + L.keys);
    uint16_t *bidx = reinterpret_cast<uint16_t *>(base + L.bidx);
    const int ww = k->width / 2 - 2 * kR, hh = k->height / 2 - 2 * kR;
    const size_t n = (size_t)4 * ww * hh;

    if (cudaMemsetAsync(base + L.h1, 0, L.keys - L.h1, s) != cudaSuccess ||
        cudaMemsetAsync(bins, 0, (size_t)k->nb_bins * sizeof(CRAWKNoiseBin), s) != cudaSuccess)
        return -5;
    k_noise_lut<<<4 * 65536 / 256, 256, 0, s>>>(*k, lut);
    k_noise_bin<<<dim3((ww + kTX - 1) / kTX, (hh + kTY - 1) / kTY), kThreads, 0, s>>>(
        *k, src, src_pitch, lut, h1, keys, bidx, bins);
    k_noise_select<<<k->nb_bins, 32, 0, s>>>(1, h1, kB1, sel, bins);
    const int grid = 152 * 8;
    k_noise_refine<2><<<grid, 256, 0, s>>>(keys, bidx, n, sel, h2);
    k_noise_select<<<k->nb_bins, 32, 0, s>>>(2, h2, kB2, sel, bins);
    k_noise_refine<3><<<grid, 256, 0, s>>>(keys, bidx, n, sel, h3);
    k_noise_select<<<k->nb_bins, 32, 0, s>>>(3, h3, kB3, sel, bins);
    return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

extern "C" int craw_k_noise_lts(const double *m, const double *v, const double *lv, int32_t nb, int32_t keep,
                                double *cost, cudaStream_t s)
{
    if (craw_launch_ready() < 0)
        return -5;
    if (nb < 2 || nb > CRAW_K_NOISE_MAX_BINS)
        return -22;
    int np2 = 32;
    while (np2 < nb)
        np2 <<= 1;
    k_noise_lts<<<dim3(nb, (nb + kLtsWarps - 1) / kLtsWarps), 32 * kLtsWarps, 0, s>>>(m, v, lv, nb, np2, keep,
                                                                                      cost);
    return cudaGetLastError() == cudaSuccess ? 0 : -5;
}
