/*
 * The AWB histogram of an RGB image that is already on the device, built
 * without allocating anything: the variant of the pipeline's AWB block
 * pass whose scratch (the three histograms, a counter and the list of
 * blocks the host bins) is one file-scope __device__ array of fixed size
 * instead of memory the pipeline allocates at creation.
 *
 * Block statistic and binning follow reference lib/awb.c:255-291 (the CPU
 * builder craw_awb_histogram_from_rgb); blocks whose bin position lies
 * within 2e-4 of an interior bin edge are binned on the host with its own
 * logf, so the histogram equals the CPU builder's bit for bit.
 */
#include <cuda_runtime.h>
#include <errno.h>
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>

extern "C" {
#include <craw/awb.h>
#include <craw/craw.h>

void craw_awb_bin_host(float rr, float bb, float g, uint32_t *count, uint32_t *weight,
                       uint32_t *weight_bright);
}

namespace {

constexpr uint32_t kBins2 = CRAW_AWB_HIST_BINS * CRAW_AWB_HIST_BINS;
constexpr uint32_t kMaxBlocks = CRAW_AWB_NOALLOC_MAX_BLOCKS;

/* Word layout of the scratch:
 *   [0, 3 * kBins2)           count, weight and weight_bright histograms
 *   [3 * kBins2]              number of deferred blocks
 *   [kDeferred, +3 * kMax)    deferred blocks, (rr, bb, g) as float bits
 * The histograms and the counter must be zero when the kernel starts;
 * every call clears them on its stream before the launch. The deferred
 * entries need no clearing: only the first `counter` of them are read. */
constexpr uint32_t kCounter = 3 * kBins2;
constexpr uint32_t kDeferred = kCounter + 64;           /* 256-byte aligned */
constexpr uint32_t kWords = kDeferred + 3 * kMaxBlocks;

} // namespace

/* 3.3 MB: the whole of the entry point's device memory. */
static __device__ __align__(256) uint32_t awb_noalloc_scratch[kWords];

namespace {

/* One thread per 8x8 block; a CTA covers 32 x 8 blocks. */
__global__ void __launch_bounds__(256)
k_awb_noalloc(const float *rgb, int w, int h, size_t stride, int ch, float wb0, float wb2,
              uint32_t *sc)
{
    const int nbx = (w + 7) / 8, nby = (h + 7) / 8;
    const int bx = blockIdx.x * 32 + (threadIdx.x & 31);
    const int by = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (bx >= nbx || by >= nby)
        return;
    const int x0 = bx * 8, y0 = by * 8;
    const int x1 = min(x0 + 8, w), y1 = min(y0 + 8, h);
    /* Row by row, left to right, over the pixels that exist: the CPU
     * builder's summation order, so the block means are its own. */
    float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f;
    for (int y = y0; y < y1; y++) {
        const float *row = rgb + (size_t)y * stride;
        for (int x = x0; x < x1; x++) {
            const float *p = row + (size_t)x * ch;
            s0 = __fadd_rn(s0, p[0]);
            s1 = __fadd_rn(s1, p[1]);
            s2 = __fadd_rn(s2, p[2]);
        }
    }
    const float n = (float)((y1 - y0) * (x1 - x0));
    const float r = __fdiv_rn(s0, n), g = __fdiv_rn(s1, n), b = __fdiv_rn(s2, n);
    float mx = r > g ? r : g;
    mx = mx > b ? mx : b;
    if (mx >= 0.98f || g < 0.002f)
        return;
    const float rr = __fdiv_rn(__fdiv_rn(r, wb0), g);
    const float bb = __fdiv_rn(__fdiv_rn(b, wb2), g);

    const float lmin = CRAW_AWB_HIST_LOG_MIN, lmax = CRAW_AWB_HIST_LOG_MAX, span = lmax - lmin;
    /* ln in double rounded once: the correctly rounded float logarithm. A
     * NaN (a negative mean) lands in the first bin, as on the CPU. */
    float x = (float)log((double)rr), y = (float)log((double)bb);
    x = x > lmin ? (x < lmax ? x : lmax) : lmin;
    y = y > lmin ? (y < lmax ? y : lmax) : lmin;
    const float fx = __fmul_rn(__fdiv_rn(__fsub_rn(x, lmin), span), (float)CRAW_AWB_HIST_BINS);
    const float fy = __fmul_rn(__fdiv_rn(__fsub_rn(y, lmin), span), (float)CRAW_AWB_HIST_BINS);
    const float rx = rintf(fx), ry = rintf(fy);
    const bool near_x = rx >= 1.0f && rx <= CRAW_AWB_HIST_BINS - 1.0f && fabsf(fx - rx) < 2e-4f;
    const bool near_y = ry >= 1.0f && ry <= CRAW_AWB_HIST_BINS - 1.0f && fabsf(fy - ry) < 2e-4f;
    if (near_x || near_y) {
        /* At most one entry per block, and the host let through no more
         * blocks than kMaxBlocks: the index stays in the list. */
        const uint32_t i = atomicAdd(&sc[kCounter], 1u);
        uint32_t *d = sc + kDeferred + 3 * i;
        d[0] = __float_as_uint(rr);
        d[1] = __float_as_uint(bb);
        d[2] = __float_as_uint(g);
        return;
    }
    int ix = (int)floorf(fx), iy = (int)floorf(fy);
    ix = ix < 0 ? 0 : (ix > CRAW_AWB_HIST_BINS - 1 ? CRAW_AWB_HIST_BINS - 1 : ix);
    iy = iy < 0 ? 0 : (iy > CRAW_AWB_HIST_BINS - 1 ? CRAW_AWB_HIST_BINS - 1 : iy);
    const float wt = g < 0.5f ? g : 0.5f;
    const uint32_t wq = (uint32_t)roundf(__fmul_rn(wt, 65536.0f));
    const uint32_t bq = (uint32_t)roundf(__fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(g, g), g), g), 65536.0f));
    const uint32_t bin = (uint32_t)(iy * CRAW_AWB_HIST_BINS + ix);
    atomicAdd(&sc[bin], 1u);
    atomicAdd(&sc[kBins2 + bin], wq);
    atomicAdd(&sc[2 * kBins2 + bin], bq);
}

/* The host side of a call's copies: the histograms and the counter, then
 * the deferred blocks a chunk at a time, through one page-locked area per
 * device. Copies into page-locked memory are asynchronous, so the call
 * makes none of the implicitly synchronising copies (pageable host
 * memory) that another thread's global-mode stream capture forbids. */
constexpr uint32_t kChunk = 1024;                       /* deferred blocks a copy */
constexpr size_t kStageWords = kCounter + 1 > 3 * kChunk ? kCounter + 1 : 3 * kChunk;
constexpr size_t kStageBytes = (kStageWords * sizeof(uint32_t) + 4095) & ~(size_t)4095;

/* Set up on the first call on each device and kept: the scratch's device
 * address (cudaGetSymbolAddress with that device current) and the staging
 * area (host memory registered with cudaHostRegister). A set-up that fails
 * keeps nothing, so the next call tries again. */
constexpr int kMaxDevices = 64;
std::mutex setup_lock;
uint32_t *setup_ptr[kMaxDevices];
uint32_t *stage_ptr[kMaxDevices];

int setup(uint32_t **sc, uint32_t **stage)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return CRAW_ERROR(ENODEV);
    std::lock_guard<std::mutex> lock(setup_lock);
    if (!setup_ptr[dev]) {
        void *p = nullptr;
        const cudaError_t err = cudaGetSymbolAddress(&p, awb_noalloc_scratch);
        if (err != cudaSuccess) {
            (void)cudaGetLastError();   /* this lookup's own error */
            craw_log(NULL, CRAW_LOG_ERROR, "craw_awb_histogram_from_rgb_cuda_noalloc: "
                     "cudaGetSymbolAddress failed on device %d: %s\n", dev, cudaGetErrorString(err));
            return CRAW_ERROR(EIO);
        }
        setup_ptr[dev] = static_cast<uint32_t *>(p);
    }
    if (!stage_ptr[dev]) {
        void *h = aligned_alloc(4096, kStageBytes);
        if (!h)
            return CRAW_ERROR(ENOMEM);
        const cudaError_t err = cudaHostRegister(h, kStageBytes, cudaHostRegisterDefault);
        if (err != cudaSuccess) {
            (void)cudaGetLastError();   /* this registration's own error */
            free(h);
            craw_log(NULL, CRAW_LOG_ERROR, "craw_awb_histogram_from_rgb_cuda_noalloc: "
                     "cudaHostRegister failed on device %d: %s\n", dev, cudaGetErrorString(err));
            return CRAW_ERROR(EIO);
        }
        stage_ptr[dev] = static_cast<uint32_t *>(h);
    }
    *sc = setup_ptr[dev];
    *stage = stage_ptr[dev];
    return 0;
}

/* A failed CUDA call of this entry point: logged with its error, which is
 * read (and so cleared) because it is the call's own; EIO. */
int cuda_failed(const char *what)
{
    const cudaError_t err = cudaGetLastError();
    craw_log(NULL, CRAW_LOG_ERROR, "craw_awb_histogram_from_rgb_cuda_noalloc: %s failed: %s\n", what,
             cudaGetErrorString(err));
    return CRAW_ERROR(EIO);
}

/* The device work and the copies of one call, once the scratch and the
 * staging area are set up. */
int histogram(const float *rgb, uint32_t width, uint32_t height, size_t stride, int channels,
              const float wb_applied[3], uint32_t *count, uint32_t *weight, uint32_t *weight_bright,
              cudaStream_t stream, uint32_t *sc, uint32_t *stage)
{
    if (cudaMemsetAsync(sc, 0, (kCounter + 1) * sizeof(uint32_t), stream) != cudaSuccess)
        return cuda_failed("cudaMemsetAsync");
    if (width && height) {
        const dim3 grid((unsigned)(((width + 7) / 8 + 31) / 32), (unsigned)(((height + 7) / 8 + 7) / 8));
        k_awb_noalloc<<<grid, 256, 0, stream>>>(rgb, (int)width, (int)height, stride, channels,
                                                 wb_applied[0], wb_applied[2], sc);
        if (cudaGetLastError() != cudaSuccess)
            return cuda_failed("the kernel launch");
    }
    /* The three histograms and the counter lie together: one copy. */
    if (cudaMemcpyAsync(stage, sc, (kCounter + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                        stream) != cudaSuccess)
        return cuda_failed("cudaMemcpyAsync");
    if (cudaStreamSynchronize(stream) != cudaSuccess)
        return cuda_failed("cudaStreamSynchronize");
    memcpy(count, stage, kBins2 * sizeof(uint32_t));
    memcpy(weight, stage + kBins2, kBins2 * sizeof(uint32_t));
    memcpy(weight_bright, stage + 2 * kBins2, kBins2 * sizeof(uint32_t));
    const uint32_t nd = stage[kCounter];
    /* Bin the deferred blocks with this host's logf, a chunk at a time. */
    for (uint32_t i = 0; i < nd;) {
        const uint32_t k = nd - i < kChunk ? nd - i : kChunk;
        if (cudaMemcpyAsync(stage, sc + kDeferred + 3 * i, 3 * k * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                            stream) != cudaSuccess)
            return cuda_failed("cudaMemcpyAsync");
        if (cudaStreamSynchronize(stream) != cudaSuccess)
            return cuda_failed("cudaStreamSynchronize");
        const float *d = reinterpret_cast<const float *>(stage);
        for (uint32_t j = 0; j < k; j++)
            craw_awb_bin_host(d[3 * j], d[3 * j + 1], d[3 * j + 2], count, weight, weight_bright);
        i += k;
    }
    return 0;
}

} // namespace

extern "C" CRAW_API int craw_awb_histogram_from_rgb_cuda_noalloc(
    const float *rgb, uint32_t width, uint32_t height, size_t stride, int channels,
    const float wb_applied[3], uint32_t *count, uint32_t *weight, uint32_t *weight_bright,
    cudaStream_t stream)
{
    const uint64_t blocks = (((uint64_t)width + 7) / 8) * (((uint64_t)height + 7) / 8);
    uint32_t *sc = nullptr, *stage = nullptr;
    int ret;

    if (!rgb || !wb_applied || !count || !weight || !weight_bright)
        return CRAW_ERROR(EINVAL);
    if ((channels != 3 && channels != 4) || stride < (size_t)width * (size_t)channels)
        return CRAW_ERROR(EINVAL);
    if (!(wb_applied[0] > 0.0f) || !(wb_applied[2] > 0.0f))
        return CRAW_ERROR(EINVAL);
    if (blocks > kMaxBlocks) {
        craw_log(NULL, CRAW_LOG_ERROR, "craw_awb_histogram_from_rgb_cuda_noalloc: %ux%u has %llu "
                 "8x8 blocks; its fixed scratch holds %u (a 4096x4096 image)\n", width, height,
                 (unsigned long long)blocks, kMaxBlocks);
        return CRAW_ERROR(EINVAL);
    }
    if (cudaPeekAtLastError() != cudaSuccess) {
        /* An error an earlier call left pending: the caller's to read. */
        craw_log(NULL, CRAW_LOG_ERROR, "craw_awb_histogram_from_rgb_cuda_noalloc: a CUDA error of an "
                 "earlier call is pending (%s)\n", cudaGetErrorString(cudaPeekAtLastError()));
        return CRAW_ERROR(EIO);
    }
    if ((ret = setup(&sc, &stage)) < 0)
        return ret;
    /* The rest touches only `stream`, the scratch and the staging area, so
     * it runs with this thread's capture interaction relaxed: a global-mode
     * capture on another thread would otherwise refuse the wait on
     * `stream`, which cannot touch a capturing stream unless it is one. The
     * thread's own mode is restored before returning. */
    cudaStreamCaptureMode mode = cudaStreamCaptureModeRelaxed;
    if (cudaThreadExchangeStreamCaptureMode(&mode) != cudaSuccess)
        return cuda_failed("cudaThreadExchangeStreamCaptureMode");
    ret = histogram(rgb, width, height, stride, channels, wb_applied, count, weight, weight_bright, stream, sc,
                    stage);
    if (cudaThreadExchangeStreamCaptureMode(&mode) != cudaSuccess && ret == 0)
        ret = cuda_failed("cudaThreadExchangeStreamCaptureMode");
    return ret;
}
