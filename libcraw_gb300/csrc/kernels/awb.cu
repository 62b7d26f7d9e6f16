/*
 * The AWB histogram reduction: 8x8-block records (one u64 each, written by
 * the develop kernels) folded into the three 128 x 128 histograms of the
 * reference (count, sum of min(g, 0.5), sum of g^4; lib/awb.c:287-291).
 *
 * Frames of more than kDirectMax blocks: each CTA keeps a private copy of
 * all three histograms in shared memory (3 x 64 KB), folds a contiguous
 * share of the records into it with warp-aggregated atomics (lanes holding
 * the same bin are found with __match_any_sync and summed with
 * __reduce_add_sync, so one leader does one shared atomic per distinct bin
 * per warp), and finally adds its non-zero bins to the device histogram.
 * Smaller frames take the same warp aggregation straight to the device
 * histogram. Every sum is a uint32 sum, as in the reference, so the order
 * of the additions does not matter.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace {

constexpr int kBins = 128 * 128;
constexpr int kThreads = 1024;

__global__ void __launch_bounds__(kThreads)
k_awb_reduce(const uint64_t *__restrict__ rec, uint32_t n, uint32_t *__restrict__ hist)
{
    extern __shared__ uint32_t h[];
    for (int i = threadIdx.x; i < 3 * kBins; i += kThreads)
        h[i] = 0;
    __syncthreads();

    const uint32_t per = (n + gridDim.x - 1) / gridDim.x;
    const uint32_t beg = blockIdx.x * per, end = min(n, beg + per);
    const int lane = threadIdx.x & 31;
    for (uint32_t base = beg; base < end; base += kThreads) {
        uint32_t i = base + threadIdx.x;
        uint64_t r = i < end ? __ldg(rec + i) : 0ull;
        bool valid = (r & CRAW_K_AWB_VALID) != 0;
        uint32_t bin = valid ? (uint32_t)(r & 0x3fffu) : 0xffffffffu;
        uint32_t w = (uint32_t)((r >> 14) & 0xffffu), wb = (uint32_t)((r >> 30) & 0xffffu);
        uint32_t group = __match_any_sync(0xffffffffu, bin);
        uint32_t ws = __reduce_add_sync(group, w), bs = __reduce_add_sync(group, wb);
        if (valid && lane == __ffs(group) - 1) {
            atomicAdd(&h[bin], (uint32_t)__popc(group));
            atomicAdd(&h[kBins + bin], ws);
            atomicAdd(&h[2 * kBins + bin], bs);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 3 * kBins; i += kThreads) {
        uint32_t v = h[i];
        if (v)
            atomicAdd(&hist[i], v);
    }
}

/* Small frames: a record a thread, the warp's records of one bin summed
 * by their leader, one device atomic per distinct bin per warp and
 * histogram. No shared-memory copy to clear and fold, which costs a fixed
 * ~10 us whatever the number of records; a frame whose records mostly
 * share one bin costs at most n / 32 atomics on one address here. */
constexpr uint32_t kDirectMax = 1u << 16;       /* records (a 4 Mpx frame) */
constexpr int kDirectThreads = 256;

__global__ void __launch_bounds__(kDirectThreads)
k_awb_reduce_direct(const uint64_t *__restrict__ rec, uint32_t n, uint32_t *__restrict__ hist)
{
    const uint32_t i = blockIdx.x * kDirectThreads + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const uint64_t r = i < n ? __ldg(rec + i) : 0ull;
    const bool valid = (r & CRAW_K_AWB_VALID) != 0;
    const uint32_t bin = valid ? (uint32_t)(r & 0x3fffu) : 0xffffffffu;
    const uint32_t w = (uint32_t)((r >> 14) & 0xffffu), wb = (uint32_t)((r >> 30) & 0xffffu);
    const uint32_t group = __match_any_sync(0xffffffffu, bin);
    const uint32_t ws = __reduce_add_sync(group, w), bs = __reduce_add_sync(group, wb);
    if (valid && lane == __ffs(group) - 1) {
        atomicAdd(&hist[bin], (uint32_t)__popc(group));
        atomicAdd(&hist[kBins + bin], ws);
        atomicAdd(&hist[2 * kBins + bin], bs);
    }
}

} // namespace

extern "C" int craw_k_awb_reduce(const uint64_t *rec, uint32_t n, uint32_t *hist, cudaStream_t s)
{
    if (craw_launch_ready() < 0)
        return -5;
    if (n <= kDirectMax) {
        if (n)
            k_awb_reduce_direct<<<(n + kDirectThreads - 1) / kDirectThreads, kDirectThreads, 0, s>>>(rec, n,
                                                                                                       hist);
        return cudaGetLastError() == cudaSuccess ? 0 : -5;
    }
    static std::atomic<uint64_t> attr_done{ 0 };
    const int smem = 3 * kBins * (int)sizeof(uint32_t);
    if (craw_smem_attr(k_awb_reduce, (size_t)smem, attr_done) < 0)
        return -5;
    /* About 2048 records a CTA, at most one CTA an SM of a 152-SM part
     * (at 5760x3240: 16384 a CTA took 39 us, 4096 18 us, 2048 14 us). */
    uint32_t grid = (n + 2047) / 2048;
    grid = grid < 1 ? 1 : (grid > 148 ? 148 : grid);
    k_awb_reduce<<<grid, kThreads, smem, s>>>(rec, n, hist);
    return cudaGetLastError() == cudaSuccess ? 0 : -5;
}
