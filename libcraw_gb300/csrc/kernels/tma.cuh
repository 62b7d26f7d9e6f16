/*
 * Tile copies by the Tensor Memory Accelerator: a 2-D box of a 16-bit
 * mosaic into shared memory, completed on an mbarrier, with a bounded
 * wait; and the host side's tensor maps.
 */
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace craw_tma {

/* try_wait suspends for a while each time; this bound is seconds. */
constexpr int kWaitTries = 1 << 20;

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

/* Thread 0 makes `bar` an mbarrier for one arrival; every thread of the
 * CTA calls this (it ends with a barrier). */
__device__ __forceinline__ void bar_init(uint64_t *bar)
{
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
}

/* One thread: the box of `tmap` at element coordinates (x, y) into `dst`
 * (bytes of it in all), completing on `bar`. x times the element size
 * must be a multiple of 16 bytes; the caller checks. */
__device__ __forceinline__ void load_2d(void *dst, const CUtensorMap *tmap, int x, int y, uint64_t *bar,
                                        uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 :: "r"(smem_u32(bar)), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3}], [%4];"
                 :: "r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y),
                    "r"(smem_u32(bar))
                 : "memory");
}

/* Waits (a bounded number of tries) for phase `parity` of `bar`; false if
 * it did not complete. */
__device__ __forceinline__ bool wait(uint64_t *bar, uint32_t parity)
{
    const uint32_t b = smem_u32(bar);
    for (int i = 0; i < kWaitTries; i++) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done) : "r"(b), "r"(parity) : "memory");
        if (done)
            return true;
    }
    return false;
}

} // namespace craw_tma

/* The tensor map of a 16-bit mosaic (w x h samples, rows `pitch` bytes
 * apart) for boxes of bw x bh samples; a few recent maps are kept per
 * thread. False where the driver call is not available or refuses the
 * layout (src and pitch must be 16-byte aligned). */
bool craw_tmap_u16(const void *src, size_t pitch, int w, int h, int bw, int bh, CUtensorMap *out);
