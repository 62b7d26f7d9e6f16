/*
 * Host side of the TMA tile copies: tensor maps of 16-bit mosaics,
 * encoded through the driver's cuTensorMapEncodeTiled (looked up once),
 * with a small per-thread cache since a pipeline encodes the same few
 * maps frame after frame.
 */
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "tma.cuh"

namespace {

typedef CUresult (*EncodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

struct Entry {
    const void *src;
    size_t pitch;
    int w, h, bw, bh;
    CUtensorMap map;
};

constexpr int kEntries = 4;

} // namespace

bool craw_tmap_u16(const void *src, size_t pitch, int w, int h, int bw, int bh, CUtensorMap *out)
{
    /* Looked up once per process (a thread-safe static initialisation). */
    static const EncodeTiled encode = [] {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        EncodeTiled e = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            e = reinterpret_cast<EncodeTiled>(fn);
        (void)cudaGetLastError();
        return e;
    }();
    thread_local Entry cache[kEntries] = {};
    thread_local int next = 0;
    if (!encode || ((uintptr_t)src & 15) || (pitch & 15))
        return false;
    for (int i = 0; i < kEntries; i++) {
        const Entry &c = cache[i];
        if (c.src == src && c.pitch == pitch && c.w == w && c.h == h && c.bw == bw && c.bh == bh) {
            *out = c.map;
            return true;
        }
    }
    Entry &c = cache[next];
    const cuuint64_t dims[2] = { (cuuint64_t)w, (cuuint64_t)h };
    const cuuint64_t strides[1] = { (cuuint64_t)pitch };
    const cuuint32_t box[2] = { (cuuint32_t)bw, (cuuint32_t)bh };
    const cuuint32_t estr[2] = { 1, 1 };
    if (encode(&c.map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, const_cast<void *>(src), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
        c.src = nullptr;
        return false;
    }
    c.src = src;
    c.pitch = pitch;
    c.w = w;
    c.h = h;
    c.bw = bw;
    c.bh = bh;
    next = (next + 1) % kEntries;
    *out = c.map;
    return true;
}
