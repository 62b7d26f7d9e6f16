/*
 * Batched development of frames of uneven sizes in one persistent launch.
 *
 * The work is a list of tiles: every denoise tile of every frame, then
 * every develop tile of every frame. A CTA takes items blockIdx.x,
 * blockIdx.x + gridDim.x, ... of each list, copies the item's frame
 * constants into shared memory and runs the same tile bodies as the
 * single-frame kernels (denoise_tile.cuh, develop_tile.cuh). Between the
 * two phases every CTA waits at a grid-wide barrier (a cooperative launch:
 * the runtime checks that the whole grid is resident, and the barrier is
 * the cooperative-groups one), because a develop tile reads its
 * neighbours' denoised samples. Unfused, the two phases are two launches.
 */
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "denoise_tile.cuh"
#include "develop_tile.cuh"

namespace {

namespace cg = cooperative_groups;
using namespace craw_dev;

constexpr int NT = 256;

template <int M> struct DnShape {
    using C = craw_dn::Cfg<2, M, 2, true, false, false>;
};

template <typename T>
CRAW_DEV void copy_words(T *dst, const T *src)
{
    static_assert(sizeof(T) % 4 == 0, "words");
    for (int i = threadIdx.x; i < (int)(sizeof(T) / 4); i += NT)
        reinterpret_cast<uint32_t *>(dst)[i] = reinterpret_cast<const uint32_t *>(src)[i];
}

/* The frame an item of a phase belongs to: the last one whose first item
 * is not after it. */
CRAW_DEV int item_frame(const CRAWKBatchFrame *F, int nb, int item, bool develop)
{
    int f = 0;
    for (int i = 1; i < nb; i++)
        if ((develop ? F[i].dv_first : F[i].dn_first) <= item)
            f = i;
    return f;
}

template <int M>
CRAW_DEV void denoise_phase(const CRAWKBatchFrame *F, int nb, int items, float *smem)
{
    __shared__ CRAWKDenoise s_dn;
    __shared__ CRAWKDenoiseIO s_dio;
    __shared__ int s_tx, s_first;
    for (int it = blockIdx.x; it < items; it += gridDim.x) {
        const int f = item_frame(F, nb, it, false);
        __syncthreads();
        copy_words(&s_dn, &F[f].dn);
        copy_words(&s_dio, &F[f].dio);
        if (threadIdx.x == 0) {
            s_tx = F[f].dn_tx;
            s_first = F[f].dn_first;
        }
        __syncthreads();
        const int local = it - s_first;
        craw_dn::denoise_tile<2, M, 2, true, false, false>(s_dn, s_dio, local % s_tx, local / s_tx, smem);
    }
}

template <int METHOD>
CRAW_DEV void develop_phase(const CRAWKBatchFrame *F, int nb, int items, float *smem)
{
    __shared__ CRAWKDevelop s_dv;
    __shared__ CRAWKDevelopIO s_vio;
    __shared__ int s_tx, s_first;
    for (int it = blockIdx.x; it < items; it += gridDim.x) {
        const int f = item_frame(F, nb, it, true);
        __syncthreads();
        copy_words(&s_dv, &F[f].dv);
        copy_words(&s_vio, &F[f].vio);
        if (threadIdx.x == 0) {
            s_tx = F[f].dv_tx;
            s_first = F[f].dv_first;
        }
        __syncthreads();
        const int local = it - s_first;
        const int x0 = (local % s_tx) * QTW, y0 = (local / s_tx) * QTH;
        if constexpr (METHOD == kRcd) {
            if (quad_interior(x0, y0, s_dv.width, s_dv.height)) {
                rcd_quad_tile(s_dv, s_vio, x0, y0, smem);
                continue;
            }
        }
        /* Per-pixel tiles of BTW x BTH cover the QTW x QTH item. */
        for (int sx = 0; sx < QTW; sx += BTW) {
            if (x0 + sx >= s_dv.width)
                break;
            __syncthreads();
            pixel_tile<METHOD, BTW, BTH, NT>(s_dv, s_vio, x0 + sx, y0, smem);
        }
    }
}

template <int M, int METHOD> struct Smem {
    static constexpr int dn = DnShape<M>::C::smem_floats;
    static constexpr int dv = METHOD == kRcd ? RcdQuads<QTW, QTH, NT>::floats : 0;
    static constexpr int px = PixelSmem<METHOD, BTW, BTH, NT>::floats;
    static constexpr int a = dn > dv ? dn : dv;
    static constexpr int floats = a > px ? a : px;
};

template <int M, int METHOD>
__global__ void __launch_bounds__(NT)
k_batch_fused(const CRAWKBatchFrame *F, int nb, int dn_items, int dv_items)
{
    extern __shared__ __align__(16) float smem[];
    denoise_phase<M>(F, nb, dn_items, smem);
    cg::this_grid().sync();
    develop_phase<METHOD>(F, nb, dv_items, smem);
}

template <int M>
__global__ void __launch_bounds__(NT)
k_batch_denoise(const CRAWKBatchFrame *F, int nb, int dn_items)
{
    extern __shared__ __align__(16) float smem[];
    denoise_phase<M>(F, nb, dn_items, smem);
}

template <int METHOD>
__global__ void __launch_bounds__(NT)
k_batch_develop(const CRAWKBatchFrame *F, int nb, int dv_items)
{
    extern __shared__ __align__(16) float smem[];
    develop_phase<METHOD>(F, nb, dv_items, smem);
}

int device_sms()
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return -1;
    return sms;
}

/* As many CTAs as fit on the device at once, at most `items`. */
template <typename K>
int resident_grid(K kernel, size_t smem, int items)
{
    int per_sm = 0, sms = device_sms();
    if (sms <= 0 ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, NT, smem) != cudaSuccess ||
        per_sm <= 0)
        return -1;
    return items < per_sm * sms ? (items > 0 ? items : 1) : per_sm * sms;
}

template <typename K>
int set_smem(K kernel, size_t smem)
{
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) ==
           cudaSuccess ? 0 : -5;
}

template <int M, int METHOD>
int run(const CRAWKBatchFrame *F, int nb, int dn_items, int dv_items, int fused, cudaStream_t s)
{
    const size_t smem = Smem<M, METHOD>::floats * sizeof(float);
    if (fused) {
        auto k = k_batch_fused<M, METHOD>;
        if (set_smem(k, smem) < 0)
            return -5;
        int grid = resident_grid(k, smem, dn_items > dv_items ? dn_items : dv_items);
        if (grid < 0)
            return -5;
        void *args[] = { (void *)&F, (void *)&nb, (void *)&dn_items, (void *)&dv_items };
        if (cudaLaunchCooperativeKernel((const void *)k, dim3(grid), dim3(NT), args, smem, s) != cudaSuccess)
            return -5;
        return 0;
    }
    if (dn_items > 0) {
        auto k = k_batch_denoise<M>;
        const size_t sm = DnShape<M>::C::smem_floats * sizeof(float);
        if (set_smem(k, sm) < 0)
            return -5;
        int grid = resident_grid(k, sm, dn_items);
        if (grid < 0)
            return -5;
        k<<<grid, NT, sm, s>>>(F, nb, dn_items);
        if (cudaGetLastError() != cudaSuccess)
            return -5;
    }
    {
        auto k = k_batch_develop<METHOD>;
        const size_t sm = (METHOD == kRcd ? RcdQuads<QTW, QTH, NT>::floats
                                          : PixelSmem<METHOD, BTW, BTH, NT>::floats) * sizeof(float);
        if (set_smem(k, sm) < 0)
            return -5;
        int grid = resident_grid(k, sm, dv_items);
        if (grid < 0)
            return -5;
        k<<<grid, NT, sm, s>>>(F, nb, dv_items);
        if (cudaGetLastError() != cudaSuccess)
            return -5;
    }
    return 0;
}

template <int M>
int run_method(const CRAWKBatchFrame *F, int nb, int dn_items, int dv_items, int method, int fused,
               cudaStream_t s)
{
    switch (method) {
    case kBilinear: return run<M, kBilinear>(F, nb, dn_items, dv_items, fused, s);
    case kMhc:      return run<M, kMhc>(F, nb, dn_items, dv_items, fused, s);
    case kRcd:      return run<M, kRcd>(F, nb, dn_items, dv_items, fused, s);
    default:        return -22;
    }
}

} // namespace

extern "C" void craw_k_batch_tiles(int32_t w, int32_t h, int shape, int32_t *dn_tx, int32_t *dn_ty,
                                   int32_t *dv_tx, int32_t *dv_ty)
{
    const int oy = shape == CRAW_K_BATCH_DN_2x8 ? DnShape<8>::C::OY : DnShape<4>::C::OY;
    const int ox = DnShape<4>::C::OX;
    *dn_tx = (w / 2 + ox - 1) / ox;
    *dn_ty = (h / 2 + oy - 1) / oy;
    *dv_tx = (w + QTW - 1) / QTW;
    *dv_ty = (h + QTH - 1) / QTH;
}

extern "C" int craw_k_batch(const CRAWKBatchFrame *frames, int32_t nb, int32_t dn_items,
                            int32_t dv_items, int method, int shape, int fused, cudaStream_t s)
{
    (void)cudaGetLastError();   /* a stale error of an earlier call is not ours */
    if (nb <= 0)
        return -22;
    switch (shape) {
    case CRAW_K_BATCH_DN_2x4: return run_method<4>(frames, nb, dn_items, dv_items, method, fused, s);
    case CRAW_K_BATCH_DN_2x8: return run_method<8>(frames, nb, dn_items, dv_items, method, fused, s);
    default:                  return -22;
    }
}
