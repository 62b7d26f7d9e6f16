/*
 * Batched development of frames of uneven sizes in one persistent launch.
 *
 * The work is a list of tiles: every denoise tile of every frame, then
 * every develop tile of every frame. A CTA takes items blockIdx.x,
 * blockIdx.x + gridDim.x, ... of each list and runs the same tile bodies
 * as the single-frame kernels (denoise_tile.cuh, develop_tile.cuh) on the
 * item's frame constants, which sit in the launch's parameter bank (the
 * frame table is a __grid_constant__ parameter): uniform constant-cache
 * loads, as the single-frame kernels read theirs. Between the
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
constexpr int BQH = 16;     /* rows of a develop item (a 64 x 16 quad tile) */

/* The denoise of a batch: the packed f32x2 search, 2 columns x M rows a
 * thread, 256 threads. */
template <int M> struct DnShape {
    using C = craw_dn::Cfg<2, M, 2, true, false, false, true, false>;
};

/* The frame an item of a phase belongs to: the last one whose first item
 * is not after it. */
CRAW_DEV int item_frame(const CRAWKBatchTable &T, int nb, int item, bool develop)
{
    int f = 0;
    for (int i = 1; i < nb; i++)
        if ((develop ? T.f[i].dv_first : T.f[i].dn_first) <= item)
            f = i;
    return f;
}

template <int M>
CRAW_DEV void denoise_phase(const CRAWKBatchTable &T, int nb, int items, float *smem)
{
    for (int it = blockIdx.x; it < items; it += gridDim.x) {
        const CRAWKBatchFrame &F = T.f[item_frame(T, nb, it, false)];
        const int local = it - F.dn_first;
        __syncthreads();   /* the previous item's shared memory is free */
        craw_dn::denoise_tile<2, M, 2, true, false, false, true, false>(F.dn, F.dio, local % F.dn_tx,
                                                                  local / F.dn_tx, smem);
    }
}

template <int METHOD>
CRAW_DEV void develop_phase(const CRAWKBatchTable &T, int nb, int items, float *smem)
{
    for (int it = blockIdx.x; it < items; it += gridDim.x) {
        const CRAWKBatchFrame &F = T.f[item_frame(T, nb, it, true)];
        const int local = it - F.dv_first;
        const int x0 = (local % F.dv_tx) * QTW, y0 = (local / F.dv_tx) * BQH;
        __syncthreads();
        if constexpr (METHOD == kRcd) {
            if (quad_interior<BQH>(x0, y0, F.dv.width, F.dv.height)) {
                rcd_quad_tile<BQH, NT>(F.dv, F.vio, x0, y0, smem);
                continue;
            }
        }
        /* Per-pixel tiles of BTW x BTH cover the QTW x BQH item. */
        for (int sx = 0; sx < QTW; sx += BTW) {
            if (x0 + sx >= F.dv.width)
                break;
            __syncthreads();
            pixel_tile<METHOD, BTW, BTH, NT, BQH>(F.dv, F.vio, x0 + sx, y0, smem);
        }
    }
}

template <int M, int METHOD> struct Smem {
    static constexpr int dn = DnShape<M>::C::smem_floats;
    static constexpr int dv = METHOD == kRcd ? RcdQuads<QTW, BQH, NT>::floats : 0;
    static constexpr int px = PixelSmem<METHOD, BTW, BTH, NT>::floats;
    static constexpr int a = dn > dv ? dn : dv;
    static constexpr int floats = a > px ? a : px;
};

template <int M, int METHOD>
__global__ void __launch_bounds__(NT)
k_batch_fused(const __grid_constant__ CRAWKBatchTable T, int nb, int dn_items, int dv_items)
{
    extern __shared__ __align__(16) float smem[];
    denoise_phase<M>(T, nb, dn_items, smem);
    cg::this_grid().sync();
    develop_phase<METHOD>(T, nb, dv_items, smem);
}

template <int M>
__global__ void __launch_bounds__(NT)
k_batch_denoise(const __grid_constant__ CRAWKBatchTable T, int nb, int dn_items, int dv_items)
{
    extern __shared__ __align__(16) float smem[];
    denoise_phase<M>(T, nb, dn_items, smem);
}

/* Four CTAs an SM, the shared memory's limit for RCD items: registers
 * kept at 64 a thread so that they do not set a lower one. */
template <int METHOD>
__global__ void __launch_bounds__(NT, 4)
k_batch_develop(const __grid_constant__ CRAWKBatchTable T, int nb, int dn_items, int dv_items)
{
    extern __shared__ __align__(16) float smem[];
    develop_phase<METHOD>(T, nb, dv_items, smem);
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
int run(const CRAWKBatchTable *T, int nb, int dn_items, int dv_items, int fused, cudaStream_t s)
{
    const size_t smem = Smem<M, METHOD>::floats * sizeof(float);
    void *args[] = { (void *)T, (void *)&nb, (void *)&dn_items, (void *)&dv_items };
    if (fused) {
        auto k = k_batch_fused<M, METHOD>;
        if (set_smem(k, smem) < 0)
            return -5;
        int grid = resident_grid(k, smem, dn_items > dv_items ? dn_items : dv_items);
        if (grid < 0)
            return -5;
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
        if (grid < 0 ||
            cudaLaunchKernel((const void *)k, dim3(grid), dim3(NT), args, sm, s) != cudaSuccess)
            return -5;
    }
    {
        auto k = k_batch_develop<METHOD>;
        const size_t sm = (METHOD == kRcd ? RcdQuads<QTW, BQH, NT>::floats
                                          : PixelSmem<METHOD, BTW, BTH, NT>::floats) * sizeof(float);
        if (set_smem(k, sm) < 0)
            return -5;
        int grid = resident_grid(k, sm, dv_items);
        if (grid < 0 ||
            cudaLaunchKernel((const void *)k, dim3(grid), dim3(NT), args, sm, s) != cudaSuccess)
            return -5;
    }
    return 0;
}

template <int M>
int run_method(const CRAWKBatchTable *T, int nb, int dn_items, int dv_items, int method, int fused,
               cudaStream_t s)
{
    switch (method) {
    case kBilinear: return run<M, kBilinear>(T, nb, dn_items, dv_items, fused, s);
    case kMhc:      return run<M, kMhc>(T, nb, dn_items, dv_items, fused, s);
    case kRcd:      return run<M, kRcd>(T, nb, dn_items, dv_items, fused, s);
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
    *dv_ty = (h + BQH - 1) / BQH;
}

extern "C" int craw_k_batch(const CRAWKBatchTable *table, int32_t nb, int32_t dn_items,
                            int32_t dv_items, int method, int shape, int fused, cudaStream_t s)
{
    if (craw_launch_ready() < 0)
        return -5;
    if (nb <= 0 || nb > CRAW_K_BATCH_MAX)
        return -22;
    switch (shape) {
    case CRAW_K_BATCH_DN_2x4: return run_method<4>(table, nb, dn_items, dv_items, method, fused, s);
    case CRAW_K_BATCH_DN_2x8: return run_method<8>(table, nb, dn_items, dv_items, method, fused, s);
    default:                  return -22;
    }
}

extern "C" int craw_k_batch_update(cudaGraphExec_t exec, cudaGraph_t graph, const CRAWKBatchTable *table,
                                   int32_t nb, int32_t dn_items, int32_t dv_items)
{
    cudaGraphNode_t nodes[8];
    size_t n = 8;
    void *args[] = { (void *)table, (void *)&nb, (void *)&dn_items, (void *)&dv_items };

    if (cudaGraphGetNodes(graph, nodes, &n) != cudaSuccess || n > 8)
        return -5;
    for (size_t i = 0; i < n; i++) {
        cudaGraphNodeType t;
        cudaKernelNodeParams p;
        if (cudaGraphNodeGetType(nodes[i], &t) != cudaSuccess)
            return -5;
        if (t != cudaGraphNodeTypeKernel)
            continue;
        if (cudaGraphKernelNodeGetParams(nodes[i], &p) != cudaSuccess)
            return -5;
        p.kernelParams = args;
        p.extra = nullptr;
        if (cudaGraphExecKernelNodeSetParams(exec, nodes[i], &p) != cudaSuccess)
            return -5;
    }
    return 0;
}
