/*
 * The fused develop kernels (tile bodies in develop_tile.cuh): prep +
 * debayer + colour + AWB records in one launch, with the RCD's interior
 * tiles done by CFA quads and the rest per pixel; and their launcher.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "develop_tile.cuh"

namespace {

using namespace craw_dev;

__global__ void __launch_bounds__(QNT)
k_develop_rcd_quads(const CRAWKDevelop k, const CRAWKDevelopIO io)
{
    extern __shared__ __align__(16) float smem[];
    const int x0 = blockIdx.x * QTW, y0 = blockIdx.y * QTH;
    if (!quad_interior(x0, y0, k.width, k.height))
        return;
    rcd_quad_tile(k, io, x0, y0, smem);
}

/* Eight CTAs an SM (full occupancy at 256 threads): the bilinear and MHC
 * tiles are bound by HBM and need every warp in flight. */
template <int METHOD, int TW, int TH, int NT>
__global__ void __launch_bounds__(NT, 2048 / NT)
k_develop(const CRAWKDevelop k, const CRAWKDevelopIO io)
{
    extern __shared__ __align__(16) float smem[];
    pixel_tile<METHOD, TW, TH, NT>(k, io, blockIdx.x * TW, blockIdx.y * TH, smem);
}

template <int METHOD, int TW, int TH, int NT>
int launch(const CRAWKDevelop *k, const CRAWKDevelopIO *io, cudaStream_t s)
{
    dim3 grid((k->width + TW - 1) / TW, (k->height + TH - 1) / TH);
    k_develop<METHOD, TW, TH, NT><<<grid, NT, PixelSmem<METHOD, TW, TH, NT>::floats * sizeof(float), s>>>(*k, *io);
    return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

int launch_rcd(const CRAWKDevelop *k, const CRAWKDevelopIO *io, cudaStream_t s)
{
    constexpr size_t smem = RcdQuads<QTW, QTH, QNT>::floats * sizeof(float);
    static bool attr_set = false;
    if (!attr_set) {
        if (cudaFuncSetAttribute(k_develop_rcd_quads, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return -5;
        attr_set = true;
    }
    dim3 grid((k->width + QTW - 1) / QTW, (k->height + QTH - 1) / QTH);
    k_develop_rcd_quads<<<grid, QNT, smem, s>>>(*k, *io);
    if (cudaGetLastError() != cudaSuccess)
        return -5;
    return launch<kRcd, BTW, BTH, 256>(k, io, s);
}

} // namespace

extern "C" int craw_k_develop(const CRAWKDevelop *k, const CRAWKDevelopIO *io, int shape,
                              cudaStream_t s)
{
    (void)cudaGetLastError();   /* a stale error of an earlier call is not ours */
    (void)shape;
    switch (k->method) {
    case kBilinear: return launch<kBilinear, 64, 16, 256>(k, io, s);
    case kMhc:      return launch<kMhc, 64, 16, 256>(k, io, s);
    case kRcd:      return launch_rcd(k, io, s);
    default:        return -22;
    }
}
