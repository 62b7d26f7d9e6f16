/*
 * The raw-domain denoise kernel: one CTA per tile of the four CFA planes
 * (the tile body is denoise_tile.cuh), and its launcher.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "denoise_tile.cuh"

namespace {

using namespace craw_dn;

/* MARK: the exact rounding's marks (spatial denoise only). */
template <int BW, int M, int WP, bool SPATIAL, bool TEMPORAL, bool HISTORY, bool X2, bool MARK>
__global__ void __launch_bounds__(Cfg<BW, M, WP, SPATIAL, TEMPORAL, HISTORY>::NT)
k_denoise(const CRAWKDenoise k, const CRAWKDenoiseIO io, const CRAWKRound rd)
{
    extern __shared__ __align__(16) float smem[];
    denoise_tile<BW, M, WP, SPATIAL, TEMPORAL, HISTORY, X2, true, MARK>(k, io, blockIdx.x, blockIdx.y, smem, &rd);
}

template <int BW, int M, int WP, bool SPATIAL, bool TEMPORAL, bool HISTORY, bool X2, bool MARK = false>
int launch(const CRAWKDenoise *k, const CRAWKDenoiseIO *io, const CRAWKRound *rd, cudaStream_t s)
{
    using C = Cfg<BW, M, WP, SPATIAL, TEMPORAL, HISTORY, X2>;
    auto fn = k_denoise<BW, M, WP, SPATIAL, TEMPORAL, HISTORY, X2, MARK>;
    const size_t smem = (size_t)C::smem_floats * sizeof(float);
    static std::atomic<uint64_t> attr_done{ 0 };
    if (craw_smem_attr(fn, smem, attr_done) < 0)
        return -5;
    dim3 grid((k->pw + C::OX - 1) / C::OX, (k->ph + C::OY - 1) / C::OY);
    const CRAWKRound none = { nullptr, nullptr, 0.0f, 0.0f };
    fn<<<grid, C::NT, smem, s>>>(*k, *io, rd ? *rd : none);
    return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

/* X2: the search in packed f32x2 arithmetic. */
template <int BW, int M, int WP, bool X2>
int dispatch(const CRAWKDenoise *k, const CRAWKDenoiseIO *io, const CRAWKRound *rd, cudaStream_t s)
{
    const bool sp = k->mode & CRAW_K_DN_SPATIAL, te = k->mode & CRAW_K_DN_TEMPORAL;
    const bool hi = te && (k->mode & CRAW_K_DN_HISTORY);
    if (sp && !te && rd && rd->flags)
        return launch<BW, M, WP, true, false, false, X2, true>(k, io, rd, s);
    if (sp && !te)  return launch<BW, M, WP, true, false, false, X2>(k, io, rd, s);
    if (sp && !hi)  return launch<BW, M, WP, true, true, false, X2>(k, io, rd, s);
    if (sp)         return launch<BW, M, WP, true, true, true, X2>(k, io, rd, s);
    if (te && !hi)  return launch<BW, M, WP, false, true, false, false>(k, io, rd, s);
    if (te)         return launch<BW, M, WP, false, true, true, false>(k, io, rd, s);
    return -22;
}

} // namespace

extern "C" int craw_k_denoise(const CRAWKDenoise *k, const CRAWKDenoiseIO *io, int shape,
                              const CRAWKRound *rd, cudaStream_t s)
{
    if (craw_launch_ready() < 0)
        return -5;
    switch (shape) {
    case CRAW_K_DN_SHAPE_2x8:    return dispatch<2, 8, 1, false>(k, io, rd, s);
    case CRAW_K_DN_SHAPE_2x4:    return dispatch<2, 4, 2, false>(k, io, rd, s);
    case CRAW_K_DN_SHAPE_2x8_X2: return dispatch<2, 8, 1, true>(k, io, rd, s);
    case CRAW_K_DN_SHAPE_2x4_X2: return dispatch<2, 4, 2, true>(k, io, rd, s);
    default:                  return -22;
    }
}
