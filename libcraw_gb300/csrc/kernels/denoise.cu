/*
 * The raw-domain denoise kernel: one CTA per tile of the four CFA planes
 * (the tile body is denoise_tile.cuh), and its launcher.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "denoise_tile.cuh"

/* Whether the packed spatial kernels bring interior tiles in by TMA (1,
 * the default) or by plain loads (0, for comparison and tests). */
extern "C" {
int craw_k_dn_tma = 1;
}

namespace {

using namespace craw_dn;

/* MARK: the exact rounding's marks (spatial denoise only). TMA: interior
 * tiles bring their mosaic in by one TMA tile copy (`tmap`; spatial
 * filtering without a temporal state only). */
template <int BW, int M, int WP, bool SPATIAL, bool TEMPORAL, bool HISTORY, bool X2, bool MARK, bool TMA>
__global__ void __launch_bounds__(Cfg<BW, M, WP, SPATIAL, TEMPORAL, HISTORY>::NT)
k_denoise(const CRAWKDenoise k, const CRAWKDenoiseIO io, const CRAWKRound rd,
          const __grid_constant__ CUtensorMap tmap, uint32_t *err)
{
    extern __shared__ __align__(16) float smem[];
    denoise_tile<BW, M, WP, SPATIAL, TEMPORAL, HISTORY, X2, true, MARK, TMA>(k, io, blockIdx.x, blockIdx.y, smem,
                                                                           &rd, &tmap, err);
}

template <int BW, int M, int WP, bool SPATIAL, bool TEMPORAL, bool HISTORY, bool X2, bool MARK, bool TMA>
int go(const CRAWKDenoise *k, const CRAWKDenoiseIO *io, const CRAWKRound *rd, const CUtensorMap &tmap,
       uint32_t *err, cudaStream_t s)
{
    using C = Cfg<BW, M, WP, SPATIAL, TEMPORAL, HISTORY, X2, true, TMA>;
    auto fn = k_denoise<BW, M, WP, SPATIAL, TEMPORAL, HISTORY, X2, MARK, TMA>;
    const size_t smem = (size_t)C::smem_floats * sizeof(float);
    static std::atomic<uint64_t> attr_done{ 0 };
    if (craw_smem_attr(fn, smem, attr_done) < 0)
        return -5;
    dim3 grid((k->pw + C::OX - 1) / C::OX, (k->ph + C::OY - 1) / C::OY);
    const CRAWKRound none = { nullptr, nullptr, 0.0f, 0.0f };
    fn<<<grid, C::NT, smem, s>>>(*k, *io, rd ? *rd : none, tmap, err);
    return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

/* The packed spatial kernels take the TMA fill when it is on and the
 * mosaic's layout allows a tensor map. */
template <int BW, int M, int WP, bool SPATIAL, bool TEMPORAL, bool HISTORY, bool X2, bool MARK = false>
int launch(const CRAWKDenoise *k, const CRAWKDenoiseIO *io, const CRAWKRound *rd, uint32_t *err, cudaStream_t s)
{
    if constexpr (SPATIAL && !TEMPORAL && X2) {
        using C = Cfg<BW, M, WP, SPATIAL, TEMPORAL, HISTORY, X2, true, true>;
        CUtensorMap tm;
        if (craw_k_dn_tma && craw_tmap_u16(io->src, io->src_pitch, 2 * k->pw, 2 * k->ph, C::BOX_W, C::BOX_H, &tm))
            return go<BW, M, WP, SPATIAL, TEMPORAL, HISTORY, X2, MARK, true>(k, io, rd, tm, err, s);
    }
    CUtensorMap none;
    memset(&none, 0, sizeof(none));
    return go<BW, M, WP, SPATIAL, TEMPORAL, HISTORY, X2, MARK, false>(k, io, rd, none, err, s);
}

/* X2: the search in packed f32x2 arithmetic. */
template <int BW, int M, int WP, bool X2>
int dispatch(const CRAWKDenoise *k, const CRAWKDenoiseIO *io, const CRAWKRound *rd, uint32_t *err,
             cudaStream_t s)
{
    const bool sp = k->mode & CRAW_K_DN_SPATIAL, te = k->mode & CRAW_K_DN_TEMPORAL;
    const bool hi = te && (k->mode & CRAW_K_DN_HISTORY);
    if (sp && !te && rd && rd->flags)
        return launch<BW, M, WP, true, false, false, X2, true>(k, io, rd, err, s);
    if (sp && !te)  return launch<BW, M, WP, true, false, false, X2>(k, io, rd, err, s);
    if (sp && !hi)  return launch<BW, M, WP, true, true, false, X2>(k, io, rd, err, s);
    if (sp)         return launch<BW, M, WP, true, true, true, X2>(k, io, rd, err, s);
    if (te && !hi)  return launch<BW, M, WP, false, true, false, false>(k, io, rd, err, s);
    if (te)         return launch<BW, M, WP, false, true, true, false>(k, io, rd, err, s);
    return -22;
}

} // namespace

extern "C" int craw_k_denoise(const CRAWKDenoise *k, const CRAWKDenoiseIO *io, int shape,
                              const CRAWKRound *rd, uint32_t *err, cudaStream_t s)
{
    if (craw_launch_ready() < 0)
        return -5;
    switch (shape) {
    case CRAW_K_DN_SHAPE_2x8:    return dispatch<2, 8, 1, false>(k, io, rd, err, s);
    case CRAW_K_DN_SHAPE_2x4:    return dispatch<2, 4, 2, false>(k, io, rd, err, s);
    case CRAW_K_DN_SHAPE_2x8_X2: return dispatch<2, 8, 1, true>(k, io, rd, err, s);
    case CRAW_K_DN_SHAPE_2x4_X2: return dispatch<2, 4, 2, true>(k, io, rd, err, s);
    default:                  return -22;
    }
}
