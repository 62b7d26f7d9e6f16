/*
 * The fused develop kernels (tile bodies in develop_tile.cuh): prep +
 * debayer + colour + AWB records in one launch, with the RCD's interior
 * tiles done by CFA quads and the rest per pixel; and their launcher.
 */
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "develop_strip.cuh"
#include "develop_tile.cuh"
#include "tma.cuh"

/* Whether the RCD interior tiles load their mosaic by TMA (1, the
 * default) or by plain loads (0, for comparison and tests); whether the
 * interior runs by 64x16 tiles (0), by strips where they are the faster
 * (1, the default) or by strips wherever they apply (2). */
extern "C" {
int craw_k_rcd_tma = 1;
int craw_k_rcd_strips = 1;
}

namespace {

using namespace craw_dev;

/* How a frame's RCD splits into QTW x QTH quad tiles: the interior ones
 * (rows r_lo..r_hi, columns c_lo..c_hi, all aprons inside the frame) go to
 * the quad kernel, the ring of the others to the per-pixel kernel, each as
 * a grid of only its own tiles. */
struct QuadGrid {
    int qx, qy;                      /* quad tiles across, down */
    int r_lo, r_hi, c_lo, c_hi;      /* the interior (empty when hi < lo) */
    int rows_full, cols_border, mid_rows;

    void init(int w, int h)
    {
        qx = (w + QTW - 1) / QTW;
        qy = (h + QTH - 1) / QTH;
        /* quad_interior(): x0 >= 6, x0 + QTW + 6 <= w, and the same in y. */
        c_lo = 1;
        c_hi = w >= QTW + 6 ? (w - QTW - 6) / QTW : -1;
        r_lo = 1;
        r_hi = h >= QTH + 6 ? (h - QTH - 6) / QTH : -1;
        const bool has_r = r_hi >= r_lo, has_c = c_hi >= c_lo;
        rows_full = has_r ? r_lo + (qy - 1 - r_hi) : qy;   /* rows with no interior tile */
        mid_rows = has_r ? r_hi - r_lo + 1 : 0;
        cols_border = has_c ? c_lo + (qx - 1 - c_hi) : qx;  /* border tiles of the other rows */
    }
    int interior_x() const { return c_hi >= c_lo ? c_hi - c_lo + 1 : 0; }
    int interior_y() const { return r_hi >= r_lo ? r_hi - r_lo + 1 : 0; }
    int border_quads() const { return rows_full * qx + mid_rows * cols_border; }

    /* Quad tile (col, row) of border tile t. */
    CRAW_DEV void border(int t, int &col, int &row) const
    {
        const bool has_r = r_hi >= r_lo, has_c = c_hi >= c_lo;
        if (t < rows_full * qx) {
            const int rr = t / qx;
            col = t % qx;
            row = (!has_r || rr < r_lo) ? rr : r_hi + 1 + (rr - r_lo);
        } else {
            t -= rows_full * qx;
            const int rr = t / cols_border, cc = t % cols_border;
            row = r_lo + rr;
            col = (!has_c || cc < c_lo) ? cc : c_hi + 1 + (cc - c_lo);
        }
    }
};

/* An interior kernel lets the border launch that follows it on the stream
 * begin at once (programmatic dependent launch): the two write disjoint
 * tiles, and the border CTAs take the SM slots that the interior's last
 * wave leaves idle. The launches after the border wait for both as usual. */
CRAW_DEV void release_border()
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__global__ void __launch_bounds__(QNT)
k_develop_rcd_quads(const CRAWKDevelop k, const CRAWKDevelopIO io, const QuadGrid g)
{
    extern __shared__ __align__(16) float smem[];
    release_border();
    rcd_quad_tile(k, io, (g.c_lo + blockIdx.x) * QTW, (g.r_lo + blockIdx.y) * QTH, smem);
}

/* ---- the same with the tile's mosaic brought in by one TMA tile copy */

/* The box: frame columns x0 - 8 .. x0 + QTW + 8 (the apron needs x0 - 6
 * .. x0 + QTW + 6; a TMA copy starts on a 16-byte boundary, and x0 - 8 is
 * a multiple of 8 samples), rows y0 - 6 .. y0 + QTH + 6. Interior tiles
 * only, so every coordinate is inside the frame except, at most, the last
 * two columns (read as zeros and never used). */
constexpr int kBoxW = QTW + 16, kBoxH = QTH + 12;
constexpr uint32_t kBoxBytes = kBoxW * kBoxH * 2;

__global__ void __launch_bounds__(QNT)
k_develop_rcd_quads_tma(const CRAWKDevelop k, const CRAWKDevelopIO io, const QuadGrid g,
                        const __grid_constant__ CUtensorMap tmap)
{
    extern __shared__ __align__(16) float smem[];
    __shared__ __align__(8) uint64_t bar_s;
    release_border();
    const int x0 = (g.c_lo + blockIdx.x) * QTW, y0 = (g.r_lo + blockIdx.y) * QTH;
    RcdQuads<QTW, QTH, QNT> t;
    t.carve(smem);
    /* The box lives in the discrimination planes' space, which the tile
     * first writes after the load; 128-byte aligned for the copy. */
    static_assert(kBoxBytes + 128 <= 4 * RcdQuads<QTW, QTH, QNT>::DN * sizeof(float), "box fits");
    uint32_t *box = reinterpret_cast<uint32_t *>(((uintptr_t)t.Dp + 127) & ~(uintptr_t)127);
    craw_tma::bar_init(&bar_s);
    if (threadIdx.x == 0)
        craw_tma::load_2d(box, &tmap, x0 - 8, y0 - 6, &bar_s, kBoxBytes);
    if (!__syncthreads_and(craw_tma::wait(&bar_s, 0))) {
        /* Never expected: record it, give the copy one more bound to land
         * before the CTA leaves, and skip the tile. */
        if (threadIdx.x == 0 && io.err)
            atomicOr(io.err, CRAW_K_ERR_TMA_WAIT);
        (void)craw_tma::wait(&bar_s, 0);
        return;
    }
    t.load_box<kBoxW>(k, io, box);
    __syncthreads();
    t.run();
    epilogue<QTW, QTH, QNT>(k, io, x0, y0, t.rgb);
}

/* The interior by strips (develop_strip.cuh): SOUT x seg output quads a
 * CTA, four CTAs an SM (55 KB of shared memory each). */
__global__ void __launch_bounds__(SNT, 4)
k_develop_rcd_strips(const CRAWKDevelop k, const CRAWKDevelopIO io, const StripGrid g)
{
    extern __shared__ __align__(16) float smem[];
    release_border();
    rcd_strip(k, io, g, blockIdx.x, blockIdx.y, *reinterpret_cast<StripSmem *>(smem));
}

/* The per-pixel RCD on the ring of border quad tiles, BTW x BTH pixels a
 * CTA (QTW / BTW of them a quad tile). */
__global__ void __launch_bounds__(256, 8)
k_develop_rcd_border(const CRAWKDevelop k, const CRAWKDevelopIO io, const QuadGrid g)
{
    extern __shared__ __align__(16) float smem[];
    constexpr int PER = QTW / BTW;
    static_assert(QTH == BTH, "a border quad tile is one row of per-pixel tiles");
    int col, row;
    g.border(blockIdx.x / PER, col, row);
    const int x0 = col * QTW + (blockIdx.x % PER) * BTW, y0 = row * QTH;
    if (x0 >= k.width)
        return;
    pixel_tile<kRcd, BTW, BTH, 256>(k, io, x0, y0, smem);
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

/* The current device's SM count, kept per device ordinal below 64 (152,
 * GB300's, if the query fails). */
int craw_sm_count()
{
    static std::atomic<int> known[64];
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return 152;
    if (dev >= 0 && dev < 64 && (sms = known[dev].load(std::memory_order_relaxed)) > 0)
        return sms;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        return 152;
    if (dev >= 0 && dev < 64)
        known[dev].store(sms, std::memory_order_relaxed);
    return sms;
}

/* The RCD kernels' shared-memory sizes, set once per device; this also
 * loads them, so that a pipeline's first frame does not wait for it. */
int prepare_rcd()
{
    constexpr size_t smem = RcdQuads<QTW, QTH, QNT>::floats * sizeof(float);
    static std::atomic<uint64_t> attr_plain{ 0 }, attr_tma{ 0 }, attr_strips{ 0 };
    if (craw_smem_attr(k_develop_rcd_quads, smem, attr_plain) < 0 ||
        craw_smem_attr(k_develop_rcd_quads_tma, smem, attr_tma) < 0 ||
        craw_smem_attr(k_develop_rcd_strips, sizeof(StripSmem), attr_strips) < 0)
        return -5;
    return 0;
}

int launch_rcd(const CRAWKDevelop *k, const CRAWKDevelopIO *io, cudaStream_t s)
{
    constexpr size_t smem = RcdQuads<QTW, QTH, QNT>::floats * sizeof(float);
    if (prepare_rcd() < 0)
        return -5;
    QuadGrid g;
    g.init(k->width, k->height);
    /* Strips unless the colour stage carries the gamut compression (its
     * long chains of MUFU work sit in front of every step's barrier with
     * 16 warps an SM to hide them: the strips take 0.260 ms against the
     * tiles' 0.255 ms at 5760x3240 with it, 0.213 against 0.250 without),
     * or the chroma path (the tiles' epilogue writes its block means). */
    const bool strips = craw_k_rcd_strips == 2 ||
                        (craw_k_rcd_strips == 1 && !(k->color.flags & CRAW_K_COLOR_RGC));
    if (g.interior_x() > 0 && g.interior_y() > 0 && strips && !io->quarter) {
        /* The interior tiles' region as strips. */
        StripGrid sg;
        sg.qx0 = g.c_lo * (QTW / 2);
        sg.nqx = g.interior_x() * (QTW / 2);
        sg.qy0 = g.r_lo * (QTH / 2);
        sg.nqy = g.interior_y() * (QTH / 2);
        /* Segments as tall as one wave of four CTAs an SM allows (a taller
         * segment recomputes less of its passes' first rows), at least 8
         * quad rows. */
        const int gx = (sg.nqx + SOUT - 1) / SOUT;
        const int nseg = (4 * craw_sm_count()) / gx > 1 ? (4 * craw_sm_count()) / gx : 1;
        sg.seg = 4 * ((sg.nqy / 4 + nseg - 1) / nseg);
        sg.seg = sg.seg < 8 ? 8 : sg.seg;
        const dim3 grid(gx, (sg.nqy + sg.seg - 1) / sg.seg);
        k_develop_rcd_strips<<<grid, SNT, sizeof(StripSmem), s>>>(*k, *io, sg);
        if (cudaGetLastError() != cudaSuccess)
            return -5;
    } else if (g.interior_x() > 0 && g.interior_y() > 0) {
        const dim3 grid(g.interior_x(), g.interior_y());
        CUtensorMap tmap;
        if (craw_k_rcd_tma && craw_tmap_u16(io->src, io->src_pitch, k->width, k->height, kBoxW, kBoxH, &tmap))
            k_develop_rcd_quads_tma<<<grid, QNT, smem, s>>>(*k, *io, g, tmap);
        else
            k_develop_rcd_quads<<<grid, QNT, smem, s>>>(*k, *io, g);
        if (cudaGetLastError() != cudaSuccess)
            return -5;
    }
    if (g.border_quads() > 0) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)(g.border_quads() * (QTW / BTW)));
        cfg.blockDim = dim3(256);
        cfg.dynamicSmemBytes = PixelSmem<kRcd, BTW, BTH, 256>::floats * sizeof(float);
        cfg.stream = s;
        cudaLaunchAttribute early[1];
        early[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        early[0].val.programmaticStreamSerializationAllowed = 1;
        /* After an interior launch only: it is the launch the border may
         * overlap. */
        cfg.attrs = early;
        cfg.numAttrs = g.interior_x() > 0 && g.interior_y() > 0 ? 1 : 0;
        if (cudaLaunchKernelEx(&cfg, k_develop_rcd_border, *k, *io, g) != cudaSuccess && cfg.numAttrs) {
            /* A driver that refuses the early start: the plain launch
             * after the interior, the launch's own error cleared. */
            (void)cudaGetLastError();
            cfg.numAttrs = 0;
            (void)cudaLaunchKernelEx(&cfg, k_develop_rcd_border, *k, *io, g);
        }
        if (cudaGetLastError() != cudaSuccess)
            return -5;
    }
    return 0;
}

} // namespace

extern "C" int craw_k_develop_prepare(int method)
{
    (void)craw_sm_count();
    if (method == kRcd)
        return prepare_rcd();
    return 0;
}

extern "C" int craw_k_develop(const CRAWKDevelop *k, const CRAWKDevelopIO *io, int shape,
                              cudaStream_t s)
{
    if (craw_launch_ready() < 0)
        return -5;
    (void)shape;
    switch (k->method) {
    case kBilinear: return launch<kBilinear, 64, 16, 256>(k, io, s);
    case kMhc:      return launch<kMhc, 64, 16, 256>(k, io, s);
    case kRcd:      return launch_rcd(k, io, s);
    default:        return -22;
    }
}
