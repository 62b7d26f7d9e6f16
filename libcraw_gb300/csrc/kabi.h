/*
 * The thin C ABI between the C23 host library (csrc/host) and the sm_103a
 * kernels (csrc/kernels). Plain structs of per-frame constants and plain
 * device pointers; every launch is asynchronous on the given stream and
 * returns 0 or a negative errno (CRAW_ERROR(EIO) when CUDA refuses the
 * launch). Internal: not installed, not part of the public API.
 */
#ifndef CRAW_KABI_H
#define CRAW_KABI_H

#include <stddef.h>
#include <stdint.h>

#include <cuda_runtime_api.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ denoise */

#define CRAW_K_DN_SPATIAL  1   /* non-local means */
#define CRAW_K_DN_TEMPORAL 2   /* recursive average; writes the next state */
#define CRAW_K_DN_HISTORY  4   /* the previous state is valid: read it */

/* Per-frame constants of the temporal + VST + NLM pass (the reference's
 * CRAWDenoisePush, lib/pipeline.c:1414-1467). */
typedef struct CRAWKDenoise {
    int32_t pw, ph;                  /* plane size: mosaic size / 2 */
    float black[4], inv_range[4], range[4];   /* per quad site */
    float gat_a, gat_c, gat_sc, gat_fwd, gat_inv, gat_off, gat_t0;
    float inv_h2;                    /* 1 / strength^2 of the NLM */
    float t_alpha, t_inv_h2;         /* temporal alpha_max and 1 / ht^2 */
    float guard_lo, guard_inv;       /* highlight guard ramp */
    int32_t mode;                    /* CRAW_K_DN_* */
} CRAWKDenoise;

typedef struct CRAWKDenoiseIO {
    const uint16_t *src;  size_t src_pitch;   /* bytes */
    uint16_t *dst;        size_t dst_pitch;
    const float *lvl_prev; float *lvl_next;   size_t lvl_pitch;
    const uint8_t *var_prev; uint8_t *var_next; size_t var_pitch;
} CRAWKDenoiseIO;

/* Tile shapes of the fused denoise kernel, chosen by the autotuner. */
enum CRAWKDenoiseShape {
    CRAW_K_DN_SHAPE_2x8 = 0,     /* a thread filters 2 columns x 8 rows */
    CRAW_K_DN_SHAPE_2x4,         /* 2 columns x 4 rows */
    CRAW_K_DN_SHAPE_2x8_X2,      /* 2x8 with the search in packed f32x2 arithmetic */
    CRAW_K_DN_SHAPE_2x4_X2,      /* 2x4 with the search in packed f32x2 arithmetic */
    CRAW_K_DN_SHAPE_NB,
};

/* Exact rounding of the denoised mosaic. The denoise re-encodes its result
 * to 16-bit codes (reference lib/ref/ref_denoise.c:318-323), so a float
 * evaluation and a double one disagree by a code wherever the value lies
 * within the float error of a rounding boundary. The denoise kernel marks
 * every sample whose float code position x lies within
 * band = c0 + c2 t^2 of a boundary (t: the sample's filtered value in the
 * stabilised domain; the float error grows as t^2 because the codes per
 * unit of t and the rounding of t both grow with t), one bit per sample;
 * craw_k_denoise_round settles the marked samples and rewrites their codes
 * as the double evaluation rounds them. */
typedef struct CRAWKRound {
    uint32_t *flags;    /* CRAW_K_ROUND_WORDS(pw, ph) words; NULL: no marking */
    uint32_t *count2;   /* [0] the length of the list of undecided samples,
                         * [1] the rounding's work counter, [2] the number
                         * of marked samples: the denoise kernel zeroes
                         * all three */
    float c0, c2;
} CRAWKRound;

/* Marks of plane p, plane row y, columns 32 w .. 32 w + 31: word
 * (p * ph + y) * CRAW_K_ROUND_WW(pw) + w, bit b < 16 for column
 * 32 w + 2 b, bit 16 + b for column 32 w + 2 b + 1 (the layout of a
 * half-warp's two columns a lane). */
#define CRAW_K_ROUND_WW(pw) (((pw) + 31) / 32)
#define CRAW_K_ROUND_WORDS(pw, ph) ((size_t)4 * (size_t)(ph) * (size_t)CRAW_K_ROUND_WW(pw))

/* The constants of the re-evaluation. Each {hi, lo} is a double value of
 * the reference's double-precision arithmetic split into two floats
 * (lib/ref/ref_denoise.c:25-58, 109-154, 298-324 evaluated in double);
 * the plain floats serve the float decision stage. */
typedef struct CRAWKDenoiseExact {
    int32_t pw, ph, mode;                   /* mode: CRAW_K_DN_* of the frame */
    float black[4][2], range[4][2], inv_range[4][2];
    float inv65535[2];
    float gat_a;                            /* the model's a (a float: exact) */
    float gat_c[2], gat_isc[2], gat_sc[2], gat_fwd[2], gat_inv[2], gat_off[2], gat_t0[2];
    float k_nlm[2];                         /* (1/9) / strength^2 */
    float guard_lo[2], guard_inv[2];
    /* Decision stage, per quad site: u = raw k1 - k0; the stabilised value
     * of a code is t = sqrt(q raw + beta) (q = 4 / (65535 range a),
     * beta = 4 c / a^2 - 4 black / (a range)), so q also turns a code
     * difference into t^2 - t'^2; k2 = 65535 range a / 4 turns
     * m^2 - m'^2 back into codes. */
    float k1[4], k0[4], q[4], k2[4];
    float qq[4][2], beta[4][2];             /* q and beta as double-floats */
    float kn, c1, c0;                       /* 1/(9 h^2); -log2(e) kn, 2 log2(e) */
    uint32_t dark_code;                     /* codes at or below it (black and the code
                                             * above) go to the double-float stage */
    int32_t decide;                         /* 0: every marked sample to the exact stage */
} CRAWKDenoiseExact;

/* The statistics craw_k_denoise_round keeps (device words, never reset by
 * the kernels): [0] samples the decision stage examined, [1] codes
 * changed, [2] records written, [3] samples listed for the double-float
 * stage; then for each changed code, up to CRAW_K_ROUND_RECORDS, four
 * floats: the sample's t and x, the distance of the exact x from its
 * rounding boundary (the float evaluation was off by at least that much),
 * the plane. */
#define CRAW_K_ROUND_RECORDS 4096
#define CRAW_K_ROUND_STATS_BYTES (16 + 16 * CRAW_K_ROUND_RECORDS)

/* Entries of each of the rounding's two lists (the marked samples, then
 * the undecided ones), for a frame of plane size pw x ph. */
#define CRAW_K_ROUND_LIST(pw, ph) (((size_t)4 * (pw) * (ph)) / 16 + 65536)

/* rd: NULL, or the marking of samples near a code boundary. err: NULL,
 * or a device word for CRAW_K_ERR_* bits. */
int craw_k_denoise(const CRAWKDenoise *k, const CRAWKDenoiseIO *io, int shape,
                   const CRAWKRound *rd, uint32_t *err, cudaStream_t s);

/* 1 (default): the packed spatial denoise kernels bring each interior
 * tile's mosaic in with one TMA tile copy; 0: with plain loads
 * (craw_debug_denoise_tma). */
extern int craw_k_dn_tma;

/* Settles the samples `rd->flags` marks (of the frame k/io describe, whose
 * denoised mosaic io->dst the denoise kernel wrote) and rewrites their
 * codes in io->dst as a double evaluation rounds them: the marks are
 * gathered into a list (the first CRAW_K_ROUND_LIST entries of `list`;
 * with more marks than that the decision stage walks the bit map
 * instead), a float decision stage with a bound on its own error settles
 * most of them, and the rest (rd->count2[0] entries of the second
 * CRAW_K_ROUND_LIST entries of `list`) are evaluated in double-float
 * arithmetic. Spatial filtering without a temporal history only
 * (e->mode). */
int craw_k_denoise_round(const CRAWKDenoise *k, const CRAWKDenoiseExact *e, const CRAWKDenoiseIO *io,
                         const CRAWKRound *rd, uint32_t *list, uint32_t *stats, int sm_count,
                         cudaStream_t s);

/* The plain baseline: one kernel for the transform and the temporal
 * average into full FP32 planes (`t` and `var`, 4 planes of pw x ph each),
 * and one straightforward NLM kernel reading them. */
int craw_k_plain_denoise(const CRAWKDenoise *k, const CRAWKDenoiseIO *io,
                         float *t, float *var, cudaStream_t s);

/* ------------------------------------------------------------ develop */

#define CRAW_K_COLOR_CLAMP 1u        /* clamp negatives */
#define CRAW_K_COLOR_RGC   2u        /* ACES 1.3 gamut compression */

/* The colour stage (the reference's CRAWColorPush, lib/pipeline.c:1905-1931). */
typedef struct CRAWKColor {
    float m[3][3];        /* rows of M_out * cam_to_xyz * gain * 2^stops */
    float gc_thr[3], gc_scl[3], gc_pwr, gc_inv_pwr;
    uint32_t flags;       /* CRAW_K_COLOR_* */
} CRAWKColor;

typedef struct CRAWKDevelop {
    int32_t width, height;
    float black[4], range[4], inv_range[4], wbs[4];   /* per site; wbs = gain of the site's channel */
    float clip;                         /* 1.0 */
    int32_t method;                     /* CRAW_DEBAYER_* */
    int32_t fp16;                       /* intermediate values rounded to half */
    CRAWKColor color;
    float awb_wb[3];                    /* white balance divided out of the block means */
} CRAWKDevelop;

/* One record per 8x8 block of the AWB histogram. 0 means "no sample".
 * Otherwise bit 46 set, bits 0-13 the bin, 14-29 the 16.16 weight
 * min(g, 0.5), 30-45 the 16.16 weight g^4. Blocks whose bin is within
 * rounding of a bin edge are not binned on the device: their raw ratios go
 * to the deferred list and the host bins them with its own logf, so the
 * histogram is bit for bit the CPU builder's. The host copy of a slot
 * holds the first CRAW_K_AWB_DEFER_MAX; more are read from the device
 * list when the histogram is asked for. */
#define CRAW_K_AWB_VALID (1ull << 46)
#define CRAW_K_AWB_DEFER_MAX 4096

typedef struct CRAWKAwbDeferred {
    float rr, bb, g;
    uint32_t pad;
} CRAWKAwbDeferred;

typedef struct CRAWKAwbOut {
    uint64_t *rec;                 /* ceil(w/8) * ceil(h/8) records, or NULL */
    CRAWKAwbDeferred *deferred;    /* room for one entry per 8x8 block of the frame */
    uint32_t *nb_deferred;         /* counter, zeroed before the frame */
} CRAWKAwbOut;

/* Layouts of an RGB image a kernel stores: four floats (alpha 1), four
 * half floats (alpha 1), three floats. */
#define CRAW_K_OUT_RGBA32F 0
#define CRAW_K_OUT_RGBA16F 1
#define CRAW_K_OUT_RGB32F 2

typedef struct CRAWKDevelopIO {
    const uint16_t *src; size_t src_pitch;
    int32_t src_f16;                                    /* src holds fp16 values already
                                                         * prepped (the rebuilt highlights) */
    void *dst; size_t dst_pitch; int32_t dst_fmt;       /* NULL: no colour stage; dst_fmt a
                                                         * CRAW_K_OUT_* layout */
    void *inter; size_t inter_pitch;                    /* NULL: not kept */
    void *quarter; size_t quarter_pitch;                /* chroma: block means out */
    CRAWKAwbOut awb;
    uint32_t *err;                                      /* device word a kernel ORs
                                                         * CRAW_K_ERR_* into; NULL: none */
} CRAWKDevelopIO;

/* Kernel error bits: a wait on a TMA copy that did not complete within
 * its bound (the tile is skipped); an index outside its buffer, found by
 * the checks of a CRAW_DEBUG_BOUNDS build (the access is skipped). */
#define CRAW_K_ERR_TMA_WAIT 1u
#define CRAW_K_ERR_BOUNDS 2u

/* Prep + debayer + (colour to dst | chroma block means) + AWB records +
 * optional intermediate, in one kernel. */
int craw_k_develop(const CRAWKDevelop *k, const CRAWKDevelopIO *io, int shape,
                   cudaStream_t s);

/* Readies the develop kernels of a debayer method on the current device
 * (their launch attributes, which also loads them): called when a
 * pipeline is created, so that its first frame starts at once. 0 or -5. */
int craw_k_develop_prepare(int method);

/* 1 (default): the RCD's interior tiles bring their mosaic in with one TMA
 * tile copy; 0: with plain loads (craw_debug_rcd_tma). */
extern int craw_k_rcd_tma;

/* The RCD's interior by 64x16 tiles (0), by strips (one quad column a
 * thread walking down a segment of quad rows) unless the colour stage
 * has the gamut compression (1, the default), or by strips wherever they
 * apply (2): craw_debug_rcd_strips. The two give the same bits. */
extern int craw_k_rcd_strips;

/* ------------------------------------------------------------- chroma */

typedef struct CRAWKChroma {
    int32_t width, height, qw, qh;
    float strength;
    int32_t fp16;
    uint32_t *err;                  /* device word for CRAW_K_ERR_* bits; NULL: none */
} CRAWKChroma;

/* 9x9 joint bilateral on the quarter grid: q -> qf. */
int craw_k_chroma_blur(const CRAWKChroma *c, const void *q, size_t q_pitch,
                       void *qf, size_t qf_pitch, cudaStream_t s);

/* The band back into every pixel of the intermediate, then the AWB records
 * and the colour stage; `inter_out` (optional) keeps the result. */
int craw_k_chroma_up_color(const CRAWKDevelop *k, const CRAWKChroma *c,
                           const void *inter, size_t inter_pitch,
                           const void *q, const void *qf, size_t q_pitch,
                           void *dst, size_t dst_pitch, int dst_fmt,
                           void *inter_out, const CRAWKAwbOut *awb, cudaStream_t s);

/* ---------------------------------------------------------------- awb */

/* Folds `n` block records into the three 128^2 histograms (zeroed by the
 * caller), through shared-memory histograms with warp-aggregated atomics. */
int craw_k_awb_reduce(const uint64_t *rec, uint32_t n, uint32_t *hist, cudaStream_t s);

/* ------------------------------------------------------ highlights */

/* The highlight reconstruction of one frame: the mosaic's sites as
 * u = (raw/65535 - black) * inv_range, their clip ramp a, a pyramid of
 * log-chroma colour fields from the unclipped quads, and the rebuilt,
 * balanced mosaic (u * gain, lifted near the clip) as fp16. */
#define CRAW_K_HL_LEVELS 16

typedef struct CRAWKHighlight {
    int32_t width, height;           /* mosaic; qw = width / 2, qh = height / 2 */
    float black[4], inv_range[4];    /* per quad site */
    float wb[3];                     /* gains of R, G, B */
    int32_t nb_levels;
    int32_t lw[CRAW_K_HL_LEVELS], lh[CRAW_K_HL_LEVELS];
    int64_t off[CRAW_K_HL_LEVELS];   /* float4 offset of each level */
} CRAWKHighlight;

typedef struct CRAWKHighlightIO {
    const uint16_t *src; size_t src_pitch;
    uint16_t *dst; size_t dst_pitch;  /* fp16 bits, balanced mosaic */
    void *levels;                   /* float4 texels (c0, c1, weight, 0) */
    uint32_t *err;                  /* device word for CRAW_K_ERR_* bits; NULL: none */
} CRAWKHighlightIO;

/* Level sizes and offsets of a width x height frame into `k`; returns the
 * float4 texels of the whole pyramid, or -1 when it needs more than
 * CRAW_K_HL_LEVELS levels. */
int64_t craw_k_highlight_levels(int32_t width, int32_t height, CRAWKHighlight *k);

int craw_k_highlights(const CRAWKHighlight *k, const CRAWKHighlightIO *io, cudaStream_t s);

/* ------------------------------------------------- noise-model estimation */

/* The device half of craw_noise_estimate(): every interior sample of the
 * four CFA planes gets its |3x3 high-pass| and a bin by its 9x9 plane
 * mean; each bin's count, the exact sum of its means and its median
 * |high-pass| come back in CRAWKNoiseBin. The host fits the line. */
typedef struct CRAWKNoise {
    int32_t width, height;       /* mosaic, both even */
    float black[4], white[4];    /* profile levels per quad site */
    int32_t nb_bins;
    float max_level;
} CRAWKNoise;

typedef struct CRAWKNoiseBin {
    uint32_t count;       /* samples in the bin */
    uint32_t median;      /* bits of the (count / 2)-th smallest |high-pass| */
    /* The sum of the bin's means x 2^64: each mean as a 96-bit integer
     * (exact for means >= 2^-40, up to 2^31), its three 32-bit words
     * summed separately: sum = sum[2] 2^64 + sum[1] 2^32 + sum[0]. */
    uint64_t sum[3];
} CRAWKNoiseBin;

/* Device scratch craw_k_noise_bins needs, in bytes. */
size_t craw_k_noise_scratch(int32_t width, int32_t height, int32_t nb_bins);

/* Fills bins[0 .. nb_bins) (device memory) on stream s. */
int craw_k_noise_bins(const CRAWKNoise *k, const uint16_t *src, size_t src_pitch, void *scratch,
                      CRAWKNoiseBin *bins, cudaStream_t s);

/* The least-trimmed-squares cost of the line through every pair of bins
 * i < j (the sum of the `keep` smallest squared log residuals, added in
 * ascending order): cost[i * nb + j], +inf where the pair gives no
 * physical line. m, v: the bins' mean level and variance; lv = ln v,
 * computed on the host. All device arrays; nb <= CRAW_K_NOISE_MAX_BINS. */
#define CRAW_K_NOISE_MAX_BINS 512
int craw_k_noise_lts(const double *m, const double *v, const double *lv, int32_t nb, int32_t keep,
                     double *cost, cudaStream_t s);

/* ------------------------------------------------------------- batch */

/* One frame of a batch: its constants and buffers, how many tiles each
 * phase has, and where its tiles start in each phase's item list. */
typedef struct CRAWKBatchFrame {
    CRAWKDenoise dn;            /* dn.mode == 0: the frame is not denoised */
    CRAWKDenoiseIO dio;
    CRAWKDevelop dv;
    CRAWKDevelopIO vio;         /* vio.src is dio.dst when denoised */
    int32_t dn_tx, dn_ty, dn_first;
    int32_t dv_tx, dv_ty, dv_first;
} CRAWKBatchFrame;

/* Denoise tile shapes of the batch kernel (256 threads). */
enum CRAWKBatchShape {
    CRAW_K_BATCH_DN_2x4 = 0,    /* 2 columns x 4 rows a thread, 32x16 tiles, packed f32x2 */
    CRAW_K_BATCH_DN_2x8,        /* 2 x 8, 32x32 tiles, packed f32x2 */
    CRAW_K_BATCH_DN_NB,
};

/* Tiles per phase for a frame of w x h with a denoise shape. */
void craw_k_batch_tiles(int32_t w, int32_t h, int shape, int32_t *dn_tx, int32_t *dn_ty,
                        int32_t *dv_tx, int32_t *dv_ty);

/* The frames of one batch launch, passed by value as a kernel parameter
 * (30 KB of the 32 KB a launch may carry): the kernels read a frame's
 * constants from the parameter bank, not from memory they must copy. */
#define CRAW_K_BATCH_MAX 64
typedef struct CRAWKBatchTable {
    CRAWKBatchFrame f[CRAW_K_BATCH_MAX];
} CRAWKBatchTable;

/* Develops the first `nb` frames of `table` (host memory, copied into the
 * launch) in one persistent launch: every denoise tile of every frame, a
 * grid-wide barrier, every develop tile (`fused`); or as two persistent
 * launches. Grid: as many CTAs as fit on the device at once. All frames
 * use the same debayer, RCD or MHC or bilinear, `method`. */
int craw_k_batch(const CRAWKBatchTable *table, int32_t nb, int32_t dn_items, int32_t dv_items,
                 int method, int shape, int fused, cudaStream_t s);

/* Points every batch kernel node of an instantiated graph (one captured
 * craw_k_batch call) at a new table and item counts. */
int craw_k_batch_update(cudaGraphExec_t exec, cudaGraph_t graph, const CRAWKBatchTable *table,
                        int32_t nb, int32_t dn_items, int32_t dv_items);

/* ------------------------------------------------------- plain baseline */

/* One straightforward FP32 kernel per stage, each through device memory:
 * prep into `v` (w*h floats), debayer into `inter` (RGBA32F, pitch in
 * bytes) using `scratch` (7 * w * h floats for RCD), chroma with `q`, `qf`
 * (qw*qh*4 floats each), AWB by global atomics, colour into dst. */
int craw_k_plain_develop(const CRAWKDevelop *k, const CRAWKDevelopIO *io,
                         const CRAWKChroma *chroma, float *v, float *inter,
                         size_t inter_pitch, float *scratch, float *q, float *qf,
                         uint32_t *hist, cudaStream_t s);

#ifdef __cplusplus
}
#endif

#endif /* CRAW_KABI_H */
