/*
 * craw-gb300: the frame-development pipeline (reference
 * include/craw/pipeline.h). CRAWPipelineParams and CRAWFrameParams keep the
 * reference's layout and sizes (256 and 264 bytes); the only change to the
 * API is that craw_pipeline_record() takes a cudaStream_t where the
 * reference takes a VkCommandBuffer.
 *
 * The chain a recording enqueues:
 *
 *   src (R16_UNORM RGGB mosaic)
 *     -> [temporal average against the previous frame's state, VST domain]
 *     -> [non-local means on the four CFA planes, VST domain]
 *     -> normalise, white balance, clip at 1.0       (fused into the debayer)
 *     -> bilinear | MHC | RCD debayer to camera RGB
 *     -> [chroma denoise on the quarter-resolution colour differences]
 *     -> [AWB histogram of 8x8 block means]
 *     -> matrix, gain, exposure to the output space, [ACES RGC], [clamp]
 *   dst (RGBA16F or RGBA32F)
 *
 * The reference's lens, false-colour, highlight, defringe and sharpening
 * stages are outside this library; their pipeline flags are refused by
 * craw_pipeline_create() with CRAW_ERROR(ENOTSUP) and their frame fields
 * are ignored.
 */
#ifndef CRAW_PIPELINE_H
#define CRAW_PIPELINE_H

#include <craw/cuda.h>
#include <craw/profile.h>
#include <craw/awb.h>
#include <craw/lens.h>

typedef struct CRAWPipeline CRAWPipeline;

enum CRAWDebayer {
    CRAW_DEBAYER_BILINEAR = 0,  /* 3x3 averages */
    CRAW_DEBAYER_MHC,           /* Malvar-He-Cutler 5x5 */
    CRAW_DEBAYER_RCD,           /* ratio-corrected demosaicing */
    CRAW_DEBAYER_NB,
};

/* Pipeline flags; values are the reference's (pipeline.h:47-170). */
#define CRAW_PIPELINE_FLAG_AWB_HISTOGRAM            (1 << 0)
#define CRAW_PIPELINE_FLAG_DENOISE                  (1 << 1)
#define CRAW_PIPELINE_FLAG_LENS                     (1 << 2)  /* not built: ENOTSUP */
#define CRAW_PIPELINE_FLAG_FALSE_COLOR              (1 << 3)  /* not built: ENOTSUP */
#define CRAW_PIPELINE_FLAG_CHROMA_DENOISE           (1 << 4)
/* Rebuild clipped highlights before the debayer (reference pipeline.h:86-103):
 * a quarter-resolution colour field of the unclipped neighbourhood and its
 * pyramid predict the channels that clipped; the rebuilt mosaic (fp16) may
 * exceed the balanced clip point. Switched per frame by
 * CRAW_FRAME_FLAG_HIGHLIGHT_RECONSTRUCTION. Not with CRAW_IMPL_PLAIN. */
#define CRAW_PIPELINE_FLAG_HIGHLIGHT_RECONSTRUCTION (1 << 5)
#define CRAW_PIPELINE_FLAG_DEFRINGE                 (1 << 6)  /* not built: ENOTSUP */
#define CRAW_PIPELINE_FLAG_TEMPORAL_DENOISE         (1 << 7)
#define CRAW_PIPELINE_FLAG_SHARPEN                  (1 << 8)  /* not built: ENOTSUP */
#define CRAW_PIPELINE_FLAG_PROFILE                  (1 << 9)

/* Extension, no counterpart in the reference: keep the camera RGB
 * intermediate (after the debayer and the chroma denoise, exactly what the
 * AWB histogram and the colour stage read) and the mosaic the debayer read
 * (the denoised R16_UNORM one, or the rebuilt R16F one after a highlight
 * reconstruction) in device memory where craw_pipeline_get_intermediate()
 * can hand them out.
 * Without it the fused kernels never write the intermediate at all. */
#define CRAW_PIPELINE_FLAG_KEEP_INTERMEDIATE        (1 << 16)

/* Extension, no counterpart in the reference: skip the autotuner. By
 * default craw_pipeline_create() of a denoising pipeline times every tile
 * shape of the denoise kernel on a scratch frame of the pipeline's size and
 * keeps the fastest (cached per size for the process); with this flag the
 * default shape is used. */
#define CRAW_PIPELINE_FLAG_NO_AUTOTUNE              (1 << 17)

/* Extension, no counterpart in the reference: round the denoised codes as
 * a double-precision evaluation of the filter does. The denoise re-encodes
 * its result to 16-bit codes, and a float evaluation (the reference's own
 * CPU and GPU code, and this library's default) rounds about 0.03 % of the
 * samples to the neighbouring code of the double one; one code is up to
 * 1e-2 of a dark pixel, so the developed frame is then up to a few 1e-3
 * from an FP64 run. With this flag the samples whose float code lies near
 * a rounding boundary are evaluated again (a float evaluation that bounds
 * its own error, double-float arithmetic for what it cannot settle), and
 * the denoised mosaic equals the double evaluation's code for code: the
 * developed frame is then within 1e-3 of FP64. Costs about 0.15 ms a
 * 5760x3240 frame on a GB300 (0.04 ms in the denoise, which marks the
 * samples and centres its weighted sums, 0.11 ms in the two rounding
 * kernels); 10 MB of device memory at that size. Applies
 * to the spatial denoise without a temporal history; the temporal modes
 * round as the float path does. */
#define CRAW_PIPELINE_FLAG_EXACT_ROUNDING           (1 << 18)

#define CRAW_FALSE_COLOR_MAX_PASSES 5
#define CRAW_SHARPEN_MAX_RADIUS     2.0f
#define CRAW_SHARPEN_MAX_ITERATIONS 100
#define CRAW_PIPELINE_PROFILE_SLOTS 4

/* Storage of the intermediates (extension; zero is the default). FP32
 * keeps every intermediate in float. FP16 rounds the camera RGB
 * intermediate to half floats (and stores it, and the chroma quarter
 * planes, as half where they go to memory), as the reference's RGBA16F
 * intermediate does; the VST planes, NLM weights and patch distances, the
 * colour matrices, the inverse VST, the temporal state and agreement test
 * and the histogram binning stay FP32. */
enum CRAWStorage {
    CRAW_STORAGE_FP32 = 0,
    CRAW_STORAGE_FP16,
};

/* Kernel set (extension; zero is the default). FUSED is the tuned
 * pipeline. PLAIN runs the same algorithm as one straightforward FP32
 * kernel per stage, each reading and writing full-resolution FP32 images
 * in device memory: the baseline the fused pipeline is measured against. */
enum CRAWImpl {
    CRAW_IMPL_FUSED = 0,
    CRAW_IMPL_PLAIN,
};

/* Fixed configuration of a pipeline; 256 bytes as in the reference
 * (pipeline.h:174-201). */
typedef struct CRAWPipelineParams {
    uint32_t width, height;     /* both even, at least 8 (16 with denoise) */
    enum CRAWCfa cfa;           /* CRAW_CFA_RGGB */
    enum CRAWDebayer debayer;
    enum CRAWColorSpace out_space;   /* default; a frame may override it */
    CRAWFormat out_format;      /* CRAW_FORMAT_RGBA16F, CRAW_FORMAT_RGBA32F or (an extension)
                                 * CRAW_FORMAT_RGB32F */
    uint32_t flags;             /* CRAW_PIPELINE_FLAG_* */
    uint32_t nb_awb_slots;      /* host-visible histogram copies, 1..4 (0 = 1) */

    /* Extensions, zero for the defaults. */
    enum CRAWStorage storage;
    enum CRAWImpl impl;

    uint8_t padding[256 - 10*4];
} CRAWPipelineParams;

/* Frame flags; values are the reference's (pipeline.h:206-260). */
#define CRAW_FRAME_FLAG_CLAMP_NEGATIVE           (1 << 0)
#define CRAW_FRAME_FLAG_LENS_KEEP_ALL            (1 << 1)  /* ignored */
#define CRAW_FRAME_FLAG_NO_GAMUT_COMPRESSION     (1 << 2)
#define CRAW_FRAME_FLAG_HIGHLIGHT_RECONSTRUCTION (1 << 3)  /* needs the pipeline flag */
#define CRAW_FRAME_FLAG_TEMPORAL_RESET           (1 << 4)

/* Per-frame settings; 264 bytes, field for field the reference's
 * (pipeline.h:251-407). */
typedef struct CRAWFrameParams {
    const CRAWProfile *profile;

    enum CRAWWbMode wb_mode;
    CRAWIlluminant  illuminant;      /* for CRAW_WB_REBALANCE */

    float exposure_stops;            /* on top of the profile's gain */
    uint32_t flags;                  /* CRAW_FRAME_FLAG_* */

    enum CRAWColorSpace out_space;   /* used when out_space_set */
    bool out_space_set;

    /* Spatial NLM strength in units of the modelled noise; 0 skips it. */
    float denoise_strength;

    /* Used when a > 0; otherwise the profile's table at as_shot_ei. */
    CRAWNoiseModel noise_override;

    uint32_t false_color_passes;     /* ignored (stage not built) */

    /* Chroma denoise blend, 0..1; 0 skips it, > 1 is EINVAL. */
    float denoise_chroma_strength;

    CRAWLensCorrection lens;         /* ignored (stage not built) */
    float defringe_strength;         /* ignored (stage not built) */

    /* Temporal alpha_max, 0..1; 0 skips it, > 1 is EINVAL. With replay
     * set the recording develops the last recorded frame again. */
    float denoise_temporal_strength;
    bool denoise_temporal_replay;

    float    sharpen_radius;         /* ignored (stage not built) */
    uint32_t sharpen_iterations;     /* ignored */
    float    sharpen_contrast;       /* ignored */
    float    rotation;               /* ignored */

    uint8_t padding[256 - 4*4 - 8 - 12 - 64 - 8 - 4 - 4 - 4 - 4 - 4 - 12 - 4];
} CRAWFrameParams;

/* Defaults: RGGB, RCD, XYZ D65, RGBA16F, one AWB slot, no flags, FP32
 * storage, fused kernels; width and height 0. Reference pipeline.h:411
 * (lib/pipeline.c:543-553). */
CRAW_API void craw_pipeline_params_init(CRAWPipelineParams *p);

/* Defaults: as shot, the pipeline's space, no exposure change, every
 * optional stage off; profile NULL. Reference pipeline.h:418
 * (lib/pipeline.c:555-565). */
CRAW_API void craw_frame_params_init(CRAWFrameParams *fp);

/* Allocates the pipeline's intermediates, state and histogram slots for
 * exactly width x height. Reference pipeline.h:422-424. */
CRAW_API int craw_pipeline_create(CRAWContext *ctx,
                                  const CRAWPipelineParams *params,
                                  CRAWPipeline **pipe);

/* Frees everything the pipeline owns. Work it enqueued must have
 * completed. Reference pipeline.h:426. */
CRAW_API void craw_pipeline_free(CRAWPipeline **pipe);

/* Enqueues the whole chain on `stream`. src is R16_UNORM and dst the
 * pipeline's out_format, both width x height, not aliasing. The pipeline's
 * intermediates are single-buffered: recordings onto one stream run in
 * order; recordings of one pipeline onto different streams must be
 * ordered by the caller with events.
 *
 * Temporal state (CRAW_PIPELINE_FLAG_TEMPORAL_DENOISE), the reference's
 * rules (pipeline.h:457-484): nothing is valid after creation or a
 * CRAW_FRAME_FLAG_TEMPORAL_RESET; a recording without replay reads what
 * the last recording wrote and writes the other set; a replay reads the
 * set the last recording read and rewrites the one it wrote, bit for bit
 * the same for the same parameters; a next frame with the pass off leaves
 * no state, a replay with it off leaves the state alone; a recording that
 * fails changes nothing.
 *
 * Errors: CRAW_ERROR(EINVAL) for arguments and ranges, CRAW_ERROR(ENOTSUP)
 * for a missing noise model, CRAW_ERROR(EIO) when a CUDA launch fails.
 * Replaces reference pipeline.h:485-487. */
CRAW_API int craw_pipeline_record(CRAWPipeline *pipe, cudaStream_t stream,
                                  const CRAWImage *src, const CRAWImage *dst,
                                  const CRAWFrameParams *fp);

/* The histogram of the last recording (or of the one `frames_back`
 * recordings ago, up to nb_awb_slots - 1), in pinned host memory. Valid
 * once the caller has synchronised with that recording's stream.
 * CRAW_ERROR(EINVAL) without CRAW_PIPELINE_FLAG_AWB_HISTOGRAM.
 * Reference pipeline.h:494-501. */
CRAW_API int craw_pipeline_get_awb_histogram(CRAWPipeline *pipe,
                                             CRAWAwbHistogram *out);
CRAW_API int craw_pipeline_get_awb_histogram_n(CRAWPipeline *pipe, uint32_t frames_back,
                                               CRAWAwbHistogram *out);

typedef struct CRAWStageTime {
    const char *name;   /* kernel name, owned by the pipeline */
    uint32_t count;     /* launches of it in the recording */
    double   ms;        /* their GPU time, summed */
} CRAWStageTime;

/* GPU time per stage of the last recording (or `frames_back` ago, up to
 * CRAW_PIPELINE_PROFILE_SLOTS - 1), from CUDA events around every launch.
 * Returns the number of entries and writes up to `max` of them;
 * CRAW_ERROR(EAGAIN) while that recording has not finished (checked with
 * cudaEventQuery, never blocking); CRAW_ERROR(EINVAL) without
 * CRAW_PIPELINE_FLAG_PROFILE. Reference pipeline.h:523-529. */
CRAW_API int craw_pipeline_get_stage_times(CRAWPipeline *pipe, CRAWStageTime *out,
                                           uint32_t max);
CRAW_API int craw_pipeline_get_stage_times_n(CRAWPipeline *pipe, uint32_t frames_back,
                                             CRAWStageTime *out, uint32_t max);

/* Extension, no counterpart in the reference: device views of the last
 * recording's camera RGB intermediate (RGBA32F, or RGBA16F with
 * CRAW_STORAGE_FP16) and denoised mosaic (R16_UNORM; data NULL when that
 * recording did not denoise). Needs CRAW_PIPELINE_FLAG_KEEP_INTERMEDIATE. */
CRAW_API int craw_pipeline_get_intermediate(CRAWPipeline *pipe, CRAWImage *rgb,
                                            CRAWImage *mosaic);

/* Extension, no counterpart in the reference: device views of the
 * temporal state the last recording wrote: the level of every sample
 * (R32F, one float per mosaic sample, as the reference's R32F state image)
 * and the square root of the variance left in it (one byte per sample,
 * value / 255, as the reference's R8_UNORM image). CRAW_ERROR(EAGAIN)
 * when no state is valid. */
CRAW_API int craw_pipeline_get_temporal_state(CRAWPipeline *pipe, CRAWImage *level,
                                              CRAWImage *sqrt_var);

/* Extension, no counterpart in the reference: the tile shapes the
 * autotuner chose for the denoise kernel, without and with a temporal
 * history (0: 2 columns x 8 rows a thread, 1: 2 x 4; 2 and 3: the same
 * with the search in packed f32x2 arithmetic). */
CRAW_API int craw_pipeline_get_kernel_config(CRAWPipeline *pipe, int *denoise_shape,
                                             int *denoise_shape_history);

#endif /* CRAW_PIPELINE_H */
