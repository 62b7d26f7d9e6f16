/*
 * Internals of the C23 host library: the context and pipeline objects and
 * the host-side helpers the pipeline shares with the public functions.
 */
#ifndef CRAW_INTERNAL_H
#define CRAW_INTERNAL_H

#include <stdbool.h>
#include <stdint.h>

#include <craw/pipeline.h>

#include "../kabi.h"

struct CRAWContext {
    CRAWContextOptions opts;
    int device;
    int sm_count;
    cudaMemPool_t pool;
    bool own_pool;
    cudaStream_t stream;     /* the context's own stream, for allocation only */
};

/* ACES 1.3 RGC constants (thresholds and solved scales). */
typedef struct CRAWGamutCompress {
    float thr[3];
    float scl[3];
    float pwr;
    float inv_pwr;
} CRAWGamutCompress;

void craw_gamut_compress_params(CRAWGamutCompress *g);

/* Device allocation from the context's pool on its own stream; counts
 * allocations so a test can make the k-th one fail. */
int craw_dev_alloc(CRAWContext *ctx, void **ptr, size_t bytes);
void craw_dev_free(CRAWContext *ctx, void *ptr);
int craw_dev_sync(CRAWContext *ctx);

/* craw_debug_force_denoise_shape(): -1, or the shape every new pipeline uses. */
extern int craw_forced_denoise_shape;

/* Per-frame constants (frame.c). */
/* Bytes a pixel of an image format takes; whether a format can be an
 * output of the colour stage (RGBA16F, RGBA32F, RGB32F); and the kernels'
 * CRAW_K_OUT_* layout of such a format. */
size_t craw_format_bpp(CRAWFormat fmt);
bool craw_is_out_format(CRAWFormat fmt);
int craw_out_layout(CRAWFormat fmt);
int craw_image_check(CRAWContext *ctx, const CRAWImage *img, CRAWFormat fmt, uint32_t w, uint32_t h,
                     const char *what);
bool craw_images_overlap(const CRAWImage *a, const CRAWImage *b);
int craw_develop_consts(CRAWContext *ctx, uint32_t w, uint32_t h, int debayer, bool fp16,
                        enum CRAWColorSpace default_space, const CRAWFrameParams *fp, CRAWKDevelop *dk);
int craw_denoise_consts(CRAWContext *ctx, uint32_t w, uint32_t h, const CRAWFrameParams *fp, int mode,
                        CRAWKDenoise *k, CRAWKDenoiseExact *ex);
/* The constants of the exact rounding (ex), from the float constants k of
 * the same frame, its profile, noise model and strength. */
void craw_denoise_exact_consts(const CRAWKDenoise *k, const CRAWProfile *prof, float a, float b, float strength,
                               CRAWKDenoiseExact *ex);
/* The marking band of the exact rounding for the frame k describes,
 * `scale` times the float path's error bound (1e6 and above: every
 * sample); rd->flags and rd->count2 are left alone. */
void craw_denoise_round_band(const CRAWKDenoise *k, float scale, CRAWKRound *rd);

/* craw_debug_denoise_round(): the scale of the marking band (0: the exact
 * rounding is off); craw_debug_denoise_round_decide(): 0 sends every
 * marked sample to the double-float stage. */
extern float craw_round_scale;
extern int craw_round_decide;

/* Bins one deferred AWB block on the host, with the CPU builder's
 * arithmetic (lib/awb.c:270-291 of the reference). */
void craw_awb_bin_host(float rr, float bb, float g, uint32_t *count, uint32_t *weight,
                       uint32_t *weight_bright);

#endif /* CRAW_INTERNAL_H */
