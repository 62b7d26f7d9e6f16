/*
 * craw-gb300: test hooks (extension, no counterpart in the reference).
 */
#ifndef CRAW_DEBUG_H
#define CRAW_DEBUG_H

#include <craw/utils.h>

/* Makes the k-th device allocation from now (1-based) fail with
 * CRAW_ERROR(ENOMEM), so that tests can check that a failed
 * craw_pipeline_create() leaves nothing behind; 0 disarms it. */
CRAW_API void craw_debug_fail_alloc(int k);

/* Makes every pipeline created from now use denoise tile shape `shape`
 * (the index craw_pipeline_get_kernel_config() reports) instead of the
 * autotuner's pick, so that tests can check each shape; -1 restores the
 * autotuner. Returns CRAW_ERROR(EINVAL) for an unknown shape. */
CRAW_API int craw_debug_force_denoise_shape(int shape);

/* on = 1 (the default): the RCD's interior tiles bring their mosaic into
 * shared memory with one TMA tile copy each; 0: with plain loads, for
 * comparing the two. Returns the previous setting. */
CRAW_API int craw_debug_rcd_tma(int on);

/* How the RCD's interior runs: 0 by 64x16 tiles; 1 (the default) by
 * strips (a thread a quad column, walking down the frame) unless the
 * colour stage has the ACES gamut compression, where the tiles are the
 * faster; 2 by strips wherever they apply; for comparing the two (they
 * give the same bits). Another value only reads. Returns the previous
 * setting. */
CRAW_API int craw_debug_rcd_strips(int mode);

/* 1 (default): the denoise's interior tiles (packed kernels, spatial
 * filtering) bring their mosaic region into shared memory with one TMA
 * tile copy each; 0: with plain loads, for comparing the two. Returns the
 * previous setting. */
CRAW_API int craw_debug_denoise_tma(int on);

struct CRAWPipeline;

/* Waits for the pipeline's recordings to finish and returns the error
 * bits its kernels set (1: a TMA copy was not complete within its wait
 * bound, the tile was skipped; 2: in the bounds-checked build,
 * libcraw_bounds.so, an index lay outside its buffer, the access was
 * skipped), clearing them. 0 when all is well; a negative errno if the
 * read fails. */
CRAW_API int craw_debug_kernel_errors(struct CRAWPipeline *pipe);

/* The exact rounding of the denoised codes (the samples whose float code
 * lies near a rounding boundary re-evaluated, so that they round as a
 * double evaluation of the filter does): `scale` sets the width of the
 * band of samples re-evaluated, in units of the float evaluation's error
 * bound (the default 2; 0 turns the exact rounding off; 1e6 and more
 * re-evaluate every sample). A negative scale only reads. Returns the
 * previous scale. For tests and measurement. */
CRAW_API float craw_debug_denoise_round(float scale);

/* on = 1 (the default): the exact rounding settles what it can of the
 * marked samples with a float re-evaluation that bounds its own error, and
 * evaluates the rest in double-float arithmetic; 0: every marked sample in
 * double-float, for checking the first stage's decisions. A negative value
 * only reads. Returns the previous setting. */
CRAW_API int craw_debug_denoise_round_decide(int on);

/* Waits for the pipeline's recordings and reads the exact rounding's
 * statistics since the last call: counts[0] samples re-evaluated,
 * counts[1] codes changed, counts[2] samples the float re-evaluation could
 * not settle (evaluated in double-float); and, for up to max_records of
 * the changed codes, four floats each: the sample's filtered value t, its
 * code position x, the distance of the exact x from its rounding boundary
 * (the float evaluation was off by at least that much), its plane. Clears
 * them. Returns the records written, or a negative errno. */
CRAW_API int craw_debug_denoise_round_stats(struct CRAWPipeline *pipe, uint32_t counts[3], float *records,
                                            uint32_t max_records);

#endif /* CRAW_DEBUG_H */
