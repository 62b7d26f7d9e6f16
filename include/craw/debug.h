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

struct CRAWPipeline;

/* Waits for the pipeline's recordings to finish and returns the error
 * bits its kernels set (1: a TMA copy was not complete within its wait
 * bound; the tile was skipped), clearing them. 0 when all is well; a
 * negative errno if the read fails. */
CRAW_API int craw_debug_kernel_errors(struct CRAWPipeline *pipe);

#endif /* CRAW_DEBUG_H */
