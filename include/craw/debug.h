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

#endif /* CRAW_DEBUG_H */
