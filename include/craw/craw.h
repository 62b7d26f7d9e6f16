/*
 * craw-gb300: Bayer RAW frame development on one NVIDIA GB300 (sm_103a).
 *
 * A drop-in for the frame-development path of libcraw (reference
 * include/craw/craw.h). The caller owns the CUDA device, its streams and
 * every image; the library owns only its intermediates, its temporal state
 * and its histogram slots. A recording enqueues kernels on the stream the
 * caller passes and returns: the library never synchronises a stream or
 * the device on the caller's behalf.
 *
 * Sequence of use, as with the reference:
 *   1. craw_context_create() on a CUDA device (<craw/cuda.h>);
 *   2. fill a CRAWProfile (<craw/profile.h>);
 *   3. craw_pipeline_create() for one frame size and stage set;
 *   4. per frame, craw_pipeline_record() onto the caller's cudaStream_t;
 *   5. optionally read the AWB histogram back and run the estimator and
 *      smoother of <craw/awb.h>.
 *
 * No internal locking: one context or pipeline must not be used from two
 * threads at once.
 */
#ifndef CRAW_H
#define CRAW_H

#include <stdint.h>
#include <stdarg.h>

#include <craw/utils.h>
#include <craw/version.h>

typedef struct CRAWContext CRAWContext;

/* Log levels, numerically identical to the reference's (craw.h:63-72). */
enum CRAWLogLevel {
    CRAW_LOG_QUIET    = -(1 << 0),
    CRAW_LOG_FATAL    =  (0 << 0),
    CRAW_LOG_ERROR    = +(1 << 0),
    CRAW_LOG_WARN     = +(1 << 1),
    CRAW_LOG_INFO     = +(1 << 2),
    CRAW_LOG_VERBOSE  = +(1 << 3),
    CRAW_LOG_DEBUG    = +(1 << 4),
    CRAW_LOG_TRACE    = +(1 << 5),
};

/* Context options; zero-initialise for the defaults. 1024 bytes, laid out
 * as the reference's (craw.h:76-90). */
typedef struct CRAWContextOptions {
    void *log_opaque;

    /* Receives every message at or above log_level. NULL sends WARN and
     * more severe messages to stderr. */
    void (*log_cb)(void *log_opaque, enum CRAWLogLevel level,
                   const char *format, va_list args);

    enum CRAWLogLevel log_level;

    /* Reserved, must be zero. */
    uint8_t padding[1024 - 1*4 - 2*8];
} CRAWContextOptions;

/* Frees a context. Its pipelines must have been freed first. Leaves the
 * caller's device and streams alone. Replaces reference craw.h:99. */
CRAW_API void craw_context_free(CRAWContext **ctx);

/* Logs through the context's callback; `ctx` may be NULL (stderr).
 * Replaces reference craw.h:102. */
CRAW_API void craw_log(void *ctx, enum CRAWLogLevel level, const char *fmt, ...)
    craw_printf_format(3, 4);

#endif /* CRAW_H */
