/*
 * craw-gb300: shared macros of the public C ABI.
 *
 * Same contract as the reference's <craw/utils.h> (include/craw/utils.h):
 * every call returns 0 or a positive count on success and a negated errno
 * value on failure, and exported symbols carry CRAW_API.
 */
#ifndef CRAW_UTILS_H
#define CRAW_UTILS_H

#include <stddef.h>
#include <stdint.h>
#include <stdbool.h>
#include <errno.h>

/* Turns an errno value into the negative return code the API uses. */
#define CRAW_ERROR(err) (-(err))

#define CRAW_MIN(a, b) ((a) < (b) ? (a) : (b))
#define CRAW_MAX(a, b) ((a) > (b) ? (a) : (b))
#define CRAW_CLAMP(v, lo, hi) CRAW_MIN(CRAW_MAX((v), (lo)), (hi))
#define CRAW_ARRAY_ELEMS(a) (sizeof(a) / sizeof((a)[0]))

#ifndef CRAW_API
#  if defined(__GNUC__) && __GNUC__ >= 4
#    define CRAW_API __attribute__((visibility("default")))
#  else
#    define CRAW_API
#  endif
#endif

#if defined(__GNUC__) || defined(__clang__)
#define craw_printf_format(fmt, args) __attribute__((__format__(__printf__, fmt, args)))
#else
#define craw_printf_format(fmt, args)
#endif

#endif /* CRAW_UTILS_H */
