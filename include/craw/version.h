/* craw-gb300 version. The API follows libcraw 0.0.1 (reference
 * meson.build:11), with the Vulkan binding replaced by a CUDA one. */
#ifndef CRAW_VERSION_H
#define CRAW_VERSION_H

#include <stdint.h>
#include <craw/utils.h>

#define CRAW_VERSION_MAJOR 0
#define CRAW_VERSION_MINOR 0
#define CRAW_VERSION_MICRO 1

#define CRAW_GET_VER_MAJOR(v) (((v) >> 16) & 0xFF)
#define CRAW_GET_VER_MINOR(v) (((v) >>  8) & 0xFF)
#define CRAW_GET_VER_MICRO(v) (((v) >>  0) & 0xFF)

/* (major << 16) | (minor << 8) | micro */
CRAW_API uint32_t craw_version_int(void);

#endif /* CRAW_VERSION_H */
