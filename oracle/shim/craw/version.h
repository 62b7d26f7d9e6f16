/* Version header the reference's build would generate from version.h.in
 * (reference meson.build: version 0.0.1). Used only to compile the
 * reference's CPU code for the oracle. */
#ifndef CRAW_VERSION_H
#define CRAW_VERSION_H

#include <stdint.h>
#include <craw/utils.h>

#define CRAW_VERSION_MAJOR 0
#define CRAW_VERSION_MINOR 0
#define CRAW_VERSION_MICRO 1

CRAW_API uint32_t craw_version_int(void);

#endif /* CRAW_VERSION_H */
