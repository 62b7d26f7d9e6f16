/*
 * craw-gb300: camera profile and colour parameters
 * (reference include/craw/profile.h). Struct layouts are the reference's,
 * field for field.
 */
#ifndef CRAW_PROFILE_H
#define CRAW_PROFILE_H

#include <stdint.h>
#include <stdbool.h>

#include <craw/utils.h>
#include <craw/noise.h>

/* CFA phase, named by the 2x2 quad read left to right, top to bottom from
 * even (x, y). The pipeline implements RGGB; the others are refused by
 * craw_pipeline_create() with CRAW_ERROR(ENOTSUP), as in the reference. */
enum CRAWCfa {
    CRAW_CFA_RGGB = 0,
    CRAW_CFA_BGGR,
    CRAW_CFA_GRBG,
    CRAW_CFA_GBRG,
};

/* Quad site index of every per-site array: (y & 1) * 2 + (x & 1). */
#define CRAW_SITE_TL 0
#define CRAW_SITE_TR 1
#define CRAW_SITE_BL 2
#define CRAW_SITE_BR 3

/* An illuminant on the profile's locus: a CCT in Kelvin and a tint, the
 * signed offset from the locus along (-1, -1)/sqrt(2) in the plane of
 * (ln R/G, ln B/G); a positive tint raises the R and B gains by
 * exp(tint / sqrt(2)). */
typedef struct CRAWIlluminant {
    float cct;
    float tint;
} CRAWIlluminant;

#define CRAW_PROFILE_MAX_KNOTS 16

/* White balance gains (R, G, B) for a neutral at `cct`. */
typedef struct CRAWWbKnot {
    float cct;
    float wb[3];
} CRAWWbKnot;

/* Balanced camera RGB to XYZ (D65), row major, at `cct`. */
typedef struct CRAWMatrixKnot {
    float cct;
    float m[3][3];
} CRAWMatrixKnot;

typedef struct CRAWProfile {
    enum CRAWCfa cfa;

    /* Per quad site, in units of the input samples (UNORM 0..1); white is
     * the clip point. */
    float black_level[4];
    float white_level[4];

    float as_shot_wb[3];          /* gains R G B the camera applied */
    float as_shot_matrix[3][3];   /* balanced camera RGB -> XYZ D65 */
    float as_shot_cct;            /* Kelvin, 0 if unknown */

    /* Scene-linear scale after the matrix (diffuse white to 1.0). */
    float gain;

    /* When both are positive the output is also scaled by
     * exposure_index / as_shot_ei. */
    float as_shot_ei;
    float exposure_index;

    /* Re-balancing tables, ascending in cct; either may be empty. */
    CRAWWbKnot     wb_knots[CRAW_PROFILE_MAX_KNOTS];
    uint32_t       nb_wb_knots;
    CRAWMatrixKnot matrix_knots[CRAW_PROFILE_MAX_KNOTS];
    uint32_t       nb_matrix_knots;

    char name[64];

    /* Noise model per exposure index, ascending in iso; empty means the
     * caller supplies CRAWFrameParams.noise_override. */
    CRAWNoiseKnot noise_knots[CRAW_PROFILE_MAX_NOISE_KNOTS];
    uint32_t      nb_noise_knots;
} CRAWProfile;

enum CRAWWbMode {
    CRAW_WB_AS_SHOT = 0,   /* as_shot_wb and as_shot_matrix verbatim */
    CRAW_WB_REBALANCE,     /* the tables at CRAWFrameParams.illuminant */
};

/* Colour parameters of one frame, evaluated from a profile. */
typedef struct CRAWColorParams {
    float wb[3];
    float cam_to_xyz[3][3];
    float gain;
} CRAWColorParams;

/* Identity profile: RGGB, black 0, white 1, unit gains, identity matrix,
 * gain 1, no tables. Reference profile.h:152. */
CRAW_API void craw_profile_init(CRAWProfile *p);

/* Levels, table ordering and matrix sanity; 0 or CRAW_ERROR(EINVAL).
 * Reference profile.h:156 (lib/profile.c:50-147). */
CRAW_API int craw_profile_validate(const CRAWProfile *p);

/* Evaluates the frame's colour parameters. AS_SHOT ignores `illum`;
 * REBALANCE interpolates both tables linearly in Kelvin at the clamped
 * cct and raises R and B by exp(tint / sqrt(2)); no white balance table
 * is CRAW_ERROR(ENOTSUP), no matrix table falls back to as_shot_matrix.
 * out->gain includes the exposure-index ratio. Reference profile.h:170-172
 * (lib/profile.c:198-253). */
CRAW_API int craw_profile_eval(const CRAWProfile *p, enum CRAWWbMode mode,
                               const CRAWIlluminant *illum,
                               CRAWColorParams *out);

/* The illuminant under which a neutral surface gives the raw ratios
 * (raw_rg, raw_bg) = (R/G, B/G) before white balance: out->cct is the
 * point of the white balance locus that the neutral lies from along the
 * green direction (ln R/G and ln B/G moving together, the direction of a
 * tint), out->tint the signed distance along it, so that
 * craw_profile_illuminant_to_neutral() returns the ratios wherever the
 * table reaches. A neutral beyond either end of the locus goes to that
 * end. Needs a white balance table of two knots or more
 * (CRAW_ERROR(ENOTSUP)); ratios that are not finite and positive are
 * CRAW_ERROR(EINVAL). Reference profile.h:169-181 (lib/profile.c:254-389). */
CRAW_API int craw_profile_neutral_to_illuminant(const CRAWProfile *p,
                                                float raw_rg, float raw_bg,
                                                CRAWIlluminant *out);

/* The raw ratios of a neutral surface under `illum` (its cct clamped to
 * the table): the inverse of the gains craw_profile_eval() applies with
 * CRAW_WB_REBALANCE. Reference profile.h:183-187 (lib/profile.c:391-418). */
CRAW_API int craw_profile_illuminant_to_neutral(const CRAWProfile *p,
                                                const CRAWIlluminant *illum,
                                                float *raw_rg, float *raw_bg);

/* Output colour spaces, linear and scene referred. Values as the
 * reference's (profile.h:207-216). */
enum CRAWColorSpace {
    CRAW_CS_XYZ_D65 = 0,
    CRAW_CS_BT709_LINEAR,
    CRAW_CS_BT2020_LINEAR,
    CRAW_CS_P3D65_LINEAR,
    CRAW_CS_V_GAMUT_LINEAR,
    CRAW_CS_ACES_AP0_LINEAR,
    CRAW_CS_ACES_AP1_LINEAR,
    CRAW_CS_NB,
};

/* The noise table at `iso` (as_shot_ei when iso <= 0);
 * CRAW_ERROR(ENOTSUP) without a table. Reference profile.h:224
 * (lib/noise.c:112-123). */
CRAW_API int craw_profile_noise_eval(const CRAWProfile *p, float iso,
                                     CRAWNoiseModel *out);

/* Row-major XYZ (D65) -> `cs`, and back. The ACES spaces include a
 * Bradford adaptation between D65 and the ACES white. Reference
 * profile.h:229, 237 (lib/colorspace.c:234-270). */
CRAW_API int craw_colorspace_from_xyz_d65(enum CRAWColorSpace cs, float m[3][3]);
CRAW_API int craw_colorspace_to_xyz_d65(enum CRAWColorSpace cs, float m[3][3]);

/* CIE 1931 xy of a Planckian radiator (Krystek's approximation),
 * 1000..15000 K. Reference profile.h:243 (lib/colorspace.c:272-294). */
CRAW_API int craw_planckian_xy(float cct, float xy[2]);

/* Bradford von Kries adaptation from white `src` to white `dst` (xy).
 * Reference profile.h:250-251 (lib/colorspace.c:296-319). */
CRAW_API int craw_bradford_adaptation(const float src[2], const float dst[2],
                                      float m[3][3]);

#endif /* CRAW_PROFILE_H */
