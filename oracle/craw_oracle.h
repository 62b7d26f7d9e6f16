/*
 * CPU oracle for the frame-development path (test infrastructure only).
 * See craw_oracle.c. Every array is row major; RGBA buffers hold four
 * values per pixel; temporal states hold 2 * width * height values (the
 * level of every mosaic sample, then the variance left in it).
 */
#ifndef CRAW_ORACLE_H
#define CRAW_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#include <craw/pipeline.h>

struct orc_gamut {
    float thr[3];
    float scl[3];
    float pwr;
    float inv_pwr;
};

int orc_profile_eval(const CRAWProfile *p, int mode, const CRAWIlluminant *illum,
                     CRAWColorParams *out);
int orc_colorspace_from_xyz_d(int cs, double o[3][3]);
int orc_colorspace_from_xyz_f(int cs, float o[3][3]);
void orc_gamut_params(struct orc_gamut *g);
int orc_noise_model_eval(const CRAWNoiseKnot *k, uint32_t n, float iso, CRAWNoiseModel *out);
int orc_noise_model(const CRAWFrameParams *fp, CRAWNoiseModel *out);
int orc_noise_estimate(const uint16_t *bayer, uint32_t width, uint32_t height, size_t stride,
                       const CRAWProfile *profile, const CRAWNoiseEstimateParams *params,
                       CRAWNoiseEstimate *out);
int orc_awb_histogram(const float *rgb, uint32_t width, uint32_t height, size_t stride,
                      int channels, const float wb[3], uint32_t *count,
                      uint32_t *weight, uint32_t *weight_bright);

#define ORC_DECLARE(R, S)                                                              \
    int orc_debayer_mosaic_##S(const R *v, uint32_t w, uint32_t h, int method, R *rgb); \
    int orc_debayer_wb_##S(const uint16_t *bayer, uint32_t w, uint32_t h, size_t stride, \
                           const CRAWProfile *profile, const float wb[3], int method,     \
                           R *rgb);                                                      \
    int orc_denoise_temporal_##S(const uint16_t *bayer, uint32_t w, uint32_t h,          \
                                 size_t stride, const CRAWProfile *profile,               \
                                 const CRAWNoiseModel *model, float strength,             \
                                 float alpha_max, const R *prev, R *next,                 \
                                 uint16_t *out, size_t out_stride);                       \
    int orc_chroma_denoise_##S(R *rgb, uint32_t w, uint32_t h, float strength);           \
    int orc_highlights_##S(const uint16_t *bayer, uint32_t w, uint32_t h, size_t stride,   \
                           const CRAWProfile *profile, const float wb[3], R *out);        \
    int orc_color_##S(R *rgb, uint32_t w, uint32_t h, const CRAWFrameParams *fp,          \
                      int out_space);                                                     \
    int orc_process_##S(const uint16_t *bayer, uint32_t w, uint32_t h, size_t stride,     \
                        const CRAWPipelineParams *params, const CRAWFrameParams *fp,      \
                        R *out);

ORC_DECLARE(float, f32)
ORC_DECLARE(double, f64)

#endif /* CRAW_ORACLE_H */
