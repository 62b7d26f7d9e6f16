/*
 * Noise-model table evaluation (reference lib/noise.c:37-110): a power law
 * between knots, a in proportion to iso outside the table, b with iso^2
 * above it and constant below it.
 */
#include <math.h>

#include <craw/noise.h>

CRAW_API int craw_noise_model_eval(const CRAWNoiseKnot *k, uint32_t n, float iso,
                                   CRAWNoiseModel *out)
{
    uint32_t i;
    float t;

    if (!k || !n || !out)
        return CRAW_ERROR(EINVAL);
    if (!(iso > 0.0f) || !isfinite(iso)) {
        *out = (CRAWNoiseModel) { .a = k[0].a, .b = k[0].b };
        return 0;
    }
    if (iso <= k[0].iso) {
        *out = (CRAWNoiseModel) { .a = k[0].a * (iso / k[0].iso), .b = k[0].b };
        return 0;
    }
    if (iso >= k[n - 1].iso) {
        float g = iso / k[n - 1].iso;
        *out = (CRAWNoiseModel) { .a = k[n - 1].a * g, .b = k[n - 1].b * g * g };
        return 0;
    }
    for (i = 0; i + 1 < n && iso > k[i + 1].iso; i++)
        ;
    if (!(k[i + 1].iso > k[i].iso)) {
        *out = (CRAWNoiseModel) { .a = k[i].a, .b = k[i].b };
        return 0;
    }
    t = (logf(iso) - logf(k[i].iso)) / (logf(k[i + 1].iso) - logf(k[i].iso));
    /* Log-log where both terms are positive, linear where one is zero. */
    if (k[i].a > 0.0f && k[i + 1].a > 0.0f)
        out->a = expf(logf(k[i].a) + t * (logf(k[i + 1].a) - logf(k[i].a)));
    else
        out->a = k[i].a + t * (k[i + 1].a - k[i].a);
    if (k[i].b > 0.0f && k[i + 1].b > 0.0f)
        out->b = expf(logf(k[i].b) + t * (logf(k[i + 1].b) - logf(k[i].b)));
    else
        out->b = k[i].b + t * (k[i + 1].b - k[i].b);
    return 0;
}
