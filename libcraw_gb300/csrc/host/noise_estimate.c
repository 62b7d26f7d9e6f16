/*
 * Noise-model estimation (reference lib/noise.c:125-504). The frame is
 * binned on the GPU (kernels/noise.cu): per bin the count, the exact sum
 * of the 9x9 means and the median |high-pass|. The least-trimmed-squares
 * cost of every pair of bins is evaluated on the GPU too, one warp per
 * pair; the host picks the seed in the reference's order, re-measures the
 * chosen pair's cost with its own log, and runs the reweighted
 * Gauss-Newton refinement (40 steps of a few hundred logs at most).
 */
#include <errno.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include <craw/cuda.h>
#include <craw/noise.h>
#include <craw/profile.h>

#include "internal.h"

/* The reference's constants (lib/noise.c:14-27, 145): Phi^-1(0.75), the
 * Tukey cut, the floor on the residual scale, the plane-mean radius. */
#define NE_MAD 0.674489750196081746f
#define NE_TUKEY 4.685
#define NE_SCALE_FLOOR 0.02
#define NE_R 4

CRAW_API void craw_noise_estimate_params_init(CRAWNoiseEstimateParams *p)
{
    if (!p)
        return;
    memset(p, 0, sizeof(*p));
    p->nb_bins = 128;
    p->min_bin_samples = 20000;
    p->max_level = 0.98f;
}

/* The reference's argument checks (lib/noise.c:352-388), defaults applied. */
static int ne_args(uint32_t w, uint32_t h, const CRAWProfile *pr, const CRAWNoiseEstimateParams *params,
                   CRAWKNoise *k, uint32_t *min_n)
{
    if (!pr)
        return CRAW_ERROR(EINVAL);
    if (pr->cfa != CRAW_CFA_RGGB)
        return CRAW_ERROR(ENOTSUP);
    if ((w & 1) || (h & 1) || w < 32 || h < 32)
        return CRAW_ERROR(EINVAL);
    k->nb_bins = params && params->nb_bins ? (int32_t)params->nb_bins : 128;
    *min_n = params && params->min_bin_samples ? params->min_bin_samples : 20000;
    k->max_level = params && params->max_level > 0.0f ? params->max_level : 0.98f;
    if (params && (params->nb_bins && (params->nb_bins < 8 || params->nb_bins > CRAW_NOISE_MAX_BINS)))
        return CRAW_ERROR(EINVAL);
    for (int s = 0; s < 4; s++) {
        if (!(pr->white_level[s] > pr->black_level[s]))
            return CRAW_ERROR(EINVAL);
        k->black[s] = pr->black_level[s];
        k->white[s] = pr->white_level[s];
    }
    if ((int)w / 2 < 2 * NE_R + 1 || (int)h / 2 < 2 * NE_R + 1)
        return CRAW_ERROR(EINVAL);
    k->width = (int32_t)w;
    k->height = (int32_t)h;
    return 0;
}

static int ne_cmp_d(const void *a, const void *b)
{
    const double x = *(const double *)a, y = *(const double *)b;
    return (x > y) - (x < y);
}

/* The bins the fit uses: level, variance, sample count, ln variance. */
typedef struct NeBins {
    int nb;
    double m[CRAW_NOISE_MAX_BINS], v[CRAW_NOISE_MAX_BINS], c[CRAW_NOISE_MAX_BINS];
    double lv[CRAW_NOISE_MAX_BINS];
} NeBins;

/* Bins with at least min_n samples and a positive spread (reference
 * lib/noise.c:452-467); the level is the exact sum of the means, rounded
 * once, over the count. */
static void ne_collect(const CRAWKNoiseBin *kb, int nb_bins, uint32_t min_n, NeBins *B)
{
    B->nb = 0;
    for (int i = 0; i < nb_bins; i++) {
        double sigma;
        unsigned __int128 sum;
        if (kb[i].count < min_n)
            continue;
        {
            float med;
            memcpy(&med, &kb[i].median, sizeof(med));
            sigma = med / NE_MAD;
        }
        if (!(sigma > 0.0))
            continue;
        sum = ((unsigned __int128)kb[i].sum[2] << 64) + ((unsigned __int128)kb[i].sum[1] << 32) +
              (unsigned __int128)kb[i].sum[0];
        B->m[B->nb] = ldexp((double)sum, -64) / (double)kb[i].count;
        B->v[B->nb] = sigma * sigma;
        B->c[B->nb] = (double)kb[i].count;
        B->lv[B->nb] = log(B->v[B->nb]);
        B->nb++;
    }
}

/* The line through bins i and j, or false where the reference skips the
 * pair (lib/noise.c:199-207). */
static bool ne_pair(const NeBins *B, int i, int j, double *a, double *b)
{
    if (B->m[j] - B->m[i] < 1e-5)
        return false;
    *a = (B->v[j] - B->v[i]) / (B->m[j] - B->m[i]);
    *b = B->v[i] - *a * B->m[i];
    return *a > 0.0 && !(*b < 0.0);
}

/* The pair's trimmed cost with the host's log, as the reference adds it. */
static double ne_pair_cost(const NeBins *B, double a, double b, int keep, double *work)
{
    double c = 0.0;
    for (int k = 0; k < B->nb; k++) {
        const double d = B->lv[k] - log(a * B->m[k] + b);
        work[k] = d * d;
    }
    qsort(work, (size_t)B->nb, sizeof(*work), ne_cmp_d);
    for (int k = 0; k < keep; k++)
        c += work[k];
    return c;
}

/* Reweighted Gauss-Newton on ln(a m + b) in (ln a, ln b) with a Tukey
 * biweight times ln(1 + count), the residual scale re-measured every
 * eighth step (reference lib/noise.c:252-336). */
static void ne_refine(const NeBins *B, double scale, double *a_io, double *b_io, double *res, double *work)
{
    double la = log(*a_io), lb = log(*b_io > 1e-16 ? *b_io : 1e-16);
    if (scale < NE_SCALE_FLOOR)
        scale = NE_SCALE_FLOOR;
    for (int it = 0; it < 40; it++) {
        const double ea = exp(la), eb = exp(lb);
        double aa = 0.0, ab = 0.0, bb = 0.0, ra = 0.0, rb = 0.0, det, d0, d1, cut;
        for (int k = 0; k < B->nb; k++)
            res[k] = B->lv[k] - log(ea * B->m[k] + eb);
        if ((it & 7) == 0) {
            for (int k = 0; k < B->nb; k++)
                work[k] = fabs(res[k]);
            qsort(work, (size_t)B->nb, sizeof(*work), ne_cmp_d);
            scale = 1.4826 * work[B->nb / 2];
            if (scale < NE_SCALE_FLOOR)
                scale = NE_SCALE_FLOOR;
        }
        cut = NE_TUKEY * scale;
        for (int k = 0; k < B->nb; k++) {
            const double den = ea * B->m[k] + eb, ja = ea * B->m[k] / den, jb = eb / den;
            const double u = res[k] / cut;
            double w = fabs(u) < 1.0 ? (1.0 - u * u) * (1.0 - u * u) : 0.0;
            w *= log(1.0 + B->c[k]);
            aa += w * ja * ja;
            ab += w * ja * jb;
            bb += w * jb * jb;
            ra += w * ja * res[k];
            rb += w * jb * res[k];
        }
        det = (aa + 1e-9) * (bb + 1e-9) - ab * ab;
        if (!(fabs(det) > 1e-30))
            break;
        d0 = ((bb + 1e-9) * ra - ab * rb) / det;
        d1 = (-ab * ra + (aa + 1e-9) * rb) / det;
        d0 = d0 < -0.5 ? -0.5 : (d0 > 0.5 ? 0.5 : d0);
        d1 = d1 < -0.5 ? -0.5 : (d1 > 0.5 ? 0.5 : d1);
        la += d0;
        lb += d1;
        if (lb < -40.0)
            lb = -40.0;
        if (fabs(d0) < 1e-9 && fabs(d1) < 1e-9)
            break;
    }
    *a_io = exp(la);
    *b_io = lb <= -40.0 ? 0.0 : exp(lb);
}

static int ne_cuda_err(cudaError_t e)
{
    if (e == cudaSuccess)
        return 0;
    return e == cudaErrorMemoryAllocation ? CRAW_ERROR(ENOMEM) : CRAW_ERROR(EIO);
}

/* The estimate of a device mosaic whose arguments have been checked. */
static int ne_run(const CRAWKNoise *k, const void *src, size_t pitch, uint32_t min_n, const CRAWProfile *pr,
                  CRAWNoiseEstimate *out, cudaStream_t s)
{
    const int nbins = k->nb_bins;
    const size_t scratch = craw_k_noise_scratch(k->width, k->height, nbins);
    const size_t bins_at = (scratch + 255) / 256 * 256;
    const size_t fit_at = bins_at + (size_t)CRAW_K_NOISE_MAX_BINS * sizeof(CRAWKNoiseBin);
    const size_t cost_at = fit_at + (size_t)3 * CRAW_NOISE_MAX_BINS * sizeof(double);
    const size_t total = cost_at + (size_t)CRAW_NOISE_MAX_BINS * CRAW_NOISE_MAX_BINS * sizeof(double);
    CRAWKNoiseBin *kb = malloc((size_t)nbins * sizeof(*kb));
    NeBins *B = malloc(sizeof(*B));
    double *cost = NULL, *work = malloc(2 * CRAW_NOISE_MAX_BINS * sizeof(double));
    char *dev = NULL;
    int ret = 0, nb, keep, bi = -1, bj = -1;
    double a = 0.0, b = 0.0, best = INFINITY, scale, rms = 0.0, range0;
    uint32_t nin = 0;

    if (!kb || !B || !work) {
        ret = CRAW_ERROR(ENOMEM);
        goto done;
    }
    if ((ret = ne_cuda_err(cudaMallocAsync((void **)&dev, total, s))) < 0) {
        dev = NULL;
        goto done;
    }
    if (craw_k_noise_bins(k, src, pitch, dev, (CRAWKNoiseBin *)(dev + bins_at), s) < 0) {
        ret = CRAW_ERROR(EIO);
        goto done;
    }
    if ((ret = ne_cuda_err(cudaMemcpyAsync(kb, dev + bins_at, (size_t)nbins * sizeof(*kb),
                                           cudaMemcpyDeviceToHost, s))) < 0 ||
        (ret = ne_cuda_err(cudaStreamSynchronize(s))) < 0)
        goto done;

    ne_collect(kb, nbins, min_n, B);
    nb = B->nb;
    if (nb < 3) {
        ret = CRAW_ERROR(ENODATA);
        goto done;
    }
    keep = nb * 2 / 3 + 1;

    /* Every pair's cost on the device; the seed is the first pair, in
     * the reference's (i, j) order, whose cost is strictly the least. */
    if (!(cost = malloc((size_t)nb * nb * sizeof(*cost)))) {
        ret = CRAW_ERROR(ENOMEM);
        goto done;
    }
    {
        double *dm = (double *)(dev + fit_at), *dv = dm + CRAW_NOISE_MAX_BINS, *dl = dv + CRAW_NOISE_MAX_BINS;
        double *dc = (double *)(dev + cost_at);
        if ((ret = ne_cuda_err(cudaMemcpyAsync(dm, B->m, nb * sizeof(double), cudaMemcpyHostToDevice, s))) < 0 ||
            (ret = ne_cuda_err(cudaMemcpyAsync(dv, B->v, nb * sizeof(double), cudaMemcpyHostToDevice, s))) < 0 ||
            (ret = ne_cuda_err(cudaMemcpyAsync(dl, B->lv, nb * sizeof(double), cudaMemcpyHostToDevice, s))) < 0)
            goto done;
        if (craw_k_noise_lts(dm, dv, dl, nb, keep, dc, s) < 0) {
            ret = CRAW_ERROR(EIO);
            goto done;
        }
        if ((ret = ne_cuda_err(cudaMemcpyAsync(cost, dc, (size_t)nb * nb * sizeof(double),
                                               cudaMemcpyDeviceToHost, s))) < 0 ||
            (ret = ne_cuda_err(cudaStreamSynchronize(s))) < 0)
            goto done;
    }
    for (int i = 0; i < nb; i++)
        for (int j = i + 1; j < nb; j++)
            if (cost[(size_t)i * nb + j] < best) {
                best = cost[(size_t)i * nb + j];
                bi = i;
                bj = j;
            }
    if (bi < 0 || !ne_pair(B, bi, bj, &a, &b) || !(a > 0.0)) {
        ret = CRAW_ERROR(ENODATA);
        goto done;
    }
    best = ne_pair_cost(B, a, b, keep, work);
    scale = sqrt(best / keep);

    ne_refine(B, scale, &a, &b, work + CRAW_NOISE_MAX_BINS, work);

    for (int i = 0; i < nb; i++) {
        const double d = B->lv[i] - log(a * B->m[i] + b);
        if (fabs(d) < 0.35) {
            rms += d * d;
            nin++;
        }
    }
    rms = sqrt(rms / (nin ? nin : 1));
    range0 = pr->white_level[0] - pr->black_level[0];
    memset(out, 0, sizeof(*out));
    out->model.a = (float)a;
    out->model.b = (float)b;
    out->nb_bins = (uint32_t)nb;
    out->nb_inliers = nin;
    out->fit_rms = (float)rms;
    out->read_noise_lsb = (float)(sqrt(b) * range0 * 65535.0);

done:
    if (dev) {
        cudaFreeAsync(dev, s);
        if (cudaStreamSynchronize(s) != cudaSuccess && ret == 0)
            ret = CRAW_ERROR(EIO);
    }
    free(cost);
    free(work);
    free(B);
    free(kb);
    return ret;
}

CRAW_API int craw_noise_estimate_cuda(const CRAWImage *mosaic, const CRAWProfile *profile,
                                      const CRAWNoiseEstimateParams *params, CRAWNoiseEstimate *out,
                                      cudaStream_t stream)
{
    CRAWKNoise k;
    uint32_t min_n;
    int ret;

    if (!mosaic || !out)
        return CRAW_ERROR(EINVAL);
    if ((ret = ne_args(mosaic->width, mosaic->height, profile, params, &k, &min_n)) < 0)
        return ret;
    if (mosaic->format != CRAW_FORMAT_R16_UNORM || !mosaic->data || ((uintptr_t)mosaic->data & 15) ||
        (mosaic->pitch & 15) || mosaic->pitch < (size_t)mosaic->width * 2)
        return CRAW_ERROR(EINVAL);
    if (cudaPeekAtLastError() != cudaSuccess)
        return CRAW_ERROR(EIO);         /* the caller's pending error is not ours to clear */
    return ne_run(&k, mosaic->data, mosaic->pitch, min_n, profile, out, stream);
}

CRAW_API int craw_noise_estimate(const uint16_t *bayer, uint32_t width, uint32_t height, size_t stride,
                                 const CRAWProfile *profile, const CRAWNoiseEstimateParams *params,
                                 CRAWNoiseEstimate *out)
{
    CRAWKNoise k;
    uint32_t min_n;
    cudaStream_t s = NULL;
    void *frame = NULL;
    size_t pitch = ((size_t)width * 2 + 15) / 16 * 16;
    int ret;

    if (!bayer || !out)
        return CRAW_ERROR(EINVAL);
    if ((ret = ne_args(width, height, profile, params, &k, &min_n)) < 0)
        return ret;
    if (stride < width)
        return CRAW_ERROR(EINVAL);
    if (cudaPeekAtLastError() != cudaSuccess)
        return CRAW_ERROR(EIO);         /* the caller's pending error is not ours to clear */
    if ((ret = ne_cuda_err(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking))) < 0)
        return ret == CRAW_ERROR(ENOMEM) ? ret : CRAW_ERROR(EIO);
    if ((ret = ne_cuda_err(cudaMallocAsync(&frame, pitch * height, s))) < 0) {
        frame = NULL;
        goto done;
    }
    if ((ret = ne_cuda_err(cudaMemcpy2DAsync(frame, pitch, bayer, stride * 2, (size_t)width * 2, height,
                                             cudaMemcpyHostToDevice, s))) < 0)
        goto done;
    ret = ne_run(&k, frame, pitch, min_n, profile, out, s);
done:
    if (frame)
        cudaFreeAsync(frame, s);
    if (cudaStreamSynchronize(s) != cudaSuccess && ret == 0)
        ret = CRAW_ERROR(EIO);
    cudaStreamDestroy(s);
    return ret;
}
