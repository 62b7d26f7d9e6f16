/*
 * craw-gb300: the CUDA binding, which takes the place of the reference's
 * <craw/vulkan.h> (include/craw/vulkan.h).
 *
 * Where the reference is handed a VkInstance/VkDevice and records into a
 * VkCommandBuffer, this library is handed a CUDA device ordinal and
 * enqueues onto a cudaStream_t. Images are plain device allocations:
 * a pointer, a row pitch in bytes, a format and a size.
 */
#ifndef CRAW_CUDA_H
#define CRAW_CUDA_H

#include <cuda_runtime_api.h>

#include <craw/craw.h>

/* Image formats. The values are the VkFormat numbers of the reference's
 * three formats, so code ported from the Vulkan binding keeps its
 * constants (VK_FORMAT_R16_UNORM, VK_FORMAT_R16G16B16A16_SFLOAT,
 * VK_FORMAT_R32G32B32A32_SFLOAT). */
typedef enum CRAWFormat {
    CRAW_FORMAT_R16_UNORM = 70,   /* Bayer mosaic, one uint16 per sample */
    CRAW_FORMAT_R16F      = 76,   /* one half float per sample (VK_FORMAT_R16_SFLOAT): the
                                   * rebuilt highlight mosaic, read back for tests only */
    CRAW_FORMAT_RGBA16F   = 97,   /* four IEEE half floats per pixel */
    CRAW_FORMAT_RGB32F    = 106,  /* three IEEE floats per pixel, no alpha
                                   * (VK_FORMAT_R32G32B32_SFLOAT); an extension for
                                   * outputs that leave the device: a quarter fewer bytes
                                   * than RGBA32F, rows 16-byte aligned as every image's */
    CRAW_FORMAT_RGBA32F   = 109,  /* four IEEE floats per pixel */
} CRAWFormat;

/* Reports whether CUDA device `device` can run this library: an sm_103
 * part (the kernels are built for sm_103a only) with enough shared memory
 * per block. 0 when it can, CRAW_ERROR(ENOTSUP) otherwise with `*missing`
 * (may be NULL) naming what is missing. Replaces
 * craw_vulkan_check_device() (reference vulkan.h:99-101). */
CRAW_API int craw_cuda_check_device(int device, const char **missing);

/* What the library needs to know about the caller's device. Replaces
 * CRAWVulkanInitParams (reference vulkan.h:108-126). */
typedef struct CRAWCudaInitParams {
    /* CUDA device ordinal. The library makes it current in the calling
     * thread whenever it allocates, and expects it to be current when
     * craw_pipeline_record() is called. */
    int device;

    /* Memory pool the intermediates are allocated from with
     * cudaMallocFromPoolAsync. NULL uses a pool the context creates (and
     * frees) for itself. */
    cudaMemPool_t mem_pool;

    /* Reserved, must be zero. */
    uint8_t padding[64 - 16];
} CRAWCudaInitParams;

/* Creates a context on the device. Fails with CRAW_ERROR(ENOTSUP) on a
 * device craw_cuda_check_device() refuses. Replaces craw_context_create()
 * (reference vulkan.h:130-132). */
CRAW_API int craw_context_create(CRAWContext **ctx,
                                 const CRAWCudaInitParams *params,
                                 const CRAWContextOptions *opts);

/* A 2D image the library reads or writes: device memory the caller owns.
 * Rows are `pitch` bytes apart; pitch must be at least width times the
 * pixel size and a multiple of 16, and `data` 16-byte aligned, so that
 * every row can be moved with 128-bit accesses. The caller orders prior
 * writes to the image before the recording on the stream it passes (or
 * with events). Replaces CRAWImage (reference vulkan.h:147-153). */
typedef struct CRAWImage {
    void      *data;
    size_t     pitch;
    CRAWFormat format;
    uint32_t   width, height;
} CRAWImage;

struct CRAWProfile;
struct CRAWNoiseEstimateParams;
struct CRAWNoiseEstimate;

/* craw_noise_estimate() (craw/noise.h) of a mosaic already on the device:
 * an R16_UNORM image, 16-byte aligned rows. The work is enqueued on
 * `stream` (after whatever the caller put there before), which this call
 * then synchronises: it returns the estimate. Device scratch (about
 * 6 bytes per sample) is allocated on the stream from the device's
 * current memory pool and freed before returning. No reference
 * counterpart (the reference estimates on the CPU). */
CRAW_API int craw_noise_estimate_cuda(const CRAWImage *mosaic, const struct CRAWProfile *profile,
                                      const struct CRAWNoiseEstimateParams *params,
                                      struct CRAWNoiseEstimate *out, cudaStream_t stream);

#endif /* CRAW_CUDA_H */
