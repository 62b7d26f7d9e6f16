/*
 * Stand-in for the reference's <craw/vulkan.h>, used only to compile the
 * reference's CPU code (lib/ref and the host colour/noise/AWB files) without
 * a Vulkan SDK. It defines the handful of Vulkan names that <craw/pipeline.h>
 * mentions; nothing here is ever called. Test infrastructure, not product.
 */
#ifndef CRAW_VULKAN_H
#define CRAW_VULKAN_H

#include <craw/craw.h>

typedef enum VkFormat {
    VK_FORMAT_R16_UNORM           = 70,
    VK_FORMAT_R16G16B16A16_SFLOAT = 97,
    VK_FORMAT_R32G32B32A32_SFLOAT = 109,
} VkFormat;

typedef struct VkCommandBuffer_T *VkCommandBuffer;
typedef struct CRAWImage CRAWImage;

#endif /* CRAW_VULKAN_H */
