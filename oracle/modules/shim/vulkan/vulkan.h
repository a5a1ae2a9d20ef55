/* Type-only stand-in for <vulkan/vulkan.h>, so that the reference's module
 * host code (create_nodes, commit_params, modify_roi_*) and the scheduler
 * headers it includes compile for the CPU tests of the node plan. It declares
 * the handle, enum and struct names those headers mention and nothing else:
 * no function of the API exists, and the module code compiled against it
 * calls none. */
#pragma once
#include <stdint.h>
#include <stddef.h>

#define VK_MAX_PHYSICAL_DEVICE_NAME_SIZE 256u
#define VK_MAX_MEMORY_TYPES 32u
#define VK_MAX_MEMORY_HEAPS 16u
#define VK_MAX_EXTENSION_NAME_SIZE 256u
#define VK_MAX_DESCRIPTION_SIZE 256u

typedef uint64_t VkDeviceSize;
typedef uint32_t VkFlags;
typedef VkFlags VkMemoryPropertyFlags;
typedef VkFlags VkSubgroupFeatureFlags;
typedef int32_t VkResult;
typedef int32_t VkFormat;
typedef int32_t VkImageLayout;
typedef int32_t VkColorSpaceKHR;

#define VK_SHIM_HANDLE(n) typedef struct n##_shim *n
VK_SHIM_HANDLE(VkInstance);
VK_SHIM_HANDLE(VkPhysicalDevice);
VK_SHIM_HANDLE(VkDevice);
VK_SHIM_HANDLE(VkQueue);
VK_SHIM_HANDLE(VkCommandBuffer);
VK_SHIM_HANDLE(VkCommandPool);
VK_SHIM_HANDLE(VkBuffer);
VK_SHIM_HANDLE(VkImage);
VK_SHIM_HANDLE(VkImageView);
VK_SHIM_HANDLE(VkSampler);
VK_SHIM_HANDLE(VkSamplerYcbcrConversion);
VK_SHIM_HANDLE(VkDeviceMemory);
VK_SHIM_HANDLE(VkDescriptorSetLayout);
VK_SHIM_HANDLE(VkDescriptorSet);
VK_SHIM_HANDLE(VkDescriptorPool);
VK_SHIM_HANDLE(VkPipelineLayout);
VK_SHIM_HANDLE(VkPipeline);
VK_SHIM_HANDLE(VkShaderModule);
VK_SHIM_HANDLE(VkSemaphore);
VK_SHIM_HANDLE(VkQueryPool);
VK_SHIM_HANDLE(VkAccelerationStructureKHR);
VK_SHIM_HANDLE(VkDebugUtilsMessengerEXT);
VK_SHIM_HANDLE(VkSurfaceKHR);
VK_SHIM_HANDLE(VkSwapchainKHR);
VK_SHIM_HANDLE(VkFence);
VK_SHIM_HANDLE(VkFramebuffer);
VK_SHIM_HANDLE(VkRenderPass);
#undef VK_SHIM_HANDLE

typedef struct VkMemoryType { VkMemoryPropertyFlags propertyFlags; uint32_t heapIndex; } VkMemoryType;
typedef struct VkMemoryHeap { VkDeviceSize size; VkFlags flags; } VkMemoryHeap;
typedef struct VkPhysicalDeviceMemoryProperties
{
  uint32_t memoryTypeCount;
  VkMemoryType memoryTypes[VK_MAX_MEMORY_TYPES];
  uint32_t memoryHeapCount;
  VkMemoryHeap memoryHeaps[VK_MAX_MEMORY_HEAPS];
} VkPhysicalDeviceMemoryProperties;
typedef struct VkLayerProperties { char layerName[VK_MAX_EXTENSION_NAME_SIZE]; uint32_t specVersion, implementationVersion; char description[VK_MAX_DESCRIPTION_SIZE]; } VkLayerProperties;
typedef struct VkExtensionProperties { char extensionName[VK_MAX_EXTENSION_NAME_SIZE]; uint32_t specVersion; } VkExtensionProperties;
typedef struct VkAccelerationStructureGeometryKHR { int32_t shim; } VkAccelerationStructureGeometryKHR;
typedef struct VkAccelerationStructureBuildGeometryInfoKHR { int32_t shim; } VkAccelerationStructureBuildGeometryInfoKHR;
typedef struct VkAccelerationStructureBuildRangeInfoKHR { int32_t shim; } VkAccelerationStructureBuildRangeInfoKHR;
typedef void (*PFN_vkCmdPushDescriptorSetKHR)(void);
