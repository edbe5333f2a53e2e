// Minimal stand-in for <GLFW/glfw3.h> so the reference's SkyManager.cpp and ImageUtils.cpp
// compile without GLFW or Vulkan: their headers use only VkDescriptorSetLayoutBinding and a few
// enum values, for a descriptor-binding helper that the oracle never calls.
#pragma once
#include <cstdint>
typedef int VkDescriptorType;
typedef uint32_t VkShaderStageFlags;
typedef struct VkSampler_T* VkSampler;
typedef struct VkDescriptorSetLayoutBinding {
    uint32_t binding;
    VkDescriptorType descriptorType;
    uint32_t descriptorCount;
    VkShaderStageFlags stageFlags;
    const VkSampler* pImmutableSamplers;
} VkDescriptorSetLayoutBinding;
enum {
    VK_DESCRIPTOR_TYPE_UNIFORM_BUFFER = 6,
    VK_SHADER_STAGE_VERTEX_BIT = 0x1,
    VK_SHADER_STAGE_FRAGMENT_BIT = 0x10,
    VK_SHADER_STAGE_COMPUTE_BIT = 0x20
};
