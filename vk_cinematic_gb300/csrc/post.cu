// Display conversion of a path-traced frame, headless: the reference's
// post-processing shader (src/shaders/post_processing.frag.glsl:19-26:
// exposure 1, Reinhard c / (1 + c), gamma 1/2.2) followed by ToColor
// (src/math_lib.h:523-532: floor(c * 255) per channel, packed A8B8G8R8).
// The reference runs the shader on a Vulkan swapchain; here the 8-bit image
// is written to device memory.

#include "gbsp_internal.h"

namespace gbsp {

__device__ __forceinline__ uint32_t to_u8(float c)
{
    float f = floorf(c * 255.0f);
    f = fminf(fmaxf(f, 0.0f), 255.0f);  // the reference's (u8) cast of in-range values
    return (uint32_t)f;
}

__global__ void k_tonemap(const float4 *__restrict__ frame, uint64_t n, uint32_t *__restrict__ out)
{
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 c = frame[i];
    float r = c.x * 1.0f, g = c.y * 1.0f, b = c.z * 1.0f;
    r = r / (1.0f + r);
    g = g / (1.0f + g);
    b = b / (1.0f + b);
    const float e = 1.0f / 2.2f;
    r = powf(r, e);
    g = powf(g, e);
    b = powf(b, e);
    out[i] = (255u << 24) | (to_u8(b) << 16) | (to_u8(g) << 8) | to_u8(r);
}

}  // namespace gbsp

extern "C" int gbsp_tonemap(void *stream, const float *frame, uint64_t pixels, uint32_t *out)
{
    if (!frame || !out) return gbsp::set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!pixels) return GBSP_OK;
    gbsp::k_tonemap<<<(unsigned)((pixels + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const float4 *>(frame), pixels, out);
    GBSP_CUDA_TRY(cudaGetLastError());
    return GBSP_OK;
}
