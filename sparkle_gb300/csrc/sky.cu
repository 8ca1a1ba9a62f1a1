// sky.cu -- the sky cube map cooked from an equirectangular sky map (spk_sky_from_equirect).
//
// Restates SkyLightCookJob::Execute (scene/component/light/SkyLight.cpp:83-113), which the reference runs
// when a sky map is set: for every face f and texel (i, j) of an N x N RGBAFloat16 cube, u = (i + 0.5) / N
// * 2 - 1, v = (j + 0.5) / N * 2 - 1, the direction Image2DCube::TextureCoordinateToDirection(f, u, v)
// (io/Image.h:287-314, normalised), its equirectangular coordinate utilities::CartesianToEquirectangular
// ((atan2(y, x), asin(-z)) * (1 / 2pi, 1 / pi) + 0.5, Utilities.h:510-518), the sky map's Image2D::Sample
// there (bilinear with wrap, sRGB decoded after the filter), stored as half RGB with alpha 1 (SetPixel).
// The path tracer then samples this cube on a miss (SkyRenderProxy::Evaluate). One thread per texel.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/spk.h"
#include "spk_math.cuh"

namespace spk {
namespace {

__device__ __forceinline__ unsigned wrap_index(int a, unsigned b) {
    return (static_cast<unsigned>(a % static_cast<int>(b)) + b) % b;  // utilities::WrapMod
}

__device__ __forceinline__ float srgb_to_linear(float c) {
    return c < 0.04045f ? c / 12.92f : powf((c + 0.055f) / 1.055f, 2.4f);
}

__device__ __forceinline__ float half_round(float x) { return __half2float(__float2half_rn(x)); }

__global__ void k_sky_from_equirect(const float4 *map, uint32_t w, uint32_t h, uint32_t srgb, uint32_t n,
                                    float4 *cube) {
    const uint64_t idx = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    if (idx >= 6ull * n * n) return;
    const uint32_t face = static_cast<uint32_t>(idx / (static_cast<uint64_t>(n) * n));
    const uint32_t rem = static_cast<uint32_t>(idx % (static_cast<uint64_t>(n) * n));
    const uint32_t j = rem / n, i = rem % n;
    const float fn = static_cast<float>(n);
    const float u = (static_cast<float>(i) + 0.5f) / fn * 2.f - 1.f;
    const float v = (static_cast<float>(j) + 0.5f) / fn * 2.f - 1.f;
    f3 d;
    switch (face) {
    case 0: d = mk3(1.f, -v, -u); break;
    case 1: d = mk3(-1.f, -v, u); break;
    case 2: d = mk3(u, 1.f, v); break;
    case 3: d = mk3(u, -1.f, -v); break;
    case 4: d = mk3(u, -v, 1.f); break;
    default: d = mk3(-u, -v, -1.f); break;
    }
    d = normalized(d);
    const float inv_pi = 0.318309886183790671538f;  // std::numbers::inv_pi_v<float>
    const float eu = atan2f(d.y, d.x) * (inv_pi * 0.5f) + 0.5f;
    const float ev = asinf(-d.z) * inv_pi + 0.5f;
    // Image2D::Sample at (eu, ev)
    const float px = eu * static_cast<float>(w), py = ev * static_cast<float>(h);
    const int ui = static_cast<int>(px), vi = static_cast<int>(py);
    const float uc = px - static_cast<float>(ui), vc = py - static_cast<float>(vi);
    const unsigned x0 = wrap_index(ui, w), x1 = wrap_index(ui + 1, w);
    const unsigned y0 = wrap_index(vi, h), y1 = wrap_index(vi + 1, h);
    const float4 s00 = __ldg(map + static_cast<size_t>(y0) * w + x0), s10 = __ldg(map + static_cast<size_t>(y0) * w + x1);
    const float4 s01 = __ldg(map + static_cast<size_t>(y1) * w + x0), s11 = __ldg(map + static_cast<size_t>(y1) * w + x1);
    const f3 l0 = mk3(s00.x + (s10.x - s00.x) * uc, s00.y + (s10.y - s00.y) * uc, s00.z + (s10.z - s00.z) * uc);
    const f3 l1 = mk3(s01.x + (s11.x - s01.x) * uc, s01.y + (s11.y - s01.y) * uc, s01.z + (s11.z - s01.z) * uc);
    f3 r = mk3(l0.x + (l1.x - l0.x) * vc, l0.y + (l1.y - l0.y) * vc, l0.z + (l1.z - l0.z) * vc);
    if (srgb) r = mk3(srgb_to_linear(r.x), srgb_to_linear(r.y), srgb_to_linear(r.z));
    cube[idx] = make_float4(half_round(r.x), half_round(r.y), half_round(r.z), 1.f);
}

}  // namespace
}  // namespace spk

extern "C" spk_status spk_sky_from_equirect(int32_t device, const float *rgba, uint32_t width, uint32_t height,
                                            uint32_t srgb, uint32_t cube_size, float *cube_rgba) {
    if (!rgba || !cube_rgba || width == 0 || height == 0 || cube_size == 0 || cube_size > 8192 ||
        static_cast<uint64_t>(width) * height > (1ull << 30))
        return SPK_ERR_INVALID_ARGUMENT;
    if (cudaSetDevice(device) != cudaSuccess) return SPK_ERR_CUDA;
    const uint64_t in_n = static_cast<uint64_t>(width) * height, out_n = 6ull * cube_size * cube_size;
    float4 *d_in = nullptr, *d_out = nullptr;
    cudaError_t e = cudaMalloc(&d_in, in_n * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&d_out, out_n * sizeof(float4));
    if (e == cudaSuccess) e = cudaMemcpy(d_in, rgba, in_n * sizeof(float4), cudaMemcpyDefault);
    if (e == cudaSuccess) {
        spk::k_sky_from_equirect<<<static_cast<unsigned>((out_n + 255) / 256), 256>>>(
            reinterpret_cast<const float4 *>(d_in), width, height, srgb ? 1u : 0u, cube_size, d_out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(cube_rgba, d_out, out_n * sizeof(float4), cudaMemcpyDefault);
    cudaFree(d_in);
    cudaFree(d_out);
    return e == cudaSuccess ? SPK_OK : (e == cudaErrorMemoryAllocation ? SPK_ERR_OUT_OF_MEMORY : SPK_ERR_CUDA);
}
