// kernels.cuh -- host-callable launchers of the device passes (implemented in kernels.cu / wavefront.cu).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "shading.cuh"

namespace spk {

// Device image of spk_hit (20 B).
struct spk_hit_dev {
    float t, u, v;
    uint32_t prim, face;
};

struct FrameBuffers {
    float4 *gcolor;   // BasePass G-buffer colour (rgb, valid flag), W*H
    float4 *gnormal;  // first-hit world normal (xyz), W*H; written when spatial denoise is on
    float4 *fb;       // accumulated frame buffer, W*H
    ushort4 *out;     // tonemapped RGBA16F, row 0 = top
    uint32_t width, height;
};

struct Counters {
    unsigned long long extension_rays;
    unsigned long long shadow_rays;
    unsigned int error_flags;
    unsigned int pad;
    unsigned long long queue_counters[8];
};

struct RenderParams {
    uint32_t frame_seed;
    uint32_t bounce;
    uint32_t rng;
    uint32_t seed;
    uint32_t spatial_denoise;
    uint32_t enable_nee;
};

// Ray-set query over spk_ray records (24 B) into spk_hit records (20 B).
cudaError_t launch_trace(const DevScene &scene, const float *rays, uint64_t n, void *hits, int mode,
                         Counters *counters, int num_sms, cudaStream_t stream);

// One BasePass frame with one thread per pixel (the whole path in one kernel).
cudaError_t launch_render_mega(const DevScene &scene, const DevCamera &cam, const FrameBuffers &fbuf,
                               const RenderParams &p, Counters *counters, cudaStream_t stream);

// DenoisePass (spatial fill + temporal lerp with weight `moving_average`) + ToneMappingPass.
cudaError_t launch_resolve(const FrameBuffers &fbuf, float moving_average, float exposure, uint32_t spatial_denoise,
                           cudaStream_t stream);

}  // namespace spk
