// wavefront.cuh -- path state and launchers of the wavefront schedule of BasePass.
//
// The per-pixel path loop of SamplePixel (CPURenderer.cpp:240-396) is split into stage kernels that run
// over queues of live paths: generate (camera rays + RNG), then per bounce extend (closest hit) and shade
// (emission / sky / BSDF sample / Russian roulette, compacting survivors into the next queue with
// warp-aggregated atomics), then finish (G-buffer write). Queue lengths live in device memory, so one
// frame is a fixed launch sequence with no host round trip. Each path runs the same arithmetic and draws
// the same random numbers in the same order as the one-kernel schedule, so both write identical G-buffers.
#pragma once

#include "kernels.cuh"

namespace spk {

struct WavefrontState {
    uint32_t capacity = 0;
    float4 *ray_o = nullptr;    // origin xyz, w = pixel index bits
    float4 *ray_d = nullptr;    // direction xyz
    float4 *thr = nullptr;      // throughput xyz
    float4 *color = nullptr;    // radiance xyz, w = valid flag
    uint4 *rng = nullptr;       // 2 x uint4 per path (xoshiro256** needs 32 B)
    float4 *hit = nullptr;      // t, u, v, inst bits
    uint32_t *hit_face = nullptr;
    uint32_t *queue[2] = {nullptr, nullptr};  // path indices
    uint32_t *sort_keys = nullptr;            // material-sort scratch
};

cudaError_t wavefront_alloc(WavefrontState &s, uint32_t capacity);
void wavefront_free(WavefrontState &s);

cudaError_t launch_render_wavefront(const DevScene &scene, const DevCamera &cam, const FrameBuffers &fbuf,
                                    const RenderParams &p, bool count, Counters *counters, WavefrontState &s,
                                    int num_sms, cudaStream_t stream, uint32_t *launches, LaunchEvents *ev);

}  // namespace spk
