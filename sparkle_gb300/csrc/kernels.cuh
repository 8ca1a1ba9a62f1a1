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
    unsigned long long node_visits;
    unsigned long long tri_tests;
    unsigned long long queue_counters[12];
};

// Sum of a per-thread count over the active lanes of a warp, added once per warp.
__device__ __forceinline__ void warp_add_u64(unsigned long long *dst, uint32_t v) {
    const uint32_t mask = __activemask();
    const uint32_t total = __reduce_add_sync(mask, v);
    if ((threadIdx.x & 31u) == static_cast<uint32_t>(__ffs(mask) - 1) && total)
        atomicAdd(dst, static_cast<unsigned long long>(total));
}

// Events bracketing each traversal launch (for per-launch device time); null = not recorded.
struct LaunchEvents {
    cudaEvent_t *pairs = nullptr;  // 2 * capacity events
    int capacity = 0;
    int used = 0;
    float graph_ms = 0.f;   // traversal time measured inside replayed CUDA graphs
    int graph_launches = 0;  // traversal launches inside replayed CUDA graphs
    // cudaEventRecordExternal while a stream is captured: the record becomes a graph node that every replay
    // performs (a plain record under capture only orders work inside the graph).
    unsigned record_flags = cudaEventRecordDefault;
    void before(cudaStream_t s) {
        if (pairs && used < capacity) cudaEventRecordWithFlags(pairs[2 * used], s, record_flags);
    }
    void after(cudaStream_t s) {
        if (pairs && used < capacity) cudaEventRecordWithFlags(pairs[2 * used++ + 1], s, record_flags);
    }
};

// SpatialDenoisePixel (CPURenderer.cpp:452-504) for pixel (i, j) of one frame's G-buffer (`color`: rgb +
// valid flag, `normal`: first-hit normal, rows of w pixels) as a gather: a valid, non-sky neighbour S fills
// the pixel when it is the first of S's 8 directions that is in bounds, invalid and has normal similarity
// >= 0.99; among several such S the one last in row-major order wins (the single-threaded order of the
// passes). Returns the pixel's G-buffer colour after the fill (`in` itself when nothing fills it).
__device__ __forceinline__ float4 spatial_fill(const float4 *color, const float4 *normal, uint32_t i, uint32_t j,
                                               uint32_t w, uint32_t h, float4 in) {
    constexpr int kDirs[8][2] = {{1, 0}, {0, 1}, {-1, 0}, {0, -1}, {-1, -1}, {1, -1}, {-1, 1}, {1, 1}};
    if (in.w > 0.f) return in;
    const int W = static_cast<int>(w), H = static_cast<int>(h);
    const size_t k = static_cast<size_t>(j) * w + i;
    long best_writer = -1;
    float4 best = in;
    for (int dk = 0; dk < 8; ++dk) {
        const int si = static_cast<int>(i) - kDirs[dk][0], sj = static_cast<int>(j) - kDirs[dk][1];
        if (si < 0 || si >= W || sj < 0 || sj >= H) continue;
        const size_t sk = static_cast<size_t>(sj) * w + si;
        const float4 sc = color[sk];
        const float4 sn = normal[sk];
        const bool sky = fabsf(sn.x) <= 1e-5f && fabsf(sn.y) <= 1e-5f && fabsf(sn.z) <= 1e-5f;
        if (!(sc.w > 0.f) || sky) continue;
        const f3 wn = mk3(sn.x, sn.y, sn.z);
        long target = -1;
        for (int tk = 0; tk < 8; ++tk) {
            const int ni = si + kDirs[tk][0], nj = sj + kDirs[tk][1];
            if (ni < 0 || ni >= W || nj < 0 || nj >= H) continue;
            const size_t nk = static_cast<size_t>(nj) * w + ni;
            if (color[nk].w > 0.f) continue;
            const float4 nn = normal[nk];
            if (dot3(mk3(nn.x, nn.y, nn.z), wn) < 0.99f) continue;
            target = static_cast<long>(nk);
            break;
        }
        if (target == static_cast<long>(k) && static_cast<long>(sk) > best_writer) {
            best_writer = static_cast<long>(sk);
            best = make_float4(sc.x, sc.y, sc.z, 1.f);
        }
    }
    return best;
}

struct RenderParams {
    uint32_t frame_seed;
    uint32_t bounce;
    uint32_t rng;
    uint32_t seed;
    uint32_t spatial_denoise;
    uint32_t enable_nee;
};

// Ray-set query over spk_ray records (24 B) into spk_hit records (20 B).
cudaError_t launch_trace(const DevScene &scene, const float *rays, uint64_t n, void *hits, int mode, bool count,
                         Counters *counters, int num_sms, cudaStream_t stream, LaunchEvents *ev);

// One BasePass frame with one thread per pixel (the whole path in one kernel).
cudaError_t launch_render_mega(const DevScene &scene, const DevCamera &cam, const FrameBuffers &fbuf,
                               const RenderParams &p, bool count, Counters *counters, cudaStream_t stream,
                               LaunchEvents *ev);

// Primary-hit guides (normal + linear depth, albedo + hit flag) of a w x h image.
cudaError_t launch_guides(const DevScene &scene, const DevCamera &cam, uint32_t w, uint32_t h, float4 *nd, float4 *alb,
                          Counters *counters, cudaStream_t stream);

// DenoisePass (spatial fill + temporal lerp with weight `moving_average`) + ToneMappingPass.
cudaError_t launch_resolve(const FrameBuffers &fbuf, float moving_average, float exposure, uint32_t spatial_denoise,
                           cudaStream_t stream);

}  // namespace spk
