// kernels.cu -- ray-set query, one-kernel path tracer (BasePass), resolve (DenoisePass + ToneMappingPass).
//
// Compiled with -fmad=false: every multiply and add rounds separately, as the reference's (contraction-free)
// host arithmetic does; the slab tests use explicit fmaf.
#include <cuda_fp16.h>

#include "kernels.cuh"

namespace spk {
namespace {

// ------------------------------------------------------------------------------------------------
// Ray-set query: persistent warps pull rays from a global counter and refill idle lanes.
// ------------------------------------------------------------------------------------------------
template <int kMode, bool kCount>
__global__ void __launch_bounds__(128, SPK_WALK_MIN_BLOCKS) k_trace(DevScene S, const float *__restrict__ rays, uint64_t n,
                                                  spk_hit_dev *__restrict__ hits, Counters *counters) {
    uint32_t err = 0, done = 0;
    TraceCounts tc;
    walk_persistent<kMode, kCount>(
        S, &counters->queue_counters[0], n, kFltMax, err, &tc,
        [&](unsigned long long q, f3 &o, f3 &d, float &) {
            const float *r = rays + q * 6;
            o = mk3(r[0], r[1], r[2]);
            d = mk3(r[3], r[4], r[5]);
            return S.tlas_root;
        },
        [&](unsigned long long q, const TraceResult &res) {
            spk_hit_dev out;
            if (res.inst == kInvalid) {
                out = spk_hit_dev{0.f, 0.f, 0.f, kInvalid, kInvalid};
            } else if (kMode == kTraceClosest) {
                out = spk_hit_dev{res.t, res.u, res.v, res.inst, res.face};
            } else {
                out = spk_hit_dev{0.f, 0.f, 0.f, res.inst, kInvalid};
            }
            hits[q] = out;
            ++done;
        });
    warp_add_u64(&counters->extension_rays, done);
    if (kCount) {
        warp_add_u64(&counters->node_visits, tc.nodes);
        warp_add_u64(&counters->tri_tests, tc.tris);
    }
    if (err) atomicOr(&counters->error_flags, err);
}

// ------------------------------------------------------------------------------------------------
// BasePass: one thread per pixel runs RenderPixel + SamplePixel (CPURenderer.cpp:240-417).
// ------------------------------------------------------------------------------------------------
template <int kKind, bool kCount, bool kNee>
__global__ void __launch_bounds__(128) k_render_mega(DevScene S, DevCamera cam, FrameBuffers fb, RenderParams p,
                                                     Counters *counters) {
    const uint32_t i = blockIdx.x * 16u + (threadIdx.x & 15u);
    const uint32_t j = blockIdx.y * 8u + (threadIdx.x >> 4);
    uint32_t err = 0, rays = 0, shadow = 0;
    TraceCounts tc;
    if (i < fb.width && j < fb.height) {
        Rng rng;
        rng_seed_pixel<kKind>(rng, p.seed, i, j, fb.width, fb.height, p.frame_seed);
        const float pw = 1.f / static_cast<float>(fb.width - 1);
        const float ph = 1.f / static_cast<float>(fb.height - 1);
        const float u = (static_cast<float>(i) + rng_unit<kKind>(rng)) * pw;
        const float v = (static_cast<float>(j) + rng_unit<kKind>(rng)) * ph;
        f3 o, d;
        camera_ray<kKind>(cam, rng, u, v, o, d);
        f3 color = mk3(0.f, 0.f, 0.f), thr = mk3(1.f, 1.f, 1.f), first_normal = mk3(0.f, 0.f, 0.f);
        float valid = 1.f;
        float prev_pdf = 0.f;  // NEE: cosine pdf of the continuation when the previous vertex sampled lights
        for (uint32_t bounce = 0; bounce < p.bounce; ++bounce) {
            ++rays;
            const TraceResult hit = trace_ray<kTraceClosest, kCount>(S, o, d, kFltMax, err, &tc);
            if (hit.inst == kInvalid) {
                if (S.sky_mode != 0u) {
                    f3 c = cmul(sky_eval(S, d), thr);
                    if (kNee && prev_pdf > 0.f) c = c * mis_weight(prev_pdf, prev_pdf);
                    color = color + c;
                }
                break;
            }
            const Surface surf = make_surface(S, hit, o, d);
            const DevMaterial mat = resolve_material(S, S.materials[surf.material], surf.uv);
            if (bounce == 0) first_normal = surf.normal;
            if (mat.is_emissive) {
                f3 c = cmul(mk3(mat.emissive[0], mat.emissive[1], mat.emissive[2]), thr);
                if (kNee && prev_pdf > 0.f) c = c * bsdf_hit_weight(S, prev_pdf, hit, d);
                color = color + c;
                break;
            }
            f3 next_dir;
            float dz = -1.f;
            const f3 this_thr =
                sample_surface<kKind>(rng, mat, d, surf.normal, surf.tangent, next_dir, kNee ? &dz : nullptr);
            prev_pdf = 0.f;
            if (kNee && dz >= 0.f) {
                nee_direct<kKind, kCount>(S, rng, surf, mk3(mat.base[0], mat.base[1], mat.base[2]), thr, color,
                                          shadow, err, &tc);
                prev_pdf = dz * kInvPi;
            }
            thr = cmul(thr, this_thr);
            if (sqnorm(thr) < kEps) {
                valid = -1.f;
                break;
            }
            if (bounce >= 3) {
                float q = max_std(thr.x, max_std(thr.y, thr.z));
                q = (q < 0.05f) ? 0.05f : (1.0f < q) ? 1.0f : q;
                if (rng_unit<kKind>(rng) > q) break;
                thr = mk3(thr.x / q, thr.y / q, thr.z / q);
            }
            o = surf.location + next_dir * kTolerance;
            d = next_dir;
        }
        const size_t k = static_cast<size_t>(j) * fb.width + i;
        fb.gcolor[k] = make_float4(clamp_sample(color.x), clamp_sample(color.y),
                                   clamp_sample(color.z), valid);
        if (p.spatial_denoise) fb.gnormal[k] = make_float4(first_normal.x, first_normal.y, first_normal.z, 0.f);
    }
    warp_add_u64(&counters->extension_rays, rays);
    warp_add_u64(&counters->shadow_rays, shadow);
    if (kCount) {
        warp_add_u64(&counters->node_visits, tc.nodes);
        warp_add_u64(&counters->tri_tests, tc.tris);
    }
    if (err) atomicOr(&counters->error_flags, err);
}

// ------------------------------------------------------------------------------------------------
// DenoisePass + ToneMappingPass (CPURenderer.cpp:452-576) as one gather kernel.
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ float aces(float c, float exposure) {
    const float x = c * exposure;
    float y = (x * (x * 2.51f + 0.03f)) / (x * (x * 2.43f + 0.59f) + 0.14f);
    y = (1.f < y) ? 1.f : y;
    y = (y < 0.f) ? 0.f : y;
    return y;
}

__global__ void __launch_bounds__(256) k_resolve(FrameBuffers fb, float f, float exposure, uint32_t spatial) {
    const uint32_t i = blockIdx.x * 32u + (threadIdx.x & 31u);
    const uint32_t j = blockIdx.y * 8u + (threadIdx.x >> 5);
    if (i >= fb.width || j >= fb.height) return;
    const size_t k = static_cast<size_t>(j) * fb.width + i;
    float4 in = fb.gcolor[k];
    if (spatial) in = spatial_fill(fb.gcolor, fb.gnormal, i, j, fb.width, fb.height, in);
    float4 a = fb.fb[k];
    a = make_float4(in.x + (a.x - in.x) * f, in.y + (a.y - in.y) * f, in.z + (a.z - in.z) * f, in.w + (a.w - in.w) * f);
    fb.fb[k] = a;
    ushort4 o;
    o.x = __half_as_ushort(__float2half_rn(aces(a.x, exposure)));
    o.y = __half_as_ushort(__float2half_rn(aces(a.y, exposure)));
    o.z = __half_as_ushort(__float2half_rn(aces(a.z, exposure)));
    o.w = __half_as_ushort(__float2half_rn(1.f));
    fb.out[static_cast<size_t>(fb.height - 1 - j) * fb.width + i] = o;
}

}  // namespace

cudaError_t launch_trace(const DevScene &scene, const float *rays, uint64_t n, void *hits, int mode, bool count,
                         Counters *counters, int num_sms, cudaStream_t stream, LaunchEvents *ev) {
    cudaError_t e = cudaMemsetAsync(&counters->queue_counters[0], 0, sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    const uint64_t warps_needed = (n + 31) / 32;
    uint64_t blocks = static_cast<uint64_t>(num_sms) * 12;  // persistent: ~12 blocks of 4 warps per SM
    blocks = std::min<uint64_t>(blocks, (warps_needed + 3) / 4);
    if (blocks == 0) blocks = 1;
    auto *h = static_cast<spk_hit_dev *>(hits);
    const unsigned g = static_cast<unsigned>(blocks);
    if (ev) ev->before(stream);
    if (mode == kTraceClosest) {
        if (count) {
            k_trace<kTraceClosest, true><<<g, 128, 0, stream>>>(scene, rays, n, h, counters);
        } else {
            k_trace<kTraceClosest, false><<<g, 128, 0, stream>>>(scene, rays, n, h, counters);
        }
    } else {
        if (count) {
            k_trace<kTraceAnyRef, true><<<g, 128, 0, stream>>>(scene, rays, n, h, counters);
        } else {
            k_trace<kTraceAnyRef, false><<<g, 128, 0, stream>>>(scene, rays, n, h, counters);
        }
    }
    if (ev) ev->after(stream);
    return cudaGetLastError();
}

cudaError_t launch_render_mega(const DevScene &scene, const DevCamera &cam, const FrameBuffers &fbuf,
                               const RenderParams &p, bool count, Counters *counters, cudaStream_t stream,
                               LaunchEvents *ev) {
    const dim3 grid((fbuf.width + 15) / 16, (fbuf.height + 7) / 8);
    using Kernel = void (*)(DevScene, DevCamera, FrameBuffers, RenderParams, Counters *);
    static const Kernel table[2][2][2] = {
        {{k_render_mega<0, false, false>, k_render_mega<0, false, true>},
         {k_render_mega<0, true, false>, k_render_mega<0, true, true>}},
        {{k_render_mega<1, false, false>, k_render_mega<1, false, true>},
         {k_render_mega<1, true, false>, k_render_mega<1, true, true>}}};
    const Kernel k = table[p.rng == 0 ? 0 : 1][count ? 1 : 0][p.enable_nee ? 1 : 0];
    if (ev) ev->before(stream);
    k<<<grid, 128, 0, stream>>>(scene, cam, fbuf, p, counters);
    if (ev) ev->after(stream);
    return cudaGetLastError();
}

// Primary-hit guides, the G-buffer WritePrimaryHitGBuffer writes (ray_trace.cs.slang:282-351): a
// pixel-centre ray from the camera position (no jitter, no lens), uv = (pixel + 0.5) / (resolution - 1)
// with v flipped for the top-down pixel row. A hit within TMax = 1000 stores normalize(normal) and the
// linear depth along normalize(cross(max_v, max_u)), the base colour and 2 (emissive) or 1; a miss stores
// zeros. Rows are bottom-up like the frame buffer.
__global__ void __launch_bounds__(128) k_guides(DevScene S, DevCamera cam, uint32_t w, uint32_t h, float4 *nd,
                                                float4 *alb, Counters *counters) {
    const uint32_t i = blockIdx.x * 16u + (threadIdx.x & 15u);
    const uint32_t j = blockIdx.y * 8u + (threadIdx.x >> 4);
    if (i >= w || j >= h) return;
    const uint32_t py = h - 1 - j;
    const float pw = 1.f / static_cast<float>(w - 1), ph = 1.f / static_cast<float>(h - 1);
    const float u = (static_cast<float>(i) + 0.5f) * pw;
    const float v = 1.f - (static_cast<float>(py) + 0.5f) * ph;
    const f3 o = mk3(cam.position[0], cam.position[1], cam.position[2]);
    const f3 focus = mk3(cam.lower_left[0], cam.lower_left[1], cam.lower_left[2]) +
                     u * mk3(cam.max_u[0], cam.max_u[1], cam.max_u[2]) + v * mk3(cam.max_v[0], cam.max_v[1], cam.max_v[2]);
    const f3 d = normalized(focus - o);
    uint32_t err = 0;
    const TraceResult hit = trace_ray<kTraceClosest>(S, o, d, kFltMax, err);
    const size_t pix = static_cast<size_t>(j) * w + i;
    if (err) atomicOr(&counters->error_flags, err);
    if (hit.inst == kInvalid || !(hit.t <= 1000.f)) {
        nd[pix] = make_float4(0.f, 0.f, 0.f, 0.f);
        alb[pix] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const Surface surf = make_surface(S, hit, o, d);
    const DevMaterial mat = resolve_material(S, S.materials[surf.material], surf.uv);
    const f3 n = normalized(surf.normal);
    const f3 front = normalized(cross(mk3(cam.max_v[0], cam.max_v[1], cam.max_v[2]), mk3(cam.max_u[0], cam.max_u[1], cam.max_u[2])));
    nd[pix] = make_float4(n.x, n.y, n.z, dot3(surf.location - o, front));
    alb[pix] = make_float4(mat.base[0], mat.base[1], mat.base[2], mat.is_emissive ? 2.f : 1.f);
}

cudaError_t launch_guides(const DevScene &scene, const DevCamera &cam, uint32_t w, uint32_t h, float4 *nd, float4 *alb,
                          Counters *counters, cudaStream_t stream) {
    const dim3 grid((w + 15) / 16, (h + 7) / 8);
    k_guides<<<grid, 128, 0, stream>>>(scene, cam, w, h, nd, alb, counters);
    return cudaGetLastError();
}

cudaError_t launch_resolve(const FrameBuffers &fbuf, float moving_average, float exposure, uint32_t spatial_denoise,
                           cudaStream_t stream) {
    const dim3 grid((fbuf.width + 31) / 32, (fbuf.height + 7) / 8);
    k_resolve<<<grid, 256, 0, stream>>>(fbuf, moving_average, exposure, spatial_denoise);
    return cudaGetLastError();
}

}  // namespace spk
