// wavefront.cu -- stage kernels of the wavefront BasePass (see wavefront.cuh).
//
// Compiled with -fmad=false like kernels.cu so every path computes bit-identically to the one-kernel form.
#include <cuda_fp16.h>

#include <algorithm>
#include <cstring>

#include "wavefront.cuh"
#include "fault.h"

#ifndef SPK_SHADE_MIN_BLOCKS
#define SPK_SHADE_MIN_BLOCKS 8  // resident 128-thread blocks per SM the shading kernels are compiled for (64 registers)
#endif

namespace spk {
namespace {

// queue_counters slots
constexpr int kLen0 = 0;          // length of queue 0 (queue 1's length is slot 1)
constexpr int kCursor = 2;         // pop cursor of the running persistent stage
constexpr int kPacketCursor = 3;   // pop cursors of the packet walks, one and two rays per lane (reset with
constexpr int kPacket2Cursor = 4;  // kCursor)
constexpr int kShadowLen = 5;      // occlusion rays queued by the iteration's shade stage
constexpr int kNeeLen = 6;         // light-sampling vertices of the iteration's shade stage
constexpr int kShadowCursor = 7;   // pop cursor of the shadow stage
// Leading extend-queue entries walked in packets (primary rays queued in sample-item order, >= kPacketMinSamples
// of a pixel in a row): the first kPacket2Queue with two rays per lane, the rest up to kPacketQueue with one.
// Both 0 after shade.
constexpr int kPacketQueue = 8;
constexpr int kPacket2Queue = 9;
constexpr int kNextItem = 10;  // next (frame, pixel) sample item to hand out

template <int kKind>
__device__ __forceinline__ void load_rng(const uint4 *rng, uint32_t pid, Rng &r) {
    const uint4 a = rng[2 * static_cast<size_t>(pid)];
    r.s[0] = a.x;
    r.s[1] = a.y;
    r.s[2] = a.z;
    r.s[3] = a.w;
    if (kKind == 1) {
        const uint4 b = rng[2 * static_cast<size_t>(pid) + 1];
        r.s[4] = b.x;
        r.s[5] = b.y;
        r.s[6] = b.z;
        r.s[7] = b.w;
    }
}

template <int kKind>
__device__ __forceinline__ void store_rng(uint4 *rng, uint32_t pid, const Rng &r) {
    rng[2 * static_cast<size_t>(pid)] = make_uint4(r.s[0], r.s[1], r.s[2], r.s[3]);
    if (kKind == 1) rng[2 * static_cast<size_t>(pid) + 1] = make_uint4(r.s[4], r.s[5], r.s[6], r.s[7]);
}

// Warp-aggregated append to a queue: one atomic per warp.
__device__ __forceinline__ void queue_push(uint32_t *queue, unsigned long long *len, uint32_t value, bool active) {
    const uint32_t mask = __ballot_sync(__activemask(), active);
    if (mask == 0) return;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t leader = __ffs(mask) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(len, static_cast<unsigned long long>(__popc(mask)));
    base = __shfl_sync(__activemask(), base, leader);
    if (active) queue[base + __popc(mask & ((1u << lane) - 1u))] = value;
}

// Queues the occlusion rays a deferred light-sampling vertex prepared (bit k of `nee_rays`: ray k) and the
// vertex itself, flagged when its path ended there. Every lane of the warp calls it.
__device__ __forceinline__ void queue_nee(const WavefrontState &s, Counters *counters, uint32_t slot,
                                          uint32_t nee_rays, bool ended) {
    unsigned long long *qc = counters->queue_counters;
    queue_push(s.shadow_queue, &qc[kShadowLen], 2u * slot, (nee_rays & 1u) != 0u);
    queue_push(s.shadow_queue, &qc[kShadowLen], 2u * slot + 1u, (nee_rays & 2u) != 0u);
    queue_push(s.nee_list, &qc[kNeeLen], slot | (ended ? 0x80000000u : 0u), nee_rays != 0u);
}

// A path's next ray in 24 bytes: origin xyz and direction x in one 16-byte record, direction yz in another.
__device__ __forceinline__ void store_ray(const WavefrontState &s, uint32_t pid, f3 o, f3 d) {
    s.ray_a[pid] = make_float4(o.x, o.y, o.z, d.x);
    s.ray_b[pid] = make_float2(d.y, d.z);
}
__device__ __forceinline__ void load_ray(const WavefrontState &s, uint32_t pid, f3 &o, f3 &d) {
    const float4 a = s.ray_a[pid];
    const float2 b = s.ray_b[pid];
    o = mk3(a.x, a.y, a.z);
    d = mk3(a.w, b.x, b.y);
}

// RenderPixel's start of a sample (CPURenderer.cpp:398-406, 436-444): reseed, jitter, camera ray.
template <int kKind>
__device__ __forceinline__ void start_path(const DevCamera &cam, const RenderParams &p, const WavefrontState &s,
                                           uint32_t pid, uint32_t i, uint32_t j, uint32_t w, uint32_t h,
                                           uint32_t frame_seed) {
    Rng rng;
    rng_seed_pixel<kKind>(rng, p.seed, i, j, w, h, frame_seed);
    const float pw = 1.f / static_cast<float>(w - 1);
    const float ph = 1.f / static_cast<float>(h - 1);
    const float u = (static_cast<float>(i) + rng_unit<kKind>(rng)) * pw;
    const float v = (static_cast<float>(j) + rng_unit<kKind>(rng)) * ph;
    f3 o, d;
    camera_ray<kKind>(cam, rng, u, v, o, d);
    store_ray(s, pid, o, d);
    // Throughput 1, colour 0 with valid flag 1 and no previous light-sampling pdf: shade_path takes these
    // at bounce 0 without reading them, so they are not stored here.
    store_rng<kKind>(s.rng, pid, rng);
}

// Next-event estimation modes of the shading kernels.
enum : int { kNeeOff = 0, kNeeInline = 1, kNeeDeferred = 2 };

// One bounce of SamplePixel's loop body (CPURenderer.cpp:261-368) for path `pid` whose closest hit is
// in s.hit: sky on a miss, emission, BSDF sample, throughput cut-off, Russian roulette, and (with NEE)
// next-event estimation at diffuse-branch vertices with MIS on the emission the BSDF rays collect.
// kNeeInline walks the two occlusion rays here; kNeeDeferred stores them with their radiance for the
// shadow stage and returns in `nee_rays` which were queued (bit k: ray k), the colour still without them.
// Returns whether the path continues (the next ray is then in s.ray_a / s.ray_b).
template <int kKind, int kNee>
__device__ __forceinline__ bool shade_path(const DevScene &S, const WavefrontState &s, uint32_t pid,
                                           uint32_t bounce, float4 *gnormal, uint32_t &shadow, uint32_t &err,
                                           uint32_t &nee_rays, size_t gnormal_index) {
    constexpr bool nee = kNee != kNeeOff;
    nee_rays = 0u;
    bool alive = false;
    const float4 hit4 = s.hit[pid];
    const uint32_t inst = __float_as_uint(hit4.w);
    f3 o, d;
    load_ray(s, pid, o, d);
    // A path's first segment starts from throughput 1, colour 0, valid flag 1 and no light-sampling pdf
    // (start_path leaves them unstored).
    const float4 c4 = bounce == 0 ? make_float4(0.f, 0.f, 0.f, 1.f) : s.color[pid];
    f3 color = mk3(c4.x, c4.y, c4.z);
    const float4 t4 = bounce == 0 ? make_float4(1.f, 1.f, 1.f, 0.f) : s.thr[pid];
    f3 thr = mk3(t4.x, t4.y, t4.z);
    float valid = c4.w;
    const float prev_pdf = nee && bounce > 0 ? s.prev_pdf[pid] : 0.f;
    if (inst == kInvalid) {
        if (S.sky_mode != 0u) {
            f3 c = cmul(sky_eval(S, d), thr);
            if (prev_pdf > 0.f) c = c * mis_weight(prev_pdf, prev_pdf);
            color = color + c;
        }
    } else {
        const TraceResult h{hit4.x, hit4.y, hit4.z, inst, s.hit_face[pid]};
        const Surface surf = make_surface(S, h, o, d);
        const DevMaterial mat = resolve_material(S, S.materials[surf.material], surf.uv);
        if (bounce == 0 && gnormal)
            gnormal[gnormal_index] = make_float4(surf.normal.x, surf.normal.y, surf.normal.z, 0.f);
        if (mat.is_emissive) {
            f3 c = cmul(mk3(mat.emissive[0], mat.emissive[1], mat.emissive[2]), thr);
            if (prev_pdf > 0.f) c = c * bsdf_hit_weight(S, prev_pdf, h, d);
            color = color + c;
        } else {
            Rng rng;
            load_rng<kKind>(s.rng, pid, rng);
            f3 next_dir;
            float dz = -1.f;
            const f3 this_thr =
                sample_surface<kKind>(rng, mat, d, surf.normal, surf.tangent, next_dir, nee ? &dz : nullptr);
            float next_pdf = 0.f;
            if (dz >= 0.f) {
                const f3 base = mk3(mat.base[0], mat.base[1], mat.base[2]);
                if (kNee == kNeeDeferred) {
                    NeeRay r[2];
                    nee_prepare<kKind>(S, rng, surf, base, thr, r[0], r[1]);
                    if (r[0].valid || r[1].valid) {
#pragma unroll
                        for (int k = 0; k < 2; ++k) {
                            const size_t e = 2 * static_cast<size_t>(pid) + k;
                            if (r[k].valid) {
                                s.shadow_o[e] = make_float4(r[k].o.x, r[k].o.y, r[k].o.z, r[k].tmax);
                                s.shadow_d[e] = make_float4(r[k].d.x, r[k].d.y, r[k].d.z, 0.f);
                                s.nee_contrib[e] = make_float4(r[k].contrib.x, r[k].contrib.y, r[k].contrib.z, 1.f);
                                nee_rays |= 1u << k;
                                ++shadow;
                            } else {
                                s.nee_contrib[e] = make_float4(0.f, 0.f, 0.f, 0.f);
                            }
                        }
                    }
                } else {
                    nee_direct<kKind, false>(S, rng, surf, base, thr, color, shadow, err, nullptr);
                }
                next_pdf = dz * kInvPi;
            }
            thr = cmul(thr, this_thr);
            if (sqnorm(thr) < kEps) {
                valid = -1.f;
            } else {
                bool survive = true;
                if (bounce >= 3) {
                    float pr = max_std(thr.x, max_std(thr.y, thr.z));
                    pr = (pr < 0.05f) ? 0.05f : (1.0f < pr) ? 1.0f : pr;
                    if (rng_unit<kKind>(rng) > pr) {
                        survive = false;
                    } else {
                        thr = mk3(thr.x / pr, thr.y / pr, thr.z / pr);
                    }
                }
                if (survive) {
                    const f3 no = surf.location + next_dir * kTolerance;
                    store_ray(s, pid, no, next_dir);
                    if (nee) s.prev_pdf[pid] = next_pdf;
                    alive = true;
                }
            }
            store_rng<kKind>(s.rng, pid, rng);
            s.thr[pid] = make_float4(thr.x, thr.y, thr.z, 0.f);
        }
    }
    s.color[pid] = make_float4(color.x, color.y, color.z, valid);
    return alive;
}

// ------------------------------------------------------------------------------------------------
// Frame-by-frame schedule
// ------------------------------------------------------------------------------------------------
template <int kKind>
__global__ void __launch_bounds__(128) k_wf_generate(DevCamera cam, FrameBuffers fb, RenderParams p, WavefrontState s,
                                                     Counters *counters) {
    const uint32_t i = blockIdx.x * 16u + (threadIdx.x & 15u);
    const uint32_t j = blockIdx.y * 8u + (threadIdx.x >> 4);
    if (i >= fb.width || j >= fb.height) return;
    const uint32_t pid = j * fb.width + i;
    start_path<kKind>(cam, p, s, pid, i, j, fb.width, fb.height, p.frame_seed);
    if (p.spatial_denoise) fb.gnormal[pid] = make_float4(0.f, 0.f, 0.f, 0.f);
    s.queue[0][pid] = pid;
    if (pid == 0) {
        counters->queue_counters[kLen0] = static_cast<unsigned long long>(fb.width) * fb.height;
        counters->queue_counters[kPacketQueue] = 0u;  // one sample per pixel: no packets
        counters->queue_counters[kPacket2Queue] = 0u;
    }
}

// Extend: persistent warps pull paths from the queue, refilling lanes whose walk has finished. With
// kBatch each path traces in its own scene (the TLAS root its slot recorded at start). The first
// kPacketQueue entries of a queue (primary rays a generate kernel queued in sample-item order: 32
// consecutive paths are a pixel's samples, or a few neighbouring pixels') are walked by the kPackets form in
// packets of 32 instead, the rest by the persistent form. Both forms are launched every stage and return at
// once when they have nothing to walk, so the split needs no host round trip (and stays inside a replayed
// graph).
template <bool kCount, bool kBatch = false, int kPackets = 0>
__global__ void __launch_bounds__(128, kPackets == 2   ? SPK_PACKET2_MIN_BLOCKS
                                       : kPackets == 1 ? SPK_PACKET_MIN_BLOCKS
                                                       : SPK_WALK_MIN_BLOCKS)
    k_wf_extend(DevScene S, WavefrontState s, int in_queue, Counters *counters) {
    const unsigned long long len = counters->queue_counters[in_queue];
    const unsigned long long p1 = min(counters->queue_counters[kPacketQueue], len);
    const unsigned long long p2 = min(counters->queue_counters[kPacket2Queue], p1);
    const unsigned long long first = kPackets == 2 ? 0ull : kPackets == 1 ? p2 : p1;
    const unsigned long long n = (kPackets == 2 ? p2 : kPackets == 1 ? p1 : len) - first;
    if (n == 0) return;
    uint32_t err = 0, done = 0;
    TraceCounts tc;
    const uint32_t *queue = s.queue[in_queue] + first;
    uint32_t pid = 0;
    auto fetch = [&](unsigned long long q, f3 &o, f3 &d, float &) {
        pid = queue[q];
        load_ray(s, pid, o, d);
        return kBatch ? s.slot_root[pid] : S.tlas_root;
    };
    auto store = [&](uint32_t p, const TraceResult &h) {
        s.hit[p] = make_float4(h.t, h.u, h.v, __uint_as_float(h.inst));
        s.hit_face[p] = h.face;
        ++done;
    };
    if constexpr (kPackets != 0) {
        walk_packets<kCount, kPackets>(S, &counters->queue_counters[kPackets == 2 ? kPacket2Cursor : kPacketCursor], n,
                                       err, &tc, fetch,
                                       [&](unsigned long long q, const TraceResult &h) { store(queue[q], h); });
    } else {
        walk_persistent<kTraceClosest, kCount>(S, &counters->queue_counters[kCursor], n, kFltMax, err, &tc, fetch,
                                               [&](unsigned long long, const TraceResult &h) { store(pid, h); });
    }
    warp_add_u64(&counters->extension_rays, done);
    if (kCount) {
        warp_add_u64(&counters->node_visits, tc.nodes);
        warp_add_u64(&counters->tri_tests, tc.tris);
    }
    if (err) atomicOr(&counters->error_flags, err);
}

template <int kKind, int kNee>
__global__ void __launch_bounds__(128, SPK_SHADE_MIN_BLOCKS) k_wf_shade(DevScene S, FrameBuffers fb, RenderParams p, WavefrontState s,
                                                  int in_queue, uint32_t bounce, Counters *counters) {
    uint32_t shadow = 0, err = 0;
    const unsigned long long n = counters->queue_counters[in_queue];
    const int out_queue = in_queue ^ 1;
    if (blockIdx.x == 0 && threadIdx.x == 0) {  // the next queue is mixed
        counters->queue_counters[kPacketQueue] = 0u;
        counters->queue_counters[kPacket2Queue] = 0u;
    }
    const uint32_t *queue = s.queue[in_queue];
    for (unsigned long long q0 = static_cast<unsigned long long>(blockIdx.x) * blockDim.x; q0 < n;
         q0 += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const unsigned long long q = q0 + threadIdx.x;
        bool alive = false;
        uint32_t pid = 0, nee_rays = 0;
        if (q < n) {
            pid = queue[q];
            alive = shade_path<kKind, kNee>(S, s, pid, bounce, p.spatial_denoise ? fb.gnormal : nullptr, shadow, err,
                                             nee_rays, pid);
        }
        if constexpr (kNee == kNeeDeferred) queue_nee(s, counters, pid, nee_rays, false);
        queue_push(s.queue[out_queue], &counters->queue_counters[out_queue], pid, alive && bounce + 1 < p.bounce);
    }
    warp_add_u64(&counters->shadow_rays, shadow);
    if (err) atomicOr(&counters->error_flags, err);
}

__global__ void __launch_bounds__(256) k_wf_finish(FrameBuffers fb, WavefrontState s) {
    const uint32_t pid = blockIdx.x * blockDim.x + threadIdx.x;
    if (pid >= fb.width * fb.height) return;
    const float4 c = s.color[pid];
    fb.gcolor[pid] = make_float4(clamp_sample(c.x), clamp_sample(c.y), clamp_sample(c.z), c.w);
}

// ------------------------------------------------------------------------------------------------
// Multi-frame schedule with path regeneration
// ------------------------------------------------------------------------------------------------

#ifndef SPK_ITEM_TILES
#define SPK_ITEM_TILES 1  // 1: a frame's items walk the image in 32-pixel tiles (0: row by row)
#endif
#ifndef SPK_ITEM_TILE_W
#define SPK_ITEM_TILE_W 4  // tile width (4, 8 or 16); the height is 32 / width
#endif

// Pixel of the q-th sample item of a frame. With SPK_ITEM_TILES the items go through the image in 8 x 4
// pixel tiles, tile after tile in row-major order, so the 32 lanes of a warp trace a compact block of
// pixels (tighter primary-ray bundles than 32 pixels of one row); row-major order when the image is not a
// whole number of tiles. Results never depend on this order: each sample keeps its own pixel and seed.
__device__ __forceinline__ uint32_t item_pixel(uint32_t q, uint32_t w, uint32_t h) {
    constexpr uint32_t tw = SPK_ITEM_TILE_W, th = 32u / SPK_ITEM_TILE_W;
    static_assert(tw * th == 32u && (tw & (tw - 1u)) == 0u, "32-pixel tiles");
    if (!SPK_ITEM_TILES || (w % tw) || (h % th)) return q;
    const uint32_t tile = q >> 5, j = q & 31u, tiles_x = w / tw;
    const uint32_t tx = tile % tiles_x, ty = tile / tiles_x;
    return (ty * th + j / tw) * w + tx * tw + (j % tw);
}

#ifndef SPK_ITEM_ORDER
#define SPK_ITEM_ORDER 1  // 1: frame fastest (a warp's items are consecutive frames of one pixel); 0: frame-major
#endif

// Slot `slot` starts sample item `item` of the pass (`total_items` = frames x pixels). Frame-fastest order:
// item = q * frames + frame, pixel item_pixel(q), so the lanes of a warp trace samples of the same pixel in
// consecutive frames (primary rays that differ only by their jitter and lens sample). Frame-major order:
// item = frame * pixels + q. The slot records the sample's index frame * pixels + pixel, where its result
// is stored; results never depend on the order (each sample keeps its pixel and seed).
template <int kKind>
__device__ __forceinline__ void start_item(const DevCamera &cam, const RenderParams &p, const WavefrontState &s,
                                           uint32_t slot, uint32_t item, uint32_t w, uint32_t h,
                                           uint32_t frame_base, uint32_t total_items) {
    const uint32_t npix = w * h;
#if SPK_ITEM_ORDER == 1
    const uint32_t frames = total_items / npix;
    const uint32_t q = item / frames, k = item - q * frames, pid = item_pixel(q, w, h);
#else
    (void)total_items;
    const uint32_t k = item / npix, pid = item_pixel(item - k * npix, w, h);
#endif
    start_path<kKind>(cam, p, s, slot, pid % w, pid / w, w, h, s.frame_seed[frame_base + k]);
    s.slot_item[slot] = k * npix + pid;
    s.slot_state[slot] = 0u;
    if (p.spatial_denoise) s.sample_normals[k * npix + pid] = make_float4(0.f, 0.f, 0.f, 0.f);  // a miss: sky
}

// Starts the first `initial` sample items of the pass, item i in slot i.
template <int kKind>
__global__ void __launch_bounds__(128) k_mf_generate(DevCamera cam, FrameBuffers fb, RenderParams p,
                                                     WavefrontState s, uint32_t frame_base, uint32_t initial,
                                                     uint32_t total_items, uint32_t packets, Counters *counters) {
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= initial) return;
    start_item<kKind>(cam, p, s, slot, slot, fb.width, fb.height, frame_base, total_items);
    s.queue[0][slot] = slot;
    if (slot == 0) {
        counters->queue_counters[kLen0] = initial;
        counters->queue_counters[kNextItem] = initial;
        const uint32_t frames = total_items / (fb.width * fb.height);
        const bool pk = SPK_ITEM_ORDER == 1 && packets && frames >= kPacketMinSamples;
        counters->queue_counters[kPacketQueue] = pk ? initial : 0u;
        counters->queue_counters[kPacket2Queue] = pk && frames >= kPacket2MinSamples ? initial : 0u;
    }
}

// Shade one segment per live slot. A finished sample stores its clamped result (RenderPixel's 6.0 clamp,
// CPURenderer.cpp:408) at its item, and the slot takes the next item from the global counter.
template <int kKind, int kNee>
__global__ void __launch_bounds__(128, SPK_SHADE_MIN_BLOCKS) k_mf_shade(DevScene S, DevCamera cam, FrameBuffers fb, RenderParams p,
                                                  WavefrontState s, int in_queue, uint32_t frame_base,
                                                  uint32_t total_items, Counters *counters) {
    uint32_t shadow = 0, err = 0;
    const unsigned long long n = counters->queue_counters[in_queue];
    const int out_queue = in_queue ^ 1;
    if (blockIdx.x == 0 && threadIdx.x == 0) {  // the next queue is mixed
        counters->queue_counters[kPacketQueue] = 0u;
        counters->queue_counters[kPacket2Queue] = 0u;
    }
    const uint32_t *queue = s.queue[in_queue];
    const uint32_t lane = threadIdx.x & 31u;
    for (unsigned long long q0 = static_cast<unsigned long long>(blockIdx.x) * blockDim.x; q0 < n;
         q0 += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const unsigned long long q = q0 + threadIdx.x;
        bool push = false, need = false, alive = false;
        uint32_t slot = 0, nee_rays = 0;
        if (q < n) {
            slot = queue[q];
            const uint32_t bounce = s.slot_state[slot];
            alive = shade_path<kKind, kNee>(S, s, slot, bounce, p.spatial_denoise ? s.sample_normals : nullptr, shadow,
                                            err, nee_rays, s.slot_item[slot]) &&
                    bounce + 1 < p.bounce;
            if (alive) {
                s.slot_state[slot] = bounce + 1u;
                push = true;
            } else if (nee_rays == 0u) {
                const float4 c = s.color[slot];
                s.samples[s.slot_item[slot]] =
                    make_float4(clamp_sample(c.x), clamp_sample(c.y), clamp_sample(c.z), c.w);
                need = true;
            }
            // else: the path ended at a light-sampling vertex; the accumulate stage adds its NEE radiance,
            // stores the sample and starts the slot's next item
        }
        if constexpr (kNee == kNeeDeferred) queue_nee(s, counters, slot, nee_rays, !alive);
        // Warp-aggregated hand-out of new sample items to the lanes whose path ended.
        const uint32_t need_mask = __ballot_sync(0xFFFFFFFFu, need);
        if (need_mask) {
            unsigned long long base = 0;
            if (lane == static_cast<uint32_t>(__ffs(need_mask) - 1))
                base = atomicAdd(&counters->queue_counters[kNextItem], static_cast<unsigned long long>(__popc(need_mask)));
            base = __shfl_sync(0xFFFFFFFFu, base, __ffs(need_mask) - 1);
            if (need) {
                const unsigned long long item = base + __popc(need_mask & ((1u << lane) - 1u));
                if (item < total_items) {
                    start_item<kKind>(cam, p, s, slot, static_cast<uint32_t>(item), fb.width, fb.height, frame_base,
                                      total_items);
                    push = true;
                }
            }
        }
        queue_push(s.queue[out_queue], &counters->queue_counters[out_queue], slot, push);
    }
    warp_add_u64(&counters->shadow_rays, shadow);
    if (err) atomicOr(&counters->error_flags, err);
}

// ------------------------------------------------------------------------------------------------
// Counting sorts of a queue (material class before shading, ray key before extension)
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t sort_class(const DevScene &S, const WavefrontState &s, uint32_t pid) {
    const uint32_t inst = __float_as_uint(s.hit[pid].w);
    if (inst == kInvalid) return kSortBuckets - 1;
    return min(S.instances[inst].material, kSortBuckets - 2);
}

__device__ __forceinline__ uint32_t spread3(uint32_t v) {  // bits b2 b1 b0 -> b2 0 0 b1 0 0 b0
    return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4);
}

__device__ __forceinline__ uint32_t ray_key(const DevScene &S, const WavefrontState &s, uint32_t pid) {
    f3 o, d;
    load_ray(s, pid, o, d);
    uint32_t c[3];
    const float ov[3] = {o.x, o.y, o.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float f = (ov[a] - S.box_lo[a]) * S.box_scale[a];
        c[a] = f > 0.f ? min(static_cast<uint32_t>(f), 7u) : 0u;
    }
    const uint32_t oct = (d.x < 0.f ? 1u : 0u) | (d.y < 0.f ? 2u : 0u) | (d.z < 0.f ? 4u : 0u);
    return ((spread3(c[0]) | (spread3(c[1]) << 1) | (spread3(c[2]) << 2)) << 3) | oct;
}

template <int kKey>  // 0: material class of the hit, 1: ray (origin cell, direction octant)
struct SortKey {
    static constexpr uint32_t kBuckets = kKey == 0 ? kSortBuckets : kRaySortBuckets;
    __device__ static uint32_t of(const DevScene &S, const WavefrontState &s, uint32_t pid) {
        return kKey == 0 ? sort_class(S, s, pid) : ray_key(S, s, pid);
    }
};

template <int kKey>
__global__ void __launch_bounds__(256) k_sort_hist(DevScene S, WavefrontState s, int in_queue, Counters *counters) {
    constexpr uint32_t B = SortKey<kKey>::kBuckets;
    __shared__ uint32_t h[B];
    for (uint32_t b = threadIdx.x; b < B; b += blockDim.x) h[b] = 0;
    __syncthreads();
    const unsigned long long n = counters->queue_counters[in_queue];
    const uint32_t *queue = s.queue[in_queue];
    for (unsigned long long q = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
         q += static_cast<unsigned long long>(gridDim.x) * blockDim.x)
        atomicAdd(&h[SortKey<kKey>::of(S, s, queue[q])], 1u);
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < B; b += blockDim.x)
        if (h[b]) atomicAdd(&s.sort_hist[b], h[b]);
}

// Exclusive scan of the histogram (1024 threads, B / 1024 buckets each) into the scatter cursors; clears
// the histogram for the next sort.
template <int kKey>
__global__ void __launch_bounds__(1024) k_sort_scan(WavefrontState s) {
    constexpr uint32_t B = SortKey<kKey>::kBuckets;
    constexpr uint32_t per = (B + 1023) / 1024;
    __shared__ uint32_t warp_sums[32];
    const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
    uint32_t v[per];
    uint32_t mine = 0;
#pragma unroll
    for (uint32_t k = 0; k < per; ++k) {
        const uint32_t b = t * per + k;
        v[k] = b < B ? s.sort_hist[b] : 0u;
        if (b < B) s.sort_hist[b] = 0;
        mine += v[k];
    }
    uint32_t incl = mine;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t x = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= static_cast<uint32_t>(o)) incl += x;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_sums[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t x = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= static_cast<uint32_t>(o)) w += x;
        }
        warp_sums[lane] = w;  // inclusive prefix of warp totals
    }
    __syncthreads();
    uint32_t run = incl - mine + (warp > 0 ? warp_sums[warp - 1] : 0u);
#pragma unroll
    for (uint32_t k = 0; k < per; ++k) {
        const uint32_t b = t * per + k;
        if (b < B) s.sort_hist[kRaySortBuckets + b] = run;
        run += v[k];
    }
}

template <int kKey>
__global__ void __launch_bounds__(256) k_sort_scatter(DevScene S, WavefrontState s, int in_queue, uint32_t *dst,
                                                      Counters *counters) {
    constexpr uint32_t B = SortKey<kKey>::kBuckets;
    const unsigned long long n = counters->queue_counters[in_queue];
    const uint32_t *queue = s.queue[in_queue];
    const uint32_t lane = threadIdx.x & 31u;
    for (unsigned long long q0 = static_cast<unsigned long long>(blockIdx.x) * blockDim.x; q0 < n;
         q0 += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const unsigned long long q = q0 + threadIdx.x;
        const bool active = q < n;
        const uint32_t pid = active ? queue[q] : 0u;
        const uint32_t key = active ? SortKey<kKey>::of(S, s, pid) : B;  // inactive lanes: own group
        // One atomic per (warp, key): lanes with the same key share a base.
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
        const uint32_t leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if (active && lane == leader) base = atomicAdd(&s.sort_hist[kRaySortBuckets + key], __popc(peers));
        base = __shfl_sync(0xFFFFFFFFu, base, leader);
        if (active) dst[base + __popc(peers & ((1u << lane) - 1u))] = pid;
    }
}

// Enqueues a counting sort of queue `in` by key kKey into `dst`; returns the state the next stage reads
// (its queue `in` replaced by the sorted copy).
// The histogram holds 2 x kRaySortBuckets counters (counts, then cursors) and `dst` the queue's capacity;
// wavefront_alloc sizes both, and sort_buffers_ok checks it before a schedule uses a sort.
bool sort_buffers_ok(const WavefrontState &s) {
    return s.sort_hist != nullptr && s.sort_keys != nullptr && s.sort_keys2 != nullptr;
}

template <int kKey>
WavefrontState enqueue_sort(const DevScene &scene, const WavefrontState &s, int in, uint32_t *dst, Counters *counters,
                            int num_sms, cudaStream_t stream) {
    const unsigned grid = static_cast<unsigned>(num_sms) * 4u;
    k_sort_hist<kKey><<<grid, 256, 0, stream>>>(scene, s, in, counters);
    k_sort_scan<kKey><<<1, 1024, 0, stream>>>(s);
    k_sort_scatter<kKey><<<grid, 256, 0, stream>>>(scene, s, in, dst, counters);
    WavefrontState sorted = s;
    sorted.queue[in] = dst;
    return sorted;
}

// Material sort: group a shade queue by the material class of each path's hit, so the warps of the
// shade stage run one BSDF branch and read one material record.
WavefrontState enqueue_material_sort(const DevScene &scene, const WavefrontState &s, int in, Counters *counters,
                                     int num_sms, cudaStream_t stream) {
    return enqueue_sort<0>(scene, s, in, s.sort_keys, counters, num_sms, stream);
}

// Ray sort: order an extend queue by origin cell and direction octant, so the lanes of a warp walk
// similar rays.
WavefrontState enqueue_ray_sort(const DevScene &scene, const WavefrontState &s, int in, Counters *counters,
                                int num_sms, cudaStream_t stream) {
    return enqueue_sort<1>(scene, s, in, s.sort_keys2, counters, num_sms, stream);
}

__device__ __forceinline__ float aces_tonemap(float c, float exposure) {
    const float x = c * exposure;
    float y = (x * (x * 2.51f + 0.03f)) / (x * (x * 2.43f + 0.59f) + 0.14f);
    y = (1.f < y) ? 1.f : y;
    y = (y < 0.f) ? 0.f : y;
    return y;
}

// DenoisePass temporal lerp of every sample of the pass, in frame order per pixel
// (fb = new + (fb - new) * w_k, CPURenderer.cpp:534-543), then ToneMappingPass (:554-576).
__global__ void __launch_bounds__(256) k_mf_resolve(FrameBuffers fb, WavefrontState s, uint32_t frame_base,
                                                    uint32_t frames, float exposure, uint32_t spatial) {
    const uint32_t pid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t npix = fb.width * fb.height;
    if (pid >= npix) return;
    float4 a = fb.fb[pid];
    for (uint32_t k = 0; k < frames; ++k) {
        float4 n = s.samples[static_cast<size_t>(k) * npix + pid];
        if (spatial)  // DenoisePass's spatial fill of frame k's G-buffer (CPURenderer.cpp:452-526)
            n = spatial_fill(s.samples + static_cast<size_t>(k) * npix, s.sample_normals + static_cast<size_t>(k) * npix,
                             pid % fb.width, pid / fb.width, fb.width, fb.height, n);
        const float f = s.frame_weight[frame_base + k];
        a = make_float4(n.x + (a.x - n.x) * f, n.y + (a.y - n.y) * f, n.z + (a.z - n.z) * f, n.w + (a.w - n.w) * f);
    }
    fb.fb[pid] = a;
    const uint32_t i = pid % fb.width, j = pid / fb.width;
    ushort4 o;
    o.x = __half_as_ushort(__float2half_rn(aces_tonemap(a.x, exposure)));
    o.y = __half_as_ushort(__float2half_rn(aces_tonemap(a.y, exposure)));
    o.z = __half_as_ushort(__float2half_rn(aces_tonemap(a.z, exposure)));
    o.w = __half_as_ushort(__float2half_rn(1.f));
    fb.out[static_cast<size_t>(fb.height - 1 - j) * fb.width + i] = o;
}

// ------------------------------------------------------------------------------------------------
// Batched requests: one wavefront over the sample items of every request (spk_render_batch)
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t find_request(const BatchParams &b, unsigned long long item) {
    uint32_t lo = 0, hi = b.num_reqs;  // last request with item_base <= item
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (b.reqs[mid].item_base <= item) {
            lo = mid;
        } else {
            hi = mid;
        }
    }
    return lo;
}

// Slot `slot` starts global item `item`: request r, frame k, pixel; the same seed, jitter and camera ray
// as frame k of spk_render on that request alone (frame seed base k: one sample per frame).
template <int kKind>
// Returns the item's request.
__device__ __forceinline__ uint32_t start_item_batch(const DevScene &S, const BatchParams &b, const WavefrontState &s,
                                                     uint32_t slot, unsigned long long item) {
    const uint32_t r = find_request(b, item);
    const DevRequest &R = b.reqs[r];
    const unsigned long long local = item - R.item_base;
#if SPK_ITEM_ORDER == 1
    // frame fastest within the request, as start_item: a warp's items are consecutive frames of one pixel
    const uint32_t q = static_cast<uint32_t>(local / R.spp);
    const uint32_t k = static_cast<uint32_t>(local - static_cast<unsigned long long>(q) * R.spp);
    const uint32_t pix = item_pixel(q, R.width, R.height);
#else
    const uint32_t k = static_cast<uint32_t>(local / R.npix);
    const uint32_t pix = static_cast<uint32_t>(local - static_cast<unsigned long long>(k) * R.npix);
#endif
    RenderParams p{k, R.bounce, b.rng, R.seed, 0u, b.enable_nee};
    start_path<kKind>(R.cam, p, s, slot, pix % R.width, pix / R.width, R.width, R.height, k);
    // the sample's index in the frame-major sample buffer k_b_resolve reads
    s.slot_item[slot] = static_cast<uint32_t>(R.item_base + static_cast<unsigned long long>(k) * R.npix + pix);
    s.slot_state[slot] = 0u;
    s.slot_req[slot] = r;
    s.slot_root[slot] = S.descs[R.scene].tlas_root;
    return r;
}

// Starts the group's first `first` sample items, item item_lo + i in slot i, queued at the position
// BatchParams lays out.
template <int kKind>
__global__ void __launch_bounds__(128) k_b_generate(DevScene S, BatchParams b, WavefrontState s, uint32_t first,
                                                    Counters *counters) {
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= first) return;
    const unsigned long long item = b.item_lo + slot;
    const DevRequest &R = b.reqs[start_item_batch<kKind>(S, b, s, slot, item)];
    s.queue[0][R.queue_base + static_cast<uint32_t>(item - R.item_base)] = slot;
    if (slot == 0) {
        counters->queue_counters[kLen0] = first;
        counters->queue_counters[kNextItem] = b.item_lo + first;
        counters->queue_counters[kPacketQueue] = SPK_ITEM_ORDER == 1 ? min(b.packet_items, 1ull * first) : 0ull;
        counters->queue_counters[kPacket2Queue] = SPK_ITEM_ORDER == 1 ? min(b.packet2_items, 1ull * first) : 0ull;
    }
}

template <int kKind, int kNee>
__global__ void __launch_bounds__(128, SPK_SHADE_MIN_BLOCKS) k_b_shade(DevScene S, BatchParams b, WavefrontState s, int in_queue,
                                                 Counters *counters) {
    uint32_t shadow = 0, err = 0;
    const unsigned long long n = counters->queue_counters[in_queue];
    const int out_queue = in_queue ^ 1;
    if (blockIdx.x == 0 && threadIdx.x == 0) {  // the next queue is mixed
        counters->queue_counters[kPacketQueue] = 0u;
        counters->queue_counters[kPacket2Queue] = 0u;
    }
    const uint32_t *queue = s.queue[in_queue];
    const uint32_t lane = threadIdx.x & 31u;
    for (unsigned long long q0 = static_cast<unsigned long long>(blockIdx.x) * blockDim.x; q0 < n;
         q0 += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const unsigned long long q = q0 + threadIdx.x;
        bool push = false, need = false, alive = false;
        uint32_t slot = 0, nee_rays = 0;
        if (q < n) {
            slot = queue[q];
            const DevRequest &R = b.reqs[s.slot_req[slot]];
            const DevScene Sv = scene_view(S, S.descs[R.scene]);
            const uint32_t bounce = s.slot_state[slot];
            alive = shade_path<kKind, kNee>(Sv, s, slot, bounce, nullptr, shadow, err, nee_rays, 0) &&
                    bounce + 1 < R.bounce;
            if (alive) {
                s.slot_state[slot] = bounce + 1u;
                push = true;
            } else if (nee_rays == 0u) {
                const float4 c = s.color[slot];
                s.samples[s.slot_item[slot]] = make_float4(clamp_sample(c.x), clamp_sample(c.y), clamp_sample(c.z), c.w);
                need = true;
            }
        }
        if constexpr (kNee == kNeeDeferred) queue_nee(s, counters, slot, nee_rays, !alive);
        const uint32_t need_mask = __ballot_sync(0xFFFFFFFFu, need);
        if (need_mask) {
            unsigned long long base = 0;
            if (lane == static_cast<uint32_t>(__ffs(need_mask) - 1))
                base = atomicAdd(&counters->queue_counters[kNextItem], static_cast<unsigned long long>(__popc(need_mask)));
            base = __shfl_sync(0xFFFFFFFFu, base, __ffs(need_mask) - 1);
            if (need) {
                const unsigned long long item = base + __popc(need_mask & ((1u << lane) - 1u));
                if (item < b.item_hi) {
                    start_item_batch<kKind>(S, b, s, slot, item);
                    push = true;
                }
            }
        }
        queue_push(s.queue[out_queue], &counters->queue_counters[out_queue], slot, push);
    }
    warp_add_u64(&counters->shadow_rays, shadow);
    if (err) atomicOr(&counters->error_flags, err);
}

// ------------------------------------------------------------------------------------------------
// Shadow stage of next-event estimation: a persistent occlusion walk over the rays the shade stage queued
// (lane refill as in extend), then the in-order addition of the unoccluded radiance.
// ------------------------------------------------------------------------------------------------
template <bool kBatch>
__global__ void __launch_bounds__(128, SPK_SHADOW_MIN_BLOCKS) k_wf_shadow(DevScene S, WavefrontState s,
                                                                       Counters *counters) {
    uint32_t err = 0;
    const unsigned long long n = counters->queue_counters[kShadowLen];
    uint32_t e = 0;
    walk_persistent<kTraceOcclusion, false>(
        S, &counters->queue_counters[kShadowCursor], n, kFltMax, err, nullptr,
        [&](unsigned long long q, f3 &o, f3 &d, float &tmax) {
            e = s.shadow_queue[q];
            const float4 o4 = s.shadow_o[e], d4 = s.shadow_d[e];
            o = mk3(o4.x, o4.y, o4.z);
            d = mk3(d4.x, d4.y, d4.z);
            tmax = o4.w;
            return kBatch ? s.slot_root[e >> 1] : S.tlas_root;
        },
        [&](unsigned long long, const TraceResult &h) {
            if (h.inst == kInvalid) reinterpret_cast<float *>(s.nee_contrib + e)[3] = 2.f;
        });
    if (err) atomicOr(&counters->error_flags, err);
}

// Adds each light-sampling vertex's unoccluded radiance to its path's colour, light before sky (the order
// nee_direct adds them in). kMode 0 (frame by frame): nothing else. kMode 1 (multi-frame) and 2 (batch):
// a path that ended at the vertex stores its clamped sample and its slot starts the next item, as the
// shade stage does for paths that end without pending radiance.
template <int kKind, int kMode>
__global__ void __launch_bounds__(128, SPK_SHADE_MIN_BLOCKS) k_nee_accumulate(DevCamera cam, FrameBuffers fb, RenderParams p,
                                                                            DevScene S, BatchParams b, WavefrontState s,
                                                                            int out_queue, uint32_t frame_base,
                                                                            uint32_t total_items, Counters *counters) {
    const unsigned long long n = counters->queue_counters[kNeeLen];
    const uint32_t lane = threadIdx.x & 31u;
    for (unsigned long long q0 = static_cast<unsigned long long>(blockIdx.x) * blockDim.x; q0 < n;
         q0 += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const unsigned long long q = q0 + threadIdx.x;
        bool push = false, need = false;
        uint32_t slot = 0;
        if (q < n) {
            const uint32_t entry = s.nee_list[q];
            slot = entry & 0x7FFFFFFFu;
            const float4 c4 = s.color[slot];
            f3 color = mk3(c4.x, c4.y, c4.z);
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const float4 a = s.nee_contrib[2 * static_cast<size_t>(slot) + k];
                if (a.w == 2.f) color = color + mk3(a.x, a.y, a.z);
            }
            s.color[slot] = make_float4(color.x, color.y, color.z, c4.w);
            if (kMode != 0 && (entry >> 31)) {
                s.samples[s.slot_item[slot]] =
                    make_float4(clamp_sample(color.x), clamp_sample(color.y), clamp_sample(color.z), c4.w);
                need = true;
            }
        }
        if constexpr (kMode != 0) {
            const uint32_t need_mask = __ballot_sync(0xFFFFFFFFu, need);
            if (need_mask) {
                unsigned long long base = 0;
                if (lane == static_cast<uint32_t>(__ffs(need_mask) - 1))
                    base = atomicAdd(&counters->queue_counters[kNextItem],
                                     static_cast<unsigned long long>(__popc(need_mask)));
                base = __shfl_sync(0xFFFFFFFFu, base, __ffs(need_mask) - 1);
                if (need) {
                    const unsigned long long item = base + __popc(need_mask & ((1u << lane) - 1u));
                    if (kMode == 1 && item < total_items) {
                        start_item<kKind>(cam, p, s, slot, static_cast<uint32_t>(item), fb.width, fb.height,
                                          frame_base, total_items);
                        push = true;
                    } else if (kMode == 2 && item < b.item_hi) {
                        start_item_batch<kKind>(S, b, s, slot, item);
                        push = true;
                    }
                }
            }
            queue_push(s.queue[out_queue], &counters->queue_counters[out_queue], slot, push);
        }
    }
}

// Per pixel of every request: fold its samples in frame order with DenoisePass's weights from a cleared
// frame buffer (frame k: cumulated k, weight k / (k + 1), CPURenderer.cpp:530-543), then tonemap.
__global__ void __launch_bounds__(256) k_b_resolve(BatchParams b, WavefrontState s) {
    const unsigned long long g = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (g >= b.total_pixels) return;
    uint32_t lo = 0, hi = b.num_reqs;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (b.reqs[mid].pixel_base <= g) {
            lo = mid;
        } else {
            hi = mid;
        }
    }
    const DevRequest &R = b.reqs[lo];
    const uint32_t pix = static_cast<uint32_t>(g - R.pixel_base);
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
    for (uint32_t k = 0; k < R.spp; ++k) {
        const float4 n = s.samples[R.item_base + static_cast<unsigned long long>(k) * R.npix + pix];
        const float f = static_cast<float>(k) / static_cast<float>(k + 1u);
        a = make_float4(n.x + (a.x - n.x) * f, n.y + (a.y - n.y) * f, n.z + (a.z - n.z) * f, n.w + (a.w - n.w) * f);
    }
    b.out_hdr[g] = a;
    const uint32_t i = pix % R.width, j = pix / R.width;
    ushort4 o;
    o.x = __half_as_ushort(__float2half_rn(aces_tonemap(a.x, R.cam.exposure)));
    o.y = __half_as_ushort(__float2half_rn(aces_tonemap(a.y, R.cam.exposure)));
    o.z = __half_as_ushort(__float2half_rn(aces_tonemap(a.z, R.cam.exposure)));
    o.w = __half_as_ushort(__float2half_rn(1.f));
    b.out_image[R.pixel_base + static_cast<unsigned long long>(R.height - 1 - j) * R.width + i] = o;
}

template <class T>
cudaError_t dmalloc(T *&p, size_t count) {
    if (fault_allocation()) return cudaErrorMemoryAllocation;
    return cudaMalloc(reinterpret_cast<void **>(&p), count * sizeof(T));
}

unsigned extend_blocks(int num_sms, uint32_t per_sm_override) {
    static int per_sm = 0;
    if (per_sm == 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_wf_extend<false>, 128, 0) != cudaSuccess ||
            per_sm <= 0)
            per_sm = 8;
    }
    const uint32_t n = per_sm_override ? std::min<uint32_t>(per_sm_override, static_cast<uint32_t>(per_sm))
                                       : static_cast<uint32_t>(per_sm);
    return static_cast<unsigned>(num_sms) * n;
}

// The shadow stage's persistent grid: SMs x its own occupancy (compiled for more blocks per SM than the
// closest-hit walk), capped like the extend grid by spk_tuning.extend_blocks_per_sm.
unsigned shadow_blocks(int num_sms, uint32_t per_sm_override) {
    static int per_sm = 0;
    if (per_sm == 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_wf_shadow<false>, 128, 0) != cudaSuccess ||
            per_sm <= 0)
            per_sm = 8;
    }
    const uint32_t n = per_sm_override ? std::min<uint32_t>(per_sm_override, static_cast<uint32_t>(per_sm))
                                       : static_cast<uint32_t>(per_sm);
    return static_cast<unsigned>(num_sms) * n;
}

// Kernel launches of one extend stage: the persistent form, and the packet forms `packet_forms` names (bit 0:
// one ray per lane, bit 1: two) where the stage may walk packets (a pass's first extend).
constexpr uint32_t extend_launches(uint32_t packet_forms) { return 1u + (packet_forms & 1u) + (packet_forms >> 1); }

// The packet forms a multi-frame pass of `frames` frames per pixel walks its primary rays with; the generate
// kernel sets the matching queue counters, which the kernels follow.
uint32_t pass_packet_forms(uint32_t frames, const WfTuning &tuning) {
    if (SPK_ITEM_ORDER != 1 || !tuning.packets || frames < kPacketMinSamples) return 0u;
    return frames >= kPacket2MinSamples ? 2u : 1u;
}

cudaError_t launch_extend(const DevScene &scene, const WavefrontState &s, int in, bool count, Counters *counters,
                          unsigned grid, cudaStream_t stream, LaunchEvents *ev, bool batch, uint32_t packet_forms) {
    unsigned long long *qc = counters->queue_counters;
    static_assert(kPacketCursor == kCursor + 1 && kPacket2Cursor == kCursor + 2, "one reset for the cursors");
    cudaError_t e = cudaMemsetAsync(qc + kCursor, 0, 3 * sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    if (ev) ev->before(stream);
    if (batch) {
        if (packet_forms & 2u)
            (count ? k_wf_extend<true, true, 2> : k_wf_extend<false, true, 2>)<<<grid, 128, 0, stream>>>(scene, s, in,
                                                                                                         counters);
        if (packet_forms & 1u)
            (count ? k_wf_extend<true, true, 1> : k_wf_extend<false, true, 1>)<<<grid, 128, 0, stream>>>(scene, s, in,
                                                                                                         counters);
        (count ? k_wf_extend<true, true> : k_wf_extend<false, true>)<<<grid, 128, 0, stream>>>(scene, s, in, counters);
    } else {
        if (packet_forms & 2u)
            (count ? k_wf_extend<true, false, 2> : k_wf_extend<false, false, 2>)<<<grid, 128, 0, stream>>>(
                scene, s, in, counters);
        if (packet_forms & 1u)
            (count ? k_wf_extend<true, false, 1> : k_wf_extend<false, false, 1>)<<<grid, 128, 0, stream>>>(
                scene, s, in, counters);
        (count ? k_wf_extend<true, false> : k_wf_extend<false, false>)<<<grid, 128, 0, stream>>>(scene, s, in,
                                                                                                 counters);
    }
    if (ev) ev->after(stream);
    return cudaSuccess;
}

int nee_mode(uint32_t enable_nee, const WfTuning &tuning) {
    return !enable_nee ? kNeeOff : (tuning.shadow_stage ? kNeeDeferred : kNeeInline);
}

using WfShadeFn = void (*)(DevScene, FrameBuffers, RenderParams, WavefrontState, int, uint32_t, Counters *);
WfShadeFn pick_wf_shade(uint32_t rng, int nee) {
    if (rng == 0) return nee == kNeeOff ? k_wf_shade<0, kNeeOff> : nee == kNeeInline ? k_wf_shade<0, kNeeInline> : k_wf_shade<0, kNeeDeferred>;
    return nee == kNeeOff ? k_wf_shade<1, kNeeOff> : nee == kNeeInline ? k_wf_shade<1, kNeeInline> : k_wf_shade<1, kNeeDeferred>;
}

using MfShadeFn = void (*)(DevScene, DevCamera, FrameBuffers, RenderParams, WavefrontState, int, uint32_t, uint32_t,
                           Counters *);
MfShadeFn pick_mf_shade(uint32_t rng, int nee) {
    if (rng == 0) return nee == kNeeOff ? k_mf_shade<0, kNeeOff> : nee == kNeeInline ? k_mf_shade<0, kNeeInline> : k_mf_shade<0, kNeeDeferred>;
    return nee == kNeeOff ? k_mf_shade<1, kNeeOff> : nee == kNeeInline ? k_mf_shade<1, kNeeInline> : k_mf_shade<1, kNeeDeferred>;
}

using BShadeFn = void (*)(DevScene, BatchParams, WavefrontState, int, Counters *);
BShadeFn pick_b_shade(uint32_t rng, int nee) {
    if (rng == 0) return nee == kNeeOff ? k_b_shade<0, kNeeOff> : nee == kNeeInline ? k_b_shade<0, kNeeInline> : k_b_shade<0, kNeeDeferred>;
    return nee == kNeeOff ? k_b_shade<1, kNeeOff> : nee == kNeeInline ? k_b_shade<1, kNeeInline> : k_b_shade<1, kNeeDeferred>;
}

// The shadow stage of one iteration (deferred NEE): the occlusion walk, then the accumulation of mode
// kMode (0 frame by frame, 1 multi-frame, 2 batch). Two launches.
template <int kMode>
void enqueue_shadow_stage(const DevScene &scene, const DevCamera &cam, const FrameBuffers &fbuf, const RenderParams &p,
                          const BatchParams &b, const WavefrontState &s, uint32_t rng, int out_queue,
                          uint32_t frame_base, uint32_t total_items, Counters *counters, unsigned walk_grid,
                          unsigned shade_grid, cudaStream_t stream) {
    k_wf_shadow<kMode == 2><<<walk_grid, 128, 0, stream>>>(scene, s, counters);
    auto *acc = rng == 0 ? k_nee_accumulate<0, kMode> : k_nee_accumulate<1, kMode>;
    acc<<<shade_grid, 128, 0, stream>>>(cam, fbuf, p, scene, b, s, out_queue, frame_base, total_items, counters);
}

// Resets the shadow stage's counters (queued rays, vertices, walk cursor) before a shade stage.
cudaError_t reset_shadow_counters(Counters *counters, cudaStream_t stream) {
    return cudaMemsetAsync(counters->queue_counters + kShadowLen, 0, 3 * sizeof(unsigned long long), stream);
}

}  // namespace

cudaError_t wavefront_alloc_nee(WavefrontState &s) {
    if (s.nee_capacity >= s.capacity && s.shadow_o) return cudaSuccess;
    void *ptrs[] = {s.shadow_o, s.shadow_d, s.nee_contrib, s.shadow_queue, s.nee_list};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    s.shadow_o = s.shadow_d = s.nee_contrib = nullptr;
    s.shadow_queue = s.nee_list = nullptr;
    s.nee_capacity = 0;
    const size_t n = s.capacity;
    cudaError_t e;
    if ((e = dmalloc(s.shadow_o, 2 * n)) != cudaSuccess || (e = dmalloc(s.shadow_d, 2 * n)) != cudaSuccess ||
        (e = dmalloc(s.nee_contrib, 2 * n)) != cudaSuccess || (e = dmalloc(s.shadow_queue, 2 * n)) != cudaSuccess ||
        (e = dmalloc(s.nee_list, n)) != cudaSuccess) {
        void *got[] = {s.shadow_o, s.shadow_d, s.nee_contrib, s.shadow_queue, s.nee_list};
        for (void *p : got)
            if (p) cudaFree(p);
        s.shadow_o = s.shadow_d = s.nee_contrib = nullptr;
        s.shadow_queue = s.nee_list = nullptr;
        return e;
    }
    s.nee_capacity = s.capacity;
    return cudaSuccess;
}

cudaError_t wavefront_alloc(WavefrontState &s, uint32_t capacity) {
    wavefront_free(s);
    cudaError_t e;
    if ((e = dmalloc(s.ray_a, capacity)) != cudaSuccess || (e = dmalloc(s.ray_b, capacity)) != cudaSuccess ||
        (e = dmalloc(s.thr, capacity)) != cudaSuccess || (e = dmalloc(s.color, capacity)) != cudaSuccess ||
        (e = dmalloc(s.rng, 2 * static_cast<size_t>(capacity))) != cudaSuccess ||
        (e = dmalloc(s.hit, capacity)) != cudaSuccess || (e = dmalloc(s.hit_face, capacity)) != cudaSuccess ||
        (e = dmalloc(s.queue[0], capacity)) != cudaSuccess || (e = dmalloc(s.queue[1], capacity)) != cudaSuccess ||
        (e = dmalloc(s.sort_keys, capacity)) != cudaSuccess || (e = dmalloc(s.slot_state, capacity)) != cudaSuccess ||
        (e = dmalloc(s.slot_item, capacity)) != cudaSuccess || (e = dmalloc(s.prev_pdf, capacity)) != cudaSuccess ||
        (e = dmalloc(s.sort_hist, 2 * kRaySortBuckets)) != cudaSuccess ||
        (e = dmalloc(s.sort_keys2, capacity)) != cudaSuccess ||
        (e = dmalloc(s.slot_req, capacity)) != cudaSuccess || (e = dmalloc(s.slot_root, capacity)) != cudaSuccess ||
        (e = cudaMemset(s.sort_hist, 0, 2 * kRaySortBuckets * sizeof(uint32_t))) != cudaSuccess ||
        (e = cudaHostAlloc(reinterpret_cast<void **>(&s.host_len), sizeof(unsigned long long), cudaHostAllocDefault)) !=
            cudaSuccess) {
        wavefront_free(s);
        return e;
    }
    s.capacity = capacity;
    return cudaSuccess;
}

void wavefront_free(WavefrontState &s) {
    void *ptrs[] = {s.ray_a,      s.ray_b,     s.thr,     s.color,        s.rng,        s.hit,
                    s.hit_face,   s.queue[0],  s.queue[1], s.sort_keys,   s.slot_state, s.slot_item,
                    s.samples,    s.frame_weight, s.frame_seed, s.prev_pdf, s.sort_hist, s.slot_req,
                    s.slot_root,  s.sort_keys2, s.shadow_o, s.shadow_d, s.nee_contrib, s.shadow_queue,
                    s.nee_list,   s.sample_normals};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (s.host_len) cudaFreeHost(s.host_len);
    s = WavefrontState{};
}

void chunk_graph_free(ChunkGraph &g) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    for (cudaEvent_t ev : g.events)
        if (ev) cudaEventDestroy(ev);
    const bool enabled = g.enabled;
    g = ChunkGraph{};
    g.enabled = enabled;
}

cudaError_t launch_render_wavefront(const DevScene &scene, const DevCamera &cam, const FrameBuffers &fbuf,
                                    const RenderParams &p, bool count, Counters *counters, WavefrontState &s,
                                    int num_sms, cudaStream_t stream, uint32_t *launches, LaunchEvents *ev,
                                    const WfTuning &tuning) {
    uint32_t nl = 0;
    const uint32_t npix = fbuf.width * fbuf.height;
    if (s.capacity < npix) return cudaErrorInvalidValue;
    if ((tuning.ray_sort || tuning.material_sort) && !sort_buffers_ok(s)) return cudaErrorInvalidValue;
    cudaError_t e;
    const int nee = nee_mode(p.enable_nee, tuning);
    if (nee == kNeeDeferred && (e = wavefront_alloc_nee(s)) != cudaSuccess) return e;
    unsigned long long *qc = counters->queue_counters;
    if ((e = cudaMemsetAsync(qc, 0, sizeof(counters->queue_counters), stream)) != cudaSuccess) return e;
    const dim3 ggrid((fbuf.width + 15) / 16, (fbuf.height + 7) / 8);
    if (p.rng == 0) {
        k_wf_generate<0><<<ggrid, 128, 0, stream>>>(cam, fbuf, p, s, counters);
    } else {
        k_wf_generate<1><<<ggrid, 128, 0, stream>>>(cam, fbuf, p, s, counters);
    }
    ++nl;
    const unsigned shade_blocks = static_cast<unsigned>(num_sms) * tuning.shade_blocks_per_sm;
    const unsigned extend_grid = extend_blocks(num_sms, tuning.extend_blocks_per_sm);
    const unsigned shadow_grid = shadow_blocks(num_sms, tuning.extend_blocks_per_sm);
    for (uint32_t b = 0; b < p.bounce; ++b) {
        const int in = static_cast<int>(b & 1u), out = in ^ 1;
        if ((e = cudaMemsetAsync(qc + out, 0, sizeof(unsigned long long), stream)) != cudaSuccess) return e;
        WavefrontState se = s;
        if (tuning.ray_sort) {
            se = enqueue_ray_sort(scene, s, in, counters, num_sms, stream);
            nl += 3;
        }
        if ((e = launch_extend(scene, se, in, count, counters, extend_grid, stream, ev, false, 0u)) != cudaSuccess)
            return e;
        nl += extend_launches(0u);
        WavefrontState ss = se;
        if (tuning.material_sort) {
            ss = enqueue_material_sort(scene, se, in, counters, num_sms, stream);
            nl += 3;
        }
        if (nee == kNeeDeferred && (e = reset_shadow_counters(counters, stream)) != cudaSuccess) return e;
        pick_wf_shade(p.rng, nee)<<<shade_blocks, 128, 0, stream>>>(scene, fbuf, p, ss, in, b, counters);
        ++nl;
        if (nee == kNeeDeferred) {
            enqueue_shadow_stage<0>(scene, cam, fbuf, p, BatchParams{}, ss, p.rng, out, 0u, 0u, counters, shadow_grid,
                                    shade_blocks, stream);
            nl += 2;
        }
    }
    k_wf_finish<<<(npix + 255) / 256, 256, 0, stream>>>(fbuf, s);
    ++nl;
    if (launches) *launches = nl;
    return cudaGetLastError();
}

namespace {
thread_local const char *t_site = "";
}

const char *wavefront_error_site() { return t_site; }

cudaError_t launch_render_multiframe(const DevScene &scene, const DevCamera &cam, const FrameBuffers &fbuf,
                                     const RenderParams &p, uint32_t num_frames, const float *weights,
                                     const uint32_t *seeds, bool count, Counters *counters, WavefrontState &s,
                                     int num_sms, cudaStream_t stream, uint32_t *launches, LaunchEvents *ev,
                                     const WfTuning &tuning, ChunkGraph *graph) {
    uint32_t nl = 0;
    const uint32_t npix = fbuf.width * fbuf.height;
    t_site = "set-up";
    if (s.capacity < npix || num_frames == 0 || p.bounce == 0) return cudaErrorInvalidValue;
    if ((tuning.ray_sort || tuning.material_sort) && !sort_buffers_ok(s)) return cudaErrorInvalidValue;
    cudaError_t e;
    const int nee = nee_mode(p.enable_nee, tuning);
    if (nee == kNeeDeferred && (e = wavefront_alloc_nee(s)) != cudaSuccess) return e;
    if (s.frame_capacity < num_frames) {
        if (s.frame_weight) cudaFree(s.frame_weight);
        if (s.frame_seed) cudaFree(s.frame_seed);
        s.frame_weight = nullptr;
        s.frame_seed = nullptr;
        s.frame_capacity = 0;
        if ((e = dmalloc(s.frame_weight, num_frames)) != cudaSuccess) return e;
        if ((e = dmalloc(s.frame_seed, num_frames)) != cudaSuccess) return e;
        s.frame_capacity = num_frames;
    }
    const uint32_t pass_frames = std::min(num_frames, kFramesPerPass);
    const size_t need = static_cast<size_t>(pass_frames) * npix;
    if (s.sample_capacity < need) {
        if (s.samples) cudaFree(s.samples);
        s.samples = nullptr;
        s.sample_capacity = 0;
        if ((e = dmalloc(s.samples, need)) != cudaSuccess) return e;
        s.sample_capacity = need;
    }
    if (p.spatial_denoise && s.normal_capacity < need) {
        if (s.sample_normals) cudaFree(s.sample_normals);
        s.sample_normals = nullptr;
        s.normal_capacity = 0;
        if ((e = dmalloc(s.sample_normals, need)) != cudaSuccess) return e;
        s.normal_capacity = need;
    }
    if ((e = cudaMemcpyAsync(s.frame_weight, weights, num_frames * sizeof(float), cudaMemcpyHostToDevice, stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(s.frame_seed, seeds, num_frames * sizeof(uint32_t), cudaMemcpyHostToDevice, stream)) !=
            cudaSuccess)
        return e;
    unsigned long long *qc = counters->queue_counters;
    const unsigned shade_blocks = static_cast<unsigned>(num_sms) * tuning.shade_blocks_per_sm;
    const unsigned extend_grid = extend_blocks(num_sms, tuning.extend_blocks_per_sm);
    const unsigned shadow_grid = shadow_blocks(num_sms, tuning.extend_blocks_per_sm);
    constexpr uint32_t kChunk = kChunkIterations;
    static_assert(kChunk % 2 == 0, "a chunk must keep the queue parity, so one graph serves every chunk");
    for (uint32_t f0 = 0; f0 < num_frames; f0 += kFramesPerPass) {
        const uint32_t frames = std::min(kFramesPerPass, num_frames - f0);
        const uint32_t packet_forms = pass_packet_forms(frames, tuning);
        const uint32_t total_items = frames * npix;
        // Paths in flight: slots_per_pixel x pixels, within the state's capacity and the pass's items.
        const uint64_t want = static_cast<uint64_t>(npix) * std::max(1u, tuning.slots_per_pixel);
        const uint32_t initial = static_cast<uint32_t>(
            std::min<uint64_t>({want, static_cast<uint64_t>(s.capacity), static_cast<uint64_t>(total_items)}));
        if ((e = cudaMemsetAsync(qc, 0, sizeof(counters->queue_counters), stream)) != cudaSuccess) return e;
        if (p.rng == 0) {
            k_mf_generate<0><<<(initial + 127) / 128, 128, 0, stream>>>(cam, fbuf, p, s, f0, initial, total_items,
                                                                     tuning.packets, counters);
        } else {
            k_mf_generate<1><<<(initial + 127) / 128, 128, 0, stream>>>(cam, fbuf, p, s, f0, initial, total_items,
                                                                     tuning.packets, counters);
        }
        ++nl;
        // One chunk: kChunk iterations of (reset the output queue, extend, shade).
        auto enqueue_chunk = [&](LaunchEvents *chunk_ev) -> cudaError_t {
            cudaError_t ce;
            for (uint32_t c = 0; c < kChunk; ++c) {
                const int in = static_cast<int>(c & 1u), out = in ^ 1;
                if ((ce = cudaMemsetAsync(qc + out, 0, sizeof(unsigned long long), stream)) != cudaSuccess) return ce;
                const WavefrontState se =
                    tuning.ray_sort ? enqueue_ray_sort(scene, s, in, counters, num_sms, stream) : s;
                if ((ce = launch_extend(scene, se, in, count, counters, extend_grid, stream, chunk_ev, false,
                                        c == 0 ? packet_forms : 0u)) != cudaSuccess)
                    return ce;
                const WavefrontState ss =
                    tuning.material_sort ? enqueue_material_sort(scene, se, in, counters, num_sms, stream) : se;
                if (nee == kNeeDeferred && (ce = reset_shadow_counters(counters, stream)) != cudaSuccess) return ce;
                pick_mf_shade(p.rng, nee)<<<shade_blocks, 128, 0, stream>>>(scene, cam, fbuf, p, ss, in, f0,
                                                                            total_items, counters);
                if (nee == kNeeDeferred)
                    enqueue_shadow_stage<1>(scene, cam, fbuf, p, BatchParams{}, ss, p.rng, out, f0, total_items,
                                            counters, shadow_grid, shade_blocks, stream);
            }
            return cudaGetLastError();
        };
        bool use_graph = false;
        LaunchEvents graph_ev{};
        if (graph && graph->enabled) {
            // The graph is keyed by every value its launches take; a new key re-captures it and updates
            // the executable graph in place when the topology allows.
            struct Key {
                DevScene scene;
                DevCamera cam;
                FrameBuffers fbuf;
                RenderParams p;
                WavefrontState s;
                uint32_t f0, total_items, count, num_sms;
                Counters *counters;
                cudaStream_t stream;
                unsigned extend_grid, shade_grid, material_sort, ray_sort, nee_mode, packet_forms;
            } key;
            std::memset(static_cast<void *>(&key), 0, sizeof(key));  // padding too: the key is compared bytewise
            key.scene = scene;
            key.cam = cam;
            key.fbuf = fbuf;
            key.p = p;
            key.s = s;
            key.f0 = f0;
            key.total_items = total_items;
            key.count = count;
            key.num_sms = static_cast<uint32_t>(num_sms);
            key.counters = counters;
            key.stream = stream;
            key.extend_grid = extend_grid;
            key.shade_grid = shade_blocks;
            key.material_sort = tuning.material_sort;
            key.ray_sort = tuning.ray_sort;
            key.nee_mode = static_cast<unsigned>(nee);
            key.packet_forms = packet_forms;
            const auto *kb = reinterpret_cast<const unsigned char *>(&key);
            graph_ev.pairs = graph->events;
            graph_ev.capacity = static_cast<int>(kChunk);
            graph_ev.record_flags = cudaEventRecordExternal;
            if (!graph->events[0]) {
                for (cudaEvent_t &g_ev : graph->events)
                    if ((e = cudaEventCreate(&g_ev)) != cudaSuccess) return e;
            }
            use_graph = true;
            if (!graph->exec || graph->key.size() != sizeof(key) || std::memcmp(graph->key.data(), kb, sizeof(key))) {
                cudaGraph_t g = nullptr;
                t_site = "graph capture";
                if ((e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
                const cudaError_t enq = enqueue_chunk(ev ? &graph_ev : nullptr);
                if ((e = cudaStreamEndCapture(stream, &g)) != cudaSuccess) return e;
                if (enq != cudaSuccess) {
                    cudaGraphDestroy(g);
                    return enq;
                }
                bool updated = false;
                if (graph->exec) {
                    cudaGraphExecUpdateResultInfo info;
                    updated = cudaGraphExecUpdate(graph->exec, g, &info) == cudaSuccess;
                    if (!updated) {
                        cudaGetLastError();
                        cudaGraphExecDestroy(graph->exec);
                        graph->exec = nullptr;
                    }
                }
                t_site = "graph instantiate";
                if (!updated) e = cudaGraphInstantiate(&graph->exec, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) {
                    graph->exec = nullptr;
                    return e;
                }
                graph->key.assign(kb, kb + sizeof(key));
                graph->timed = ev != nullptr;
                ++graph->captures;
            }
            if (graph->timed != (ev != nullptr)) {
                graph->key.clear();  // timing events differ: force a re-capture next time
                use_graph = false;
            }
        }
        // Each iteration advances every live slot by one segment and no item is started twice, so the
        // pass ends within frames * bounce iterations; the queue length is read back every kChunk.
        const uint64_t max_iters = static_cast<uint64_t>(frames) * p.bounce + kChunk;
        uint64_t iter = 0;
        for (;;) {
            t_site = use_graph ? "graph launch" : "chunk launch";
            if (use_graph) {
                if ((e = cudaGraphLaunch(graph->exec, stream)) != cudaSuccess) return e;
                ++graph->replays;
            } else if ((e = enqueue_chunk(ev)) != cudaSuccess) {
                return e;
            }
            iter += kChunk;
            nl += (2u + (tuning.material_sort ? 3u : 0u) + (tuning.ray_sort ? 3u : 0u) +
                   (nee == kNeeDeferred ? 2u : 0u)) * kChunk +
                  extend_launches(packet_forms) - 1u;
            if ((e = cudaMemcpyAsync(s.host_len, qc, sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream)) !=
                cudaSuccess)
                return e;
            if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;
            t_site = "graph timing events";
            if (use_graph && ev) {
                for (uint32_t c = 0; c < kChunk; ++c) {
                    float x = 0.f;
                    if ((e = cudaEventElapsedTime(&x, graph->events[2 * c], graph->events[2 * c + 1])) != cudaSuccess)
                        return e;
                    ev->graph_ms += x;
                }
                ev->graph_launches += static_cast<int>(kChunk);
            }
            if (*s.host_len == 0) break;
            if (iter > max_iters) return cudaErrorLaunchFailure;  // cannot happen: every slot makes progress
        }
        t_site = "resolve";
        k_mf_resolve<<<(npix + 255) / 256, 256, 0, stream>>>(fbuf, s, f0, frames, cam.exposure, p.spatial_denoise);
        ++nl;
    }
    if (launches) *launches = nl;
    return cudaGetLastError();
}

cudaError_t launch_render_batch(const DevScene &scene, const BatchParams &b, const std::vector<BatchGroup> &groups,
                                bool count, Counters *counters, WavefrontState &s, int num_sms, cudaStream_t stream,
                                uint32_t *launches, LaunchEvents *ev, const WfTuning &tuning) {
    if (b.num_reqs == 0 || b.total_items == 0 || s.capacity == 0 || s.sample_capacity < b.total_items ||
        groups.empty())
        return cudaErrorInvalidValue;
    if ((tuning.ray_sort || tuning.material_sort) && !sort_buffers_ok(s)) return cudaErrorInvalidValue;
    uint32_t nl = 0;
    cudaError_t e;
    const int nee = nee_mode(b.enable_nee, tuning);
    if (nee == kNeeDeferred && (e = wavefront_alloc_nee(s)) != cudaSuccess) return e;
    unsigned long long *qc = counters->queue_counters;
    const unsigned shade_blocks = static_cast<unsigned>(num_sms) * tuning.shade_blocks_per_sm;
    const unsigned extend_grid = extend_blocks(num_sms, tuning.extend_blocks_per_sm);
    const unsigned shadow_grid = shadow_blocks(num_sms, tuning.extend_blocks_per_sm);
    const unsigned long long want = tuning.batch_slots ? tuning.batch_slots : s.capacity;
    auto *shade = pick_b_shade(b.rng, nee);
    constexpr uint32_t kChunk = kChunkIterations;
    for (const BatchGroup &grp : groups) {
        if (grp.item_hi <= grp.item_lo || grp.item_hi > b.total_items) return cudaErrorInvalidValue;
        BatchParams bg = b;
        bg.item_lo = grp.item_lo;
        bg.item_hi = grp.item_hi;
        bg.packet_items = grp.packet_items;
        bg.packet2_items = grp.packet2_items;
        const uint32_t first =
            static_cast<uint32_t>(std::min<unsigned long long>({want, s.capacity, grp.item_hi - grp.item_lo}));
        if ((e = cudaMemsetAsync(qc, 0, sizeof(counters->queue_counters), stream)) != cudaSuccess) return e;
        if (b.rng == 0) {
            k_b_generate<0><<<(first + 127) / 128, 128, 0, stream>>>(scene, bg, s, first, counters);
        } else {
            k_b_generate<1><<<(first + 127) / 128, 128, 0, stream>>>(scene, bg, s, first, counters);
        }
        ++nl;
        // A slot finishes an item within its request's bounce limit and no item starts twice, so
        // items * 64 iterations (bounce < 64 in practice) is a loose guard against a runaway loop.
        const unsigned long long max_iters = (grp.item_hi - grp.item_lo) * 64ull + kChunk;
        unsigned long long iter = 0;
        // the group's first extend: two rays per lane for its first packet2_items entries, one for the rest
        const uint32_t packet_forms =
            SPK_ITEM_ORDER == 1 ? (grp.packet2_items ? 2u : 0u) | (grp.packet_items > grp.packet2_items ? 1u : 0u)
                                : 0u;
        for (;;) {
            for (uint32_t c = 0; c < kChunk; ++c) {
                const int in = static_cast<int>(c & 1u), out = in ^ 1;
                if ((e = cudaMemsetAsync(qc + out, 0, sizeof(unsigned long long), stream)) != cudaSuccess) return e;
                const WavefrontState se =
                    tuning.ray_sort ? enqueue_ray_sort(scene, s, in, counters, num_sms, stream) : s;
                if ((e = launch_extend(scene, se, in, count, counters, extend_grid, stream, ev, true,
                                       c == 0 ? packet_forms : 0u)) != cudaSuccess)
                    return e;
                const WavefrontState ss =
                    tuning.material_sort ? enqueue_material_sort(scene, se, in, counters, num_sms, stream) : se;
                if (nee == kNeeDeferred && (e = reset_shadow_counters(counters, stream)) != cudaSuccess) return e;
                shade<<<shade_blocks, 128, 0, stream>>>(scene, bg, ss, in, counters);
                if (nee == kNeeDeferred)
                    enqueue_shadow_stage<2>(scene, DevCamera{}, FrameBuffers{}, RenderParams{}, bg, ss, b.rng, out, 0u,
                                            0u, counters, shadow_grid, shade_blocks, stream);
            }
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            iter += kChunk;
            nl += (2u + (tuning.material_sort ? 3u : 0u) + (tuning.ray_sort ? 3u : 0u) +
                   (nee == kNeeDeferred ? 2u : 0u)) * kChunk +
                  extend_launches(packet_forms) - 1u;
            if ((e = cudaMemcpyAsync(s.host_len, qc, sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream)) !=
                cudaSuccess)
                return e;
            if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;
            if (*s.host_len == 0) break;
            if (iter > max_iters) return cudaErrorLaunchFailure;
        }
    }
    const unsigned blocks = static_cast<unsigned>((b.total_pixels + 255) / 256);
    k_b_resolve<<<blocks, 256, 0, stream>>>(b, s);
    ++nl;
    if (launches) *launches = nl;
    return cudaGetLastError();
}

}  // namespace spk
