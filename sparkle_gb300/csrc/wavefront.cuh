// wavefront.cuh -- path state and launchers of the wavefront schedule of BasePass.
//
// The per-pixel path loop of SamplePixel (CPURenderer.cpp:240-396) is split into stage kernels that run
// over queues of live paths: generate (camera rays + RNG), then per bounce extend (closest hit) and shade
// (emission / sky / BSDF sample / Russian roulette, compacting survivors into the next queue with
// warp-aggregated atomics) and, with next-event estimation, shadow (a persistent occlusion walk of the
// light and sky rays shade queued) and accumulate (their radiance added in the one-kernel order), then
// finish (G-buffer write). Queue lengths live in device memory, so one
// frame is a fixed launch sequence with no host round trip. Each path runs the same arithmetic and draws
// the same random numbers in the same order as the one-kernel schedule, so both write identical G-buffers.
#pragma once

#include <vector>

#include "kernels.cuh"

namespace spk {

struct WavefrontState {
    uint32_t capacity = 0;
    float4 *ray_a = nullptr;    // next ray: origin xyz, direction x
    float2 *ray_b = nullptr;    // next ray: direction y, z
    float4 *thr = nullptr;      // throughput xyz
    float4 *color = nullptr;    // radiance xyz, w = valid flag
    uint4 *rng = nullptr;       // 2 x uint4 per path (xoshiro256** needs 32 B)
    float4 *hit = nullptr;      // t, u, v, inst bits
    uint32_t *hit_face = nullptr;
    uint32_t *queue[2] = {nullptr, nullptr};  // path indices
    uint32_t *sort_keys = nullptr;            // material sort: the shade queue grouped by material class
    uint32_t *sort_hist = nullptr;            // sorts: 2 x kRaySortBuckets counters (histogram, cursors)
    uint32_t *sort_keys2 = nullptr;           // ray sort: the extend queue ordered by ray key
    float *prev_pdf = nullptr;                // NEE: cosine pdf of the continuation after a light-sampling vertex
    uint32_t *slot_state = nullptr;           // multi-frame mode: bounce of the slot's path
    uint32_t *slot_item = nullptr;            // multi-frame mode: sample item (frame * pixels + pixel) of the slot
    uint32_t *slot_req = nullptr;             // batch mode: request of the slot's path
    uint32_t *slot_root = nullptr;            // batch mode: TLAS root of the slot's scene
    float4 *samples = nullptr;                // multi-frame mode: clamped result of each (frame, pixel) sample
    size_t sample_capacity = 0;               // float4 entries of `samples`
    float4 *sample_normals = nullptr;         // multi-frame mode with the spatial fill: first-hit normal per sample
    size_t normal_capacity = 0;               // float4 entries of `sample_normals`
    // multi-frame mode: per-frame constants, frame k of the call
    float *frame_weight = nullptr;      // DenoisePass moving-average weight of frame k
    uint32_t *frame_seed = nullptr;     // dispatched sample count at frame k (per-pixel seed base)
    uint32_t frame_capacity = 0;
    unsigned long long *host_len = nullptr;  // pinned: queue length read back between iteration chunks
    // Shadow stage of next-event estimation (allocated on first use, `nee_capacity` slots): the two
    // occlusion rays of a light-sampling vertex (k = 0 light, 1 sky) and the radiance each adds unoccluded.
    float4 *shadow_o = nullptr;        // 2 per slot: origin xyz, w = tmax
    float4 *shadow_d = nullptr;        // 2 per slot: direction xyz
    float4 *nee_contrib = nullptr;     // 2 per slot: radiance xyz; w = 0 no ray, 1 queued, 2 unoccluded
    uint32_t *shadow_queue = nullptr;  // occlusion rays of the iteration, entry 2 * slot + k
    uint32_t *nee_list = nullptr;      // light-sampling vertices of the iteration, slot | (path ended) << 31
    uint32_t nee_capacity = 0;
};

// Material-sort classes: material ids 0..kSortBuckets-3 each, larger ids share one class, misses the last.
constexpr uint32_t kSortBuckets = 64;
// Ray-sort keys: 3-bit Morton cell per axis of the origin in the scene bounds x direction octant.
constexpr uint32_t kRaySortBuckets = 4096;

// Frames per multi-frame pass: bounds the per-sample result buffer to kFramesPerPass * pixels * 16 B.
constexpr uint32_t kFramesPerPass = 64;
// Most path slots a multi-frame schedule allocates (2^27 slots: about 20 GB of path state; a 1080p pass of
// 64 frames has 132.7 M sample items).
constexpr uint64_t kMaxPathSlots = 1ull << 27;

cudaError_t wavefront_alloc(WavefrontState &s, uint32_t capacity);
void wavefront_free(WavefrontState &s);

// Launch shapes and schedule options of the wavefront (spk_tuning); none changes a result.
struct WfTuning {
    uint32_t extend_blocks_per_sm = 0;  // 0 = occupancy maximum of the traversal kernel
    uint32_t shade_blocks_per_sm = 8;
    bool material_sort = false;
    bool ray_sort = false;
    uint32_t slots_per_pixel = 1;  // multi-frame schedule: path slots per pixel (bounded by the state's capacity)
    uint32_t batch_slots = 0;      // batch schedule: paths in flight (0 = the state's capacity)
    bool shadow_stage = true;      // NEE occlusion rays walked by their own persistent stage (false: inline in shade)
    uint32_t packets = 1;          // 1: primary rays (the first extend of a pass or frame) walked in warp packets
};

// Allocates the shadow-stage buffers of `s` for its capacity (no-op when they are large enough).
cudaError_t wavefront_alloc_nee(WavefrontState &s);

// Host-side CUDA graph of one chunk of the multi-frame loop (kChunkIterations extend + shade iterations
// with their counter resets), captured once and replayed while the kernel parameters stay the same.
constexpr uint32_t kChunkIterations = 8;
struct ChunkGraph {
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t events[2 * kChunkIterations] = {};  // start/stop of each extend launch inside the graph
    std::vector<unsigned char> key;                 // kernel parameters the graph was captured with
    bool enabled = true;
    bool timed = false;  // captured with the timing events
    uint32_t replays = 0, captures = 0;
};
void chunk_graph_free(ChunkGraph &g);

// All `num_frames` frames of a call in one wavefront with path regeneration. Slots pull (frame, pixel) sample items
// from a global counter in frame-major order; a slot whose path ends stores the sample's clamped result
// and starts the next item, so every iteration keeps about one frame of paths in flight and only the
// last few paths form a tail. A resolve pass then folds each pixel's samples into the frame buffer in
// frame order with each frame's weight (CPURenderer.cpp:530-543), so the frame buffer is bit-identical
// to rendering the frames one by one. With the spatial DenoisePass on, every sample also keeps its first-hit
// normal and the resolve applies the fill to each frame's samples before folding them (the fill reads only
// the same frame's samples, so pixels still do not interact across frames). `weights[k]` / `seeds[k]` are
// frame k's moving-average weight and seed base. Ends with the tonemap of the final frame buffer.
cudaError_t launch_render_multiframe(const DevScene &scene, const DevCamera &cam, const FrameBuffers &fbuf,
                                     const RenderParams &p, uint32_t num_frames, const float *weights,
                                     const uint32_t *seeds, bool count, Counters *counters, WavefrontState &s,
                                     int num_sms, cudaStream_t stream, uint32_t *launches, LaunchEvents *ev,
                                     const WfTuning &tuning, ChunkGraph *graph);

// One request of a batch (spk_request) as the batch kernels read it.
// Fewest samples of a pixel next to each other in the sample-item order for its primary rays to be walked
// in packets: below it a 32-ray packet spans more than 4 pixels, whose rays share too few nodes to pay
// reliably (one sample per pixel: primary rays 22% slower than walked one by one; four: 10% faster at
// 1920x1080 but slower on smaller images, where a pixel covers more of the scene).
#ifndef SPK_PACKET_MIN_SAMPLES
#define SPK_PACKET_MIN_SAMPLES 8
#endif
constexpr uint32_t kPacketMinSamples = SPK_PACKET_MIN_SAMPLES;
// Fewest samples per pixel in a multi-frame pass for packets of two rays per lane (64 consecutive samples:
// one pixel's at 64 frames, two pixels' at 32), which share each node visit between twice the rays (at 32
// frames the primary rays took 11.8 ms less than walked one by one, against 9.7 ms with one ray per lane).
#ifndef SPK_PACKET2_MIN_SAMPLES
#define SPK_PACKET2_MIN_SAMPLES 32
#endif
constexpr uint32_t kPacket2MinSamples = SPK_PACKET2_MIN_SAMPLES;

struct DevRequest {
    DevCamera cam;
    uint32_t scene, width, height, npix;
    uint32_t spp, bounce, seed;
    uint32_t queue_base;            // first-pass queue position of the request's first item (see BatchParams)
    unsigned long long item_base;   // first global sample item: items of request r are frame-major
    unsigned long long pixel_base;  // first pixel of the request in the batch output images
};

struct BatchParams {
    const DevRequest *reqs;
    uint32_t num_reqs;
    uint32_t rng, enable_nee;
    unsigned long long total_items;
    unsigned long long total_pixels;
    // The sample items of one group of whole requests, [item_lo, item_hi), run as one wavefront (set per group
    // by launch_render_batch from BatchGroup). Its first pass queues them request by request: those of requests
    // with spp >= kPacket2MinSamples first, walked in packets of two rays per lane (packet2_items entries), then
    // those with spp >= kPacketMinSamples, in packets of one ray per lane (up to packet_items entries), then the
    // rest (DevRequest::queue_base, relative to the group).
    unsigned long long item_lo, item_hi;
    unsigned long long packet_items, packet2_items;
    float4 *out_hdr;     // accumulated frame buffers of all requests, request after request
    ushort4 *out_image;  // tonemapped images (top row first per request)
};

// A group of consecutive whole requests rendered as one wavefront: items [item_lo, item_hi), the first
// packet2_items / packet_items of its first pass walked in packets (BatchParams).
struct BatchGroup {
    unsigned long long item_lo, item_hi, packet_items, packet2_items;
};

// All sample items of a batch, group after group: each group one regenerating wavefront over `s` (capacity =
// path slots; a group that fits starts all its items at once), then the ordered per-pixel resolve and
// tonemap into the batch outputs. `s.samples` must hold total_items entries.
cudaError_t launch_render_batch(const DevScene &scene, const BatchParams &b, const std::vector<BatchGroup> &groups,
                                bool count, Counters *counters, WavefrontState &s, int num_sms, cudaStream_t stream,
                                uint32_t *launches, LaunchEvents *ev, const WfTuning &tuning);

// Step of the last launch_render_multiframe call on this thread that returned an error (for messages).
const char *wavefront_error_site();

cudaError_t launch_render_wavefront(const DevScene &scene, const DevCamera &cam, const FrameBuffers &fbuf,
                                    const RenderParams &p, bool count, Counters *counters, WavefrontState &s,
                                    int num_sms, cudaStream_t stream, uint32_t *launches, LaunchEvents *ev,
                                    const WfTuning &tuning);

}  // namespace spk
