// spk_api.cu -- the C ABI (include/spk.h) and the host renderer behind it.
//
// `spk_ctx` plays CPURenderer (libraries/source/renderer/renderer/CPURenderer.cpp) for one scene: it owns
// the resident scene (SceneRenderProxy's BVHs, flattened for the device), the camera and config snapshot,
// the frame buffers, and the sample bookkeeping of CameraRenderProxy (CameraRenderProxy.cpp:66-75) and
// CPURenderer::dispatched_sample_count_ (CPURenderer.cpp:128-137, 206-207).
#include <cuda.h>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <exception>
#include <limits>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/spk.h"
#include "batch_plan.h"
#include "bvh_builder.h"
#include "bvh_device.cuh"
#include "fault.h"
#include "image_io.h"
#include "kernels.cuh"
#include "wavefront.cuh"

using namespace spk;

namespace spk {
namespace {
std::atomic<unsigned> g_fail_allocation{0};  // the nth next device allocation fails; 0: none
}  // namespace

void fault_arm_allocation(unsigned nth) { g_fail_allocation.store(nth); }

bool fault_allocation() {
    unsigned c = g_fail_allocation.load();
    while (c > 0) {
        if (g_fail_allocation.compare_exchange_weak(c, c - 1)) return c == 1;
    }
    return false;
}
}  // namespace spk

namespace {

// An NVTX range around one entry point (shown by Nsight tools; free when no tool is attached), the
// PROFILE_SCOPE of the reference's passes (core/Profiler.h:9-28).
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

template <class T>
struct DevBuf {
    T *ptr = nullptr;
    size_t count = 0;
    void reset() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        count = 0;
    }
};

// What a mesh's BLAS occupies in the scene arrays; kept to refit it after the vertices move.
struct MeshBlas {
    uint32_t root = kInvalid;  // node index of the BLAS root, kInvalid for an empty mesh
    uint32_t node_count = 0;
    std::vector<uint32_t> levels;  // first node (relative to root) of each BFS depth, then node_count
    uint32_t tri_first = 0, tri_count = 0;  // triangle records, in triangles
    uint32_t vert_base = 0, face_base = 0;
    double bounds[6] = {0, 0, 0, 0, 0, 0};  // local-space box (lo, hi)
};

// One mesh's BLAS from a BVH blob (spk_set_bvh): its wide nodes and leaf items as the builders return them,
// the mesh it was built for (face and vertex counts, a hash of positions and indices) and the BVH knobs.
struct CachedBlas {
    uint32_t num_faces = 0, num_vertices = 0;
    uint64_t hash = 0;
    WideBvh bvh;
};

// 64-bit FNV-1a over the 32-bit words of a mesh's positions and indices.
uint64_t geometry_hash(const float *positions, uint32_t num_vertices, const uint32_t *indices, uint32_t num_faces) {
    uint64_t h = 1469598103934665603ull;
    auto mix = [&h](const void *p, size_t words) {
        const auto *w = static_cast<const uint32_t *>(p);
        for (size_t i = 0; i < words; ++i) h = (h ^ w[i]) * 1099511628211ull;
    };
    if (positions) mix(positions, 3ull * num_vertices);
    if (indices) mix(indices, 3ull * num_faces);
    return h;
}

// The instance list, mesh geometry and BLAS placement of a single-scene context, kept on the host so that
// spk_set_instances / spk_set_instance_transforms / spk_update_mesh can rebuild the TLAS and the light table
// (SceneRenderProxy::UpdateBVH, SceneRenderProxy.cpp:269-297) without rebuilding any BLAS.
struct DynScene {
    bool valid = false;
    std::vector<spk_instance> instances;
    std::vector<std::vector<float>> positions;   // per mesh, 3 floats per vertex
    std::vector<std::vector<uint32_t>> indices;  // per mesh, 3 per face
    std::vector<MeshBlas> blas;
    std::vector<DevMaterial> mats;
    std::vector<DevInstance> insts;
    DevSceneDesc desc{};
    spk_tuning built_with{};     // the BVH knobs of the build (spk_save_bvh records them)
    uint32_t tlas_root = 0;      // first TLAS node = number of BLAS nodes
    uint32_t node_capacity = 0;  // nodes allocated on the device
};

spk_tuning default_tuning() {
    spk_tuning t{};
    spk_tuning_defaults(&t);
    return t;
}

}  // namespace

struct spk_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
    std::vector<cudaEvent_t> event_pool;  // start/stop pairs around traversal launches, reused across calls
    LaunchEvents launch_events{};
    uint32_t instrumentation = SPK_INSTR_NONE;
    std::string error;

    // resident scene
    DevBuf<uint4> nodes;
    DevBuf<float4> tris;
    DevBuf<uint32_t> tlas_items;
    DevBuf<DevInstance> instances;
    DevBuf<float4> verts;
    DevBuf<uint4> faces;
    DevBuf<DevMaterial> materials;
    DevBuf<float4> sky;
    DevBuf<DevLight> lights;
    DevBuf<float> light_cdf;
    DevBuf<DevSceneDesc> scene_descs;
    DevBuf<DevTexture> textures;
    DevBuf<float4> texels;
    DevScene scene{};
    bool has_scene = false;
    DynScene dyn;                          // single-scene contexts: what the incremental updates need
    std::vector<CachedBlas> bvh_cache;     // BLASes handed in by spk_set_bvh, by mesh index
    uint32_t bvh_cache_knobs[4] = {0, 0, 0, 0};  // width, leaf size, collapse, builder they were built with
    uint32_t blas_reused = 0;              // BLASes the last scene build took from bvh_cache
    DevBuf<float> dyn_pos, dyn_attr, dyn_boxes;  // refit scratch: positions, normals + tangents, node boxes
    uint32_t bvh_nodes = 0;
    uint64_t bvh_bytes = 0;

    // config / camera / frame buffers
    spk_config cfg{};
    bool has_config = false;
    uint32_t spp_eff = 1;
    DevCamera cam{};
    bool has_camera = false;
    DevBuf<float4> gcolor, gnormal, fb;
    DevBuf<ushort4> out;
    DevBuf<float4> guide_nd, guide_albedo;  // primary-hit guides (spk_render_guides)
    DevBuf<uint8_t> rgba8_tables;           // half -> RGBA8 tables of the screenshot conversion (colour, alpha)
    DevBuf<uchar4> rgba8;                   // spk_read_rgba8 scratch
    DevBuf<ushort4> fb_half;                // spk_save_image (EXR) scratch
    WavefrontState wf{};
    ChunkGraph chunk_graph{};
    // batch (spk_render_batch)
    WavefrontState wf_batch{};
    DevBuf<DevRequest> batch_reqs;
    DevBuf<float4> batch_hdr;
    DevBuf<ushort4> batch_img;
    std::vector<DevRequest> batch_host;
    spk_tuning tuning = default_tuning();

    // CameraRenderProxy / CPURenderer sample bookkeeping
    uint32_t cumulated = 0, pending = 0, dispatched = 0;
    bool dirty = true;
    // The frame buffer that bookkeeping belongs to: nullptr = fb; otherwise the caller's buffer that
    // spk_render_noalloc accumulated into last. Rendering into another buffer restarts the accumulation.
    const void *accum_target = nullptr;
    std::vector<float> frame_weights;    // multi-frame wavefront: per-frame moving-average weight
    std::vector<uint32_t> frame_seeds;   // multi-frame wavefront: per-frame seed base

    // counters
    Counters *counters = nullptr;  // device
    const Counters *noalloc_counters = nullptr;  // set when the last call was spk_render_noalloc: its counters
    spk_stats last{};
    bool stats_pending = false;
    uint32_t launches_in_call = 0;
};

namespace {

spk_status fail(spk_ctx *ctx, spk_status code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (ctx) ctx->error = buf;
    return code;
}

spk_status cuda_fail(spk_ctx *ctx, cudaError_t e, const char *what) {
    return fail(ctx, e == cudaErrorMemoryAllocation ? SPK_ERR_OUT_OF_MEMORY : SPK_ERR_CUDA, "%s: %s", what,
                cudaGetErrorString(e));
}

// The context's own frame buffers hold the accumulation unless the last frames went into a caller's
// buffer (spk_render_noalloc); reading or saving them then would return frames the counts do not describe.
spk_status require_own_buffers(spk_ctx *ctx) {
    if (ctx->accum_target)
        return fail(ctx, SPK_ERR_NOT_READY,
                    "the last frames were rendered into the caller's buffers by spk_render_noalloc; the context's "
                    "frame buffer holds none of them (spk_render restarts it)");
    return SPK_OK;
}

template <class T>
cudaError_t upload(DevBuf<T> &buf, const T *host, size_t count, cudaStream_t stream) {
    buf.reset();
    if (count == 0) return cudaSuccess;
    cudaError_t e = fault_allocation() ? cudaErrorMemoryAllocation : cudaMalloc(&buf.ptr, count * sizeof(T));
    if (e != cudaSuccess) return e;
    buf.count = count;
    e = cudaMemcpyAsync(buf.ptr, host, count * sizeof(T), cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(stream);
}

// As upload, into an allocation of max(count, capacity) elements (the tail is zeroed).
template <class T>
cudaError_t upload_with_capacity(DevBuf<T> &buf, const T *host, size_t count, size_t capacity, cudaStream_t stream) {
    buf.reset();
    capacity = std::max(capacity, count);
    if (capacity == 0) return cudaSuccess;
    cudaError_t e = fault_allocation() ? cudaErrorMemoryAllocation : cudaMalloc(&buf.ptr, capacity * sizeof(T));
    if (e != cudaSuccess) return e;
    buf.count = capacity;
    if (capacity > count &&
        (e = cudaMemsetAsync(buf.ptr + count, 0, (capacity - count) * sizeof(T), stream)) != cudaSuccess)
        return e;
    if (count && (e = cudaMemcpyAsync(buf.ptr, host, count * sizeof(T), cudaMemcpyHostToDevice, stream)) != cudaSuccess)
        return e;
    return cudaStreamSynchronize(stream);
}

template <class T>
cudaError_t alloc(DevBuf<T> &buf, size_t count) {
    buf.reset();
    if (count == 0) return cudaSuccess;
    cudaError_t e = fault_allocation() ? cudaErrorMemoryAllocation : cudaMalloc(&buf.ptr, count * sizeof(T));
    if (e == cudaSuccess) buf.count = count;
    return e;
}

int host_threads() {
    const unsigned n = std::thread::hardware_concurrency();
    return n == 0 ? 1 : static_cast<int>(std::min(n, 64u));
}

// Host loops over large meshes run in chunks on up to host_threads() threads. Every chunk writes a disjoint
// range (or its own partial result), so the output never depends on the thread count.
struct ChunkPlan {
    uint64_t n = 0, step = 0, chunks = 0;
};

ChunkPlan plan_chunks(uint64_t n) {
    constexpr uint64_t kMinChunk = 1u << 16;
    ChunkPlan p;
    p.n = n;
    p.chunks = std::max<uint64_t>(1, std::min<uint64_t>(static_cast<uint64_t>(host_threads()), (n + kMinChunk - 1) / kMinChunk));
    p.step = (n + p.chunks - 1) / p.chunks;
    return p;
}

// Runs fn(chunk, begin, end) over the chunks of `p`; a thread that cannot be started runs inline.
template <class F>
void run_chunks(const ChunkPlan &p, F &&fn) {
    if (p.n == 0) return;
    std::vector<std::thread> pool;
    pool.reserve(p.chunks);
    for (uint64_t c = 1; c < p.chunks; ++c) {
        const uint64_t lo = c * p.step, hi = std::min(p.n, lo + p.step);
        if (lo >= hi) continue;
        try {
            pool.emplace_back([&fn, c, lo, hi] { fn(c, lo, hi); });
        } catch (const std::exception &) {
            fn(c, lo, hi);
        }
    }
    fn(uint64_t{0}, uint64_t{0}, std::min(p.n, p.step));
    for (std::thread &t : pool) t.join();
}

template <class F>
void parallel_for(uint64_t n, F &&fn) {
    run_chunks(plan_chunks(n), [&fn](uint64_t, uint64_t lo, uint64_t hi) { fn(lo, hi); });
}

// Outward-rounded world box of a transformed local box (8 corners, evaluated in double).
BuildBox world_box(const float *m, const double lo[3], const double hi[3]) {
    BuildBox b;
    double mn[3] = {std::numeric_limits<double>::max(), std::numeric_limits<double>::max(),
                    std::numeric_limits<double>::max()};
    double mx[3] = {-mn[0], -mn[1], -mn[2]};
    for (int c = 0; c < 8; ++c) {
        const double p[3] = {(c & 1) ? hi[0] : lo[0], (c & 2) ? hi[1] : lo[1], (c & 4) ? hi[2] : lo[2]};
        for (int r = 0; r < 3; ++r) {
            const double w = m[4 * r + 3] + m[4 * r] * p[0] + m[4 * r + 1] * p[1] + m[4 * r + 2] * p[2];
            mn[r] = std::min(mn[r], w);
            mx[r] = std::max(mx[r], w);
        }
    }
    for (int r = 0; r < 3; ++r) {
        const double pad = 1e-6 * (std::fabs(mn[r]) + std::fabs(mx[r]) + (mx[r] - mn[r])) + 1e-30;
        b.lo[r] = std::nextafter(static_cast<float>(mn[r] - pad), -std::numeric_limits<float>::max());
        b.hi[r] = std::nextafter(static_cast<float>(mx[r] + pad), std::numeric_limits<float>::max());
    }
    return b;
}

// Makes room for `pairs` start/stop event pairs and resets the per-call launch timing.
cudaError_t prepare_events(spk_ctx *ctx, size_t pairs) {
    while (ctx->event_pool.size() < 2 * pairs) {
        cudaEvent_t ev;
        const cudaError_t e = cudaEventCreate(&ev);
        if (e != cudaSuccess) return e;
        ctx->event_pool.push_back(ev);
    }
    ctx->launch_events.pairs = ctx->event_pool.data();
    ctx->launch_events.capacity = static_cast<int>(ctx->event_pool.size() / 2);
    ctx->launch_events.used = 0;
    ctx->launch_events.graph_ms = 0.f;
    ctx->launch_events.graph_launches = 0;
    return cudaSuccess;
}

void append_wide(std::vector<WideNode> &all, const WideBvh &w, uint32_t item_offset) {
    const uint32_t base = static_cast<uint32_t>(all.size());
    for (WideNode n : w.nodes) {
        n.child_base += base;
        n.item_base += item_offset;
        all.push_back(n);
    }
}

}  // namespace

namespace {

// Binary SAH build + collapse to 8-wide nodes as the tuning asks: the SAH-optimal collapse starts from
// one item per binary leaf and chooses the wide leaves itself; the greedy one keeps the binary leaves.
WideBvh build_wide(const std::vector<BuildBox> &boxes, const spk_tuning &t, int threads) {
    if (t.bvh_collapse) {
        const Bvh2 b2 = build_bvh2(boxes, 1, threads);
        return collapse_wide_sah(b2, static_cast<int>(t.bvh_width), static_cast<int>(t.bvh_leaf_size));
    }
    const Bvh2 b2 = build_bvh2(boxes, t.bvh_leaf_size, threads);
    return collapse_wide(b2, static_cast<int>(t.bvh_width));
}

// Node ranges of the BFS depths of a collapsed BVH (children always follow their parent, depth by depth).
std::vector<uint32_t> wide_levels(const WideBvh &w) {
    std::vector<uint32_t> depth(w.nodes.size(), 0), levels{0};
    for (uint32_t i = 0; i < w.nodes.size(); ++i) {
        const WideNode &n = w.nodes[i];
        if (i > 0 && depth[i] != depth[i - 1]) levels.push_back(i);
        for (uint32_t r = 0; r < static_cast<uint32_t>(__builtin_popcount(n.imask)); ++r)
            depth[n.child_base + r] = depth[i] + 1;
    }
    levels.push_back(static_cast<uint32_t>(w.nodes.size()));
    return levels;
}

// Materials; the emissive test is SamplePixel's `emissive_color.norm() > Eps` (CPURenderer.cpp:286-287).
std::vector<DevMaterial> build_materials(const spk_material *materials, uint32_t num_materials,
                                         const spk_material_maps *maps) {
    std::vector<DevMaterial> out(num_materials);
    for (uint32_t k = 0; k < num_materials; ++k) {
        const spk_material &s = materials[k];
        DevMaterial &d = out[k];
        std::memset(&d, 0, sizeof(d));
        for (int c = 0; c < 3; ++c) {
            d.base[c] = s.base_color[c];
            d.emissive[c] = s.emissive[c];
        }
        d.type = s.type;
        const volatile float e0 = s.emissive[0] * s.emissive[0], e1 = s.emissive[1] * s.emissive[1],
                             e2 = s.emissive[2] * s.emissive[2];
        const volatile float sn = e0 + (e1 + e2);
        d.is_emissive = std::sqrt(static_cast<float>(sn)) > kEps ? 1u : 0u;
        d.metallic = s.metallic;
        d.roughness = s.roughness;
        d.eta = s.eta;
        auto tex = [](int32_t i) { return i < 0 ? kInvalid : static_cast<uint32_t>(i); };
        d.tex_base = maps ? tex(maps[k].base_color) : kInvalid;
        d.tex_mr = maps ? tex(maps[k].metallic_roughness) : kInvalid;
        d.tex_emissive = maps ? tex(maps[k].emissive) : kInvalid;
        d.tex_normal = maps ? tex(maps[k].normal) : kInvalid;
    }
    return out;
}

// Instance records and their world boxes (the TLAS build input, SceneRenderProxy.cpp:31-69).
void instance_records(const spk_instance *instances, uint32_t num_instances, const std::vector<MeshBlas> &blas,
                      const std::vector<DevMaterial> &mats, std::vector<DevInstance> &insts,
                      std::vector<BuildBox> &boxes, float &abs_x, float lo_out[3], float hi_out[3]) {
    insts.assign(num_instances, DevInstance{});
    boxes.assign(num_instances, BuildBox{});
    abs_x = 0.f;
    for (uint32_t k = 0; k < num_instances; ++k) {
        const spk_instance &in = instances[k];
        DevInstance &d = insts[k];
        std::memset(&d, 0, sizeof(d));
        std::memcpy(d.m, in.transform, sizeof(d.m));
        std::memcpy(d.minv, in.inv_transform, sizeof(d.minv));
        d.type = in.type;
        d.material = in.material_id;
        d.radius = in.radius;
        d.normal_map = kInvalid;
        d.light_base = kInvalid;
        if (in.type == SPK_PRIM_SPHERE) {
            d.blas_root = kInvalid;
            const double r = std::fabs(static_cast<double>(in.radius));
            const double lo[3] = {-r, -r, -r}, hi[3] = {r, r, r};
            const float tm[12] = {1, 0, 0, in.transform[3], 0, 1, 0, in.transform[7], 0, 0, 1, in.transform[11]};
            boxes[k] = world_box(tm, lo, hi);
        } else {
            const MeshBlas &b = blas[in.mesh_id];
            d.blas_root = b.root;
            d.vert_base = b.vert_base;
            d.face_base = b.face_base;
            d.normal_map = mats[in.material_id].tex_normal;
            if (d.blas_root == kInvalid) {
                const double z[3] = {0, 0, 0};
                boxes[k] = world_box(in.transform, z, z);
            } else {
                boxes[k] = world_box(in.transform, b.bounds, b.bounds + 3);
            }
        }
        abs_x = std::max(abs_x, std::max(std::fabs(boxes[k].lo[0]), std::fabs(boxes[k].hi[0])));
        for (int a = 0; a < 3; ++a) {
            lo_out[a] = std::min(lo_out[a], boxes[k].lo[a]);
            hi_out[a] = std::max(hi_out[a], boxes[k].hi[a]);
        }
    }
}

// Emissive triangles of mesh instances in world space (instance then face order) and their area CDF, for
// next-event estimation. A textured emission varies over the triangle: such emitters are reached by BSDF
// sampling only (no light-table entry, so their hits take the full emission).
void light_table(const spk_instance *instances, uint32_t num_instances, const spk_mesh *meshes,
                 const std::vector<DevMaterial> &mats, std::vector<DevInstance> &insts, std::vector<DevLight> &lights,
                 std::vector<float> &cdf, float &total) {
    lights.clear();
    cdf.clear();
    total = 0.f;
    for (uint32_t k = 0; k < num_instances; ++k) {
        const spk_instance &in = instances[k];
        insts[k].light_base = kInvalid;
        if (in.type != SPK_PRIM_MESH || !mats[in.material_id].is_emissive || mats[in.material_id].tex_emissive != kInvalid)
            continue;
        const spk_mesh &m = meshes[in.mesh_id];
        insts[k].light_base = static_cast<uint32_t>(lights.size());
        for (uint32_t f = 0; f < m.num_faces; ++f) {
            f3 w[3];
            for (int c = 0; c < 3; ++c) {
                const float *p = m.positions + 3 * m.indices[3 * f + c];
                w[c] = xform_point(in.transform, mk3(p[0], p[1], p[2]));
            }
            DevLight L{};
            const f3 e1 = w[1] - w[0], e2 = w[2] - w[0];
            const f3 cr = cross(e1, e2);
            const float len = std::sqrt(sqnorm(cr));
            const f3 ng = len > 0.f ? mk3(cr.x / len, cr.y / len, cr.z / len) : mk3(0.f, 0.f, 0.f);
            const float vals[5][3] = {{w[0].x, w[0].y, w[0].z}, {e1.x, e1.y, e1.z}, {e2.x, e2.y, e2.z},
                                      {ng.x, ng.y, ng.z},
                                      {mats[in.material_id].emissive[0], mats[in.material_id].emissive[1],
                                       mats[in.material_id].emissive[2]}};
            std::memcpy(L.p0, vals[0], 12);
            std::memcpy(L.e1, vals[1], 12);
            std::memcpy(L.e2, vals[2], 12);
            std::memcpy(L.ng, vals[3], 12);
            std::memcpy(L.emission, vals[4], 12);
            L.area = 0.5f * len;
            lights.push_back(L);
        }
    }
    for (const DevLight &L : lights) {
        total = total + L.area;
        cdf.push_back(total);
    }
    if (!(total > 0.f)) {
        lights.clear();
        cdf.clear();
        total = 0.f;
        for (uint32_t k = 0; k < num_instances; ++k) insts[k].light_base = kInvalid;
    }
}

struct HostScene {
    std::vector<WideNode> nodes;
    std::vector<float4> tris;
    std::vector<uint32_t> tlas_items;
    std::vector<DevInstance> insts;
    std::vector<float4> verts;
    std::vector<uint4> faces;
    std::vector<DevMaterial> mats;
    std::vector<float4> cube;
    std::vector<DevLight> lights;
    std::vector<float> light_cdf;
    std::vector<DevTexture> textures;
    std::vector<float4> texels;
    std::vector<MeshBlas> blas;  // per mesh (single-scene builds)
    uint32_t tlas_root = kInvalid;
    uint32_t sky_mode = SPK_SKY_NONE, sky_size = 0;
    float sky_color[3] = {0.f, 0.f, 0.f};
    float abs_x = 0.f, light_total = 0.f;
    float lo[3] = {std::numeric_limits<float>::max(), std::numeric_limits<float>::max(),
                   std::numeric_limits<float>::max()};
    float hi[3] = {-std::numeric_limits<float>::max(), -std::numeric_limits<float>::max(),
                   -std::numeric_limits<float>::max()};
};

// Validates one scene description and builds its host-side records (BLAS per mesh, TLAS, vertex/face
// records, materials, emissive-triangle light table, sky texels), with indices local to the scene.
spk_status build_host_scene(spk_ctx *ctx, const spk_mesh *meshes, uint32_t num_meshes, const spk_instance *instances,
                            uint32_t num_instances, const spk_material *materials, uint32_t num_materials,
                            const spk_sky *sky, const spk_texture *textures, uint32_t num_textures,
                            const spk_material_maps *maps, HostScene &hs) {
    if (!ctx) return SPK_ERR_INVALID_ARGUMENT;
    if ((num_meshes && !meshes) || (num_instances && !instances) || (num_materials && !materials))
        return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "null scene array");
    const int threads = host_threads();
    // Validate.
    for (uint32_t k = 0; k < num_meshes; ++k) {
        const spk_mesh &m = meshes[k];
        if (m.num_faces && (!m.positions || !m.normals || !m.indices))
            return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "mesh %u: positions, normals and indices are required", k);
        const uint64_t ni = m.indices ? 3ull * m.num_faces : 0;
        std::atomic<uint64_t> first_bad{ni};
        parallel_for(ni, [&](uint64_t lo, uint64_t hi) {
            for (uint64_t f = lo; f < hi; ++f) {
                if (m.indices[f] >= m.num_vertices) {
                    uint64_t cur = first_bad.load();
                    while (f < cur && !first_bad.compare_exchange_weak(cur, f)) {
                    }
                    break;
                }
            }
        });
        if (first_bad.load() < ni)
            return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "mesh %u: index %u out of range", k, m.indices[first_bad.load()]);
    }
    for (uint32_t k = 0; k < num_instances; ++k) {
        const spk_instance &in = instances[k];
        if (in.type != SPK_PRIM_MESH && in.type != SPK_PRIM_SPHERE)
            return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "instance %u: bad type", k);
        if (in.type == SPK_PRIM_MESH && in.mesh_id >= num_meshes)
            return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "instance %u: mesh_id out of range", k);
        if (in.material_id >= num_materials)
            return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "instance %u: material_id out of range", k);
    }
    if (sky && sky->mode == SPK_SKY_CUBE && (!sky->cube_rgba || sky->cube_size == 0))
        return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "cube sky without texels");
    if (num_textures && !textures) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "null texture array");
    for (uint32_t k = 0; k < num_textures; ++k)
        if (textures[k].width == 0 || textures[k].height == 0 || !textures[k].rgba)
            return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "texture %u: empty", k);
    if (maps) {
        for (uint32_t k = 0; k < num_materials; ++k) {
            const int32_t t[4] = {maps[k].base_color, maps[k].metallic_roughness, maps[k].emissive, maps[k].normal};
            for (int32_t i : t)
                if (i < -1 || i >= static_cast<int32_t>(num_textures))
                    return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "material %u: texture index %d out of range", k, i);
        }
    }
    static_assert(sizeof(float4) == 4 * sizeof(float), "texel layout");
    for (uint32_t k = 0; k < num_textures; ++k) {
        const spk_texture &t = textures[k];
        const size_t base = hs.texels.size();
        hs.textures.push_back(DevTexture{static_cast<uint32_t>(base), t.width, t.height, t.srgb ? 1u : 0u});
        const size_t nt = static_cast<size_t>(t.width) * t.height;
        hs.texels.resize(base + nt);
        std::memcpy(hs.texels.data() + base, t.rgba, nt * sizeof(float4));
    }

    // BLAS per mesh: binned SAH BVH2 (<= 3 triangles per leaf) collapsed to 8-wide nodes.
    hs.blas.assign(num_meshes, MeshBlas{});
    size_t total_verts = 0, total_faces = 0;
    for (uint32_t k = 0; k < num_meshes; ++k) {
        total_verts += meshes[k].num_vertices;
        total_faces += meshes[k].num_faces;
    }
    hs.verts.resize(3 * total_verts);
    hs.faces.resize(total_faces);
    size_t vert_base = 0, face_base = 0;
    for (uint32_t k = 0; k < num_meshes; ++k) {
        const spk_mesh &m = meshes[k];
        MeshBlas &mbl = hs.blas[k];
        mbl.vert_base = static_cast<uint32_t>(vert_base);
        mbl.face_base = static_cast<uint32_t>(face_base);
        float4 *vrec = hs.verts.data() + 3 * vert_base;
        uint4 *frec = hs.faces.data() + face_base;
        parallel_for(m.num_vertices, [&](uint64_t lo, uint64_t hi) {
            static const float kNoNormal[3] = {0.f, 0.f, 0.f};  // face-less meshes may come without normals
            for (uint64_t v = lo; v < hi; ++v) {
                const float *n = m.normals ? m.normals + 3 * v : kNoNormal;
                const float t[4] = {m.tangents ? m.tangents[4 * v] : 1.f, m.tangents ? m.tangents[4 * v + 1] : 0.f,
                                    m.tangents ? m.tangents[4 * v + 2] : 0.f, m.tangents ? m.tangents[4 * v + 3] : 1.f};
                const float uv[2] = {m.uvs ? m.uvs[2 * v] : 0.f, m.uvs ? m.uvs[2 * v + 1] : 0.f};
                vrec[3 * v] = make_float4(n[0], n[1], n[2], t[0]);
                vrec[3 * v + 1] = make_float4(t[1], t[2], t[3], uv[0]);
                vrec[3 * v + 2] = make_float4(uv[1], 0.f, 0.f, 0.f);
            }
        });
        parallel_for(m.num_faces, [&](uint64_t lo, uint64_t hi) {
            for (uint64_t f = lo; f < hi; ++f)
                frec[f] = make_uint4(m.indices[3 * f], m.indices[3 * f + 1], m.indices[3 * f + 2], 0u);
        });
        vert_base += m.num_vertices;
        face_base += m.num_faces;
        double *mb = mbl.bounds;
        for (int a = 0; a < 3; ++a) {
            mb[a] = std::numeric_limits<double>::max();
            mb[3 + a] = -std::numeric_limits<double>::max();
        }
        if (m.num_faces == 0) continue;
        const bool device_build = ctx->tuning.bvh_builder != 0;
        std::vector<BuildBox> boxes(device_build ? 0 : m.num_faces);
        // Face boxes (host build) and the mesh bounds, per chunk; min / max are exact, so combining the
        // chunks' bounds gives the same bounds in any order.
        const ChunkPlan plan = plan_chunks(m.num_faces);
        std::vector<std::array<double, 6>> part(plan.chunks);
        run_chunks(plan, [&](uint64_t c, uint64_t lo, uint64_t hi) {
            std::array<double, 6> pb;
            for (int a = 0; a < 3; ++a) {
                pb[a] = std::numeric_limits<double>::max();
                pb[3 + a] = -std::numeric_limits<double>::max();
            }
            for (uint64_t f = lo; f < hi; ++f) {
                BuildBox b;
                for (int a = 0; a < 3; ++a) {
                    b.lo[a] = std::numeric_limits<float>::max();
                    b.hi[a] = -std::numeric_limits<float>::max();
                }
                for (int cc = 0; cc < 3; ++cc) {
                    const float *p = m.positions + 3 * m.indices[3 * f + cc];
                    for (int a = 0; a < 3; ++a) {
                        b.lo[a] = std::min(b.lo[a], p[a]);
                        b.hi[a] = std::max(b.hi[a], p[a]);
                        pb[a] = std::min(pb[a], static_cast<double>(p[a]));
                        pb[3 + a] = std::max(pb[3 + a], static_cast<double>(p[a]));
                    }
                }
                if (!device_build) boxes[f] = b;
            }
            part[c] = pb;
        });
        for (const std::array<double, 6> &pb : part) {
            for (int a = 0; a < 3; ++a) {
                mb[a] = std::min(mb[a], pb[a]);
                mb[3 + a] = std::max(mb[3 + a], pb[3 + a]);
            }
        }
        WideBvh wide;
        const uint32_t knobs[4] = {ctx->tuning.bvh_width, ctx->tuning.bvh_leaf_size, ctx->tuning.bvh_collapse,
                                   ctx->tuning.bvh_builder};
        const CachedBlas *cached = nullptr;
        if (k < ctx->bvh_cache.size() && std::memcmp(knobs, ctx->bvh_cache_knobs, sizeof(knobs)) == 0) {
            const CachedBlas &c = ctx->bvh_cache[k];
            if (c.num_faces == m.num_faces && c.num_vertices == m.num_vertices &&
                c.hash == geometry_hash(m.positions, m.num_vertices, m.indices, m.num_faces))
                cached = &c;
        }
        if (cached) {
            wide = cached->bvh;
            ++ctx->blas_reused;
        } else if (device_build) {
            std::vector<uint32_t> lv;
            const cudaError_t e = build_wide_device(m.positions, m.num_vertices, m.indices, m.num_faces,
                                                    static_cast<int>(ctx->tuning.bvh_width),
                                                    static_cast<int>(ctx->tuning.bvh_leaf_size),
                                                    ctx->tuning.bvh_builder == 2, ctx->stream, wide, lv);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "device BVH build");
        } else {
            wide = build_wide(boxes, ctx->tuning, threads);
        }
        const uint32_t tri_offset = static_cast<uint32_t>(hs.tris.size() / 3);
        mbl.root = static_cast<uint32_t>(hs.nodes.size());
        mbl.node_count = static_cast<uint32_t>(wide.nodes.size());
        mbl.levels = wide_levels(wide);
        mbl.tri_first = tri_offset;
        mbl.tri_count = static_cast<uint32_t>(wide.items.size());
        append_wide(hs.nodes, wide, tri_offset);
        const size_t t0 = hs.tris.size();
        hs.tris.resize(t0 + 3 * wide.items.size());
        float4 *trec = hs.tris.data() + t0;
        parallel_for(wide.items.size(), [&](uint64_t lo, uint64_t hi) {
            for (uint64_t i = lo; i < hi; ++i) {
                const uint32_t face = wide.items[i];
                const float *p0 = m.positions + 3 * m.indices[3 * face];
                const float *p1 = m.positions + 3 * m.indices[3 * face + 1];
                const float *p2 = m.positions + 3 * m.indices[3 * face + 2];
                // BLAS::Triangle::Set: e1 = v1 - v0, e2 = v2 - v0 (MeshRenderProxy.cpp:80-86)
                const float e1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
                const float e2[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
                uint32_t fbits = face;
                float ff;
                std::memcpy(&ff, &fbits, 4);
                trec[3 * i] = make_float4(p0[0], p0[1], p0[2], e1[0]);
                trec[3 * i + 1] = make_float4(e1[1], e1[2], e2[0], e2[1]);
                trec[3 * i + 2] = make_float4(e2[2], ff, 0.f, 0.f);
            }
        });
    }
    hs.mats = build_materials(materials, num_materials, maps);
    // Instances + TLAS over their world boxes (TLAS::Build, SceneRenderProxy.cpp:31-69).
    std::vector<BuildBox> inst_boxes;
    float abs_x = 0.f;
    instance_records(instances, num_instances, hs.blas, hs.mats, hs.insts, inst_boxes, abs_x, hs.lo, hs.hi);
    if (num_instances > 0) {
        const WideBvh wide = build_wide(inst_boxes, ctx->tuning, threads);
        hs.tlas_root = static_cast<uint32_t>(hs.nodes.size());
        append_wide(hs.nodes, wide, 0);
        hs.tlas_items = wide.items;
    }
    light_table(instances, num_instances, meshes, hs.mats, hs.insts, hs.lights, hs.light_cdf, hs.light_total);
    if (sky && sky->mode == SPK_SKY_CUBE) {
        const size_t n = 6ull * sky->cube_size * sky->cube_size;
        hs.cube.resize(n);
        std::memcpy(hs.cube.data(), sky->cube_rgba, n * sizeof(float4));
    }
    hs.sky_mode = sky ? sky->mode : static_cast<uint32_t>(SPK_SKY_NONE);
    hs.sky_size = sky ? sky->cube_size : 0;
    for (int c = 0; c < 3; ++c) hs.sky_color[c] = sky ? sky->color[c] : 0.f;
    hs.abs_x = abs_x;
    return SPK_OK;
}

// Appends scene `s` to `all` (node, triangle, instance, vertex, face, material, texel and light indices
// offset into the shared arrays) and describes it in `d`.
void append_scene(HostScene &all, const HostScene &s, DevSceneDesc &d) {
    const uint32_t node_off = static_cast<uint32_t>(all.nodes.size());
    const uint32_t tri_off = static_cast<uint32_t>(all.tris.size() / 3);
    const uint32_t item_off = static_cast<uint32_t>(all.tlas_items.size());
    const uint32_t inst_off = static_cast<uint32_t>(all.insts.size());
    const uint32_t vert_off = static_cast<uint32_t>(all.verts.size() / 3);
    const uint32_t face_off = static_cast<uint32_t>(all.faces.size());
    const uint32_t mat_off = static_cast<uint32_t>(all.mats.size());
    // BLAS nodes come first, the TLAS nodes (from tlas_root on) last; items index triangles or TLAS items.
    for (size_t k = 0; k < s.nodes.size(); ++k) {
        WideNode n = s.nodes[k];
        n.child_base += node_off;
        const bool tlas = s.tlas_root != kInvalid && k >= s.tlas_root;
        n.item_base += tlas ? item_off : tri_off;
        all.nodes.push_back(n);
    }
    all.tris.insert(all.tris.end(), s.tris.begin(), s.tris.end());
    for (uint32_t it : s.tlas_items) all.tlas_items.push_back(it + inst_off);
    for (DevInstance in : s.insts) {
        if (in.blas_root != kInvalid) in.blas_root += node_off;
        in.vert_base += vert_off;
        in.face_base += face_off;
        in.material += mat_off;
        if (in.normal_map != kInvalid) in.normal_map += static_cast<uint32_t>(all.textures.size());
        all.insts.push_back(in);  // light_base stays relative to the scene's light slice
    }
    all.verts.insert(all.verts.end(), s.verts.begin(), s.verts.end());
    all.faces.insert(all.faces.end(), s.faces.begin(), s.faces.end());
    const uint32_t tex_off = static_cast<uint32_t>(all.textures.size());
    const uint32_t texel_off = static_cast<uint32_t>(all.texels.size());
    for (DevMaterial m : s.mats) {
        for (uint32_t *t : {&m.tex_base, &m.tex_mr, &m.tex_emissive, &m.tex_normal})
            if (*t != kInvalid) *t += tex_off;
        all.mats.push_back(m);
    }
    for (DevTexture t : s.textures) {
        t.offset += texel_off;
        all.textures.push_back(t);
    }
    all.texels.insert(all.texels.end(), s.texels.begin(), s.texels.end());
    d = DevSceneDesc{};
    d.tlas_root = s.tlas_root == kInvalid ? kInvalid : s.tlas_root + node_off;
    d.sky_mode = s.sky_mode;
    d.sky_size = s.sky_size;
    for (int c = 0; c < 3; ++c) d.sky_color[c] = s.sky_color[c];
    d.sky_offset = static_cast<uint32_t>(all.cube.size());
    all.cube.insert(all.cube.end(), s.cube.begin(), s.cube.end());
    d.light_base = static_cast<uint32_t>(all.lights.size());
    d.num_lights = static_cast<uint32_t>(s.lights.size());
    d.light_total = s.light_total;
    all.lights.insert(all.lights.end(), s.lights.begin(), s.lights.end());
    all.light_cdf.insert(all.light_cdf.end(), s.light_cdf.begin(), s.light_cdf.end());
    all.abs_x = std::max(all.abs_x, s.abs_x);
    for (int a = 0; a < 3; ++a) {
        all.lo[a] = std::min(all.lo[a], s.lo[a]);
        all.hi[a] = std::max(all.hi[a], s.hi[a]);
    }
}

// Uploads concatenated scene records and points the context's DevScene at them (scene 0 by default).
// `node_capacity` reserves room for a TLAS that grows on a later incremental update.
spk_status upload_scene(spk_ctx *ctx, const HostScene &hs, const std::vector<DevSceneDesc> &descs,
                        size_t node_capacity = 0) {
    ctx->has_scene = false;
    cudaError_t e;
    static_assert(sizeof(WideNode) == 5 * sizeof(uint4), "node size");
    if ((e = upload_with_capacity(ctx->nodes, reinterpret_cast<const uint4 *>(hs.nodes.data()), hs.nodes.size() * 5,
                                  node_capacity * 5, ctx->stream)) != cudaSuccess ||
        (e = upload(ctx->tris, hs.tris.data(), hs.tris.size(), ctx->stream)) != cudaSuccess ||
        (e = upload(ctx->tlas_items, hs.tlas_items.data(), hs.tlas_items.size(), ctx->stream)) != cudaSuccess ||
        (e = upload(ctx->instances, hs.insts.data(), hs.insts.size(), ctx->stream)) != cudaSuccess ||
        (e = upload(ctx->verts, hs.verts.data(), hs.verts.size(), ctx->stream)) != cudaSuccess ||
        (e = upload(ctx->faces, hs.faces.data(), hs.faces.size(), ctx->stream)) != cudaSuccess ||
        (e = upload(ctx->materials, hs.mats.data(), hs.mats.size(), ctx->stream)) != cudaSuccess ||
        (e = upload(ctx->sky, hs.cube.data(), hs.cube.size(), ctx->stream)) != cudaSuccess ||
        (e = upload(ctx->lights, hs.lights.data(), hs.lights.size(), ctx->stream)) != cudaSuccess ||
        (e = upload(ctx->light_cdf, hs.light_cdf.data(), hs.light_cdf.size(), ctx->stream)) != cudaSuccess ||
        (e = upload(ctx->scene_descs, descs.data(), descs.size(), ctx->stream)) != cudaSuccess ||
        (e = upload(ctx->textures, hs.textures.data(), hs.textures.size(), ctx->stream)) != cudaSuccess ||
        (e = upload(ctx->texels, hs.texels.data(), hs.texels.size(), ctx->stream)) != cudaSuccess) {
        return cuda_fail(ctx, e, "scene upload");
    }
    DevScene &S = ctx->scene;
    S.nodes = ctx->nodes.ptr;
    S.tris = ctx->tris.ptr;
    S.tlas_items = ctx->tlas_items.ptr;
    S.instances = ctx->instances.ptr;
    S.verts = ctx->verts.ptr;
    S.faces = ctx->faces.ptr;
    S.materials = ctx->materials.ptr;
    S.sky_cube = ctx->sky.ptr;
    S.scene_abs_x = hs.abs_x;
    S.lights = ctx->lights.ptr;
    S.light_cdf = ctx->light_cdf.ptr;
    S.descs = ctx->scene_descs.ptr;
    S.textures = ctx->textures.ptr;
    S.texels = ctx->texels.ptr;
    S.num_scenes = static_cast<uint32_t>(descs.size());
    for (int a = 0; a < 3; ++a) {
        const bool ok = hs.hi[a] > hs.lo[a];
        S.box_lo[a] = ok ? hs.lo[a] : 0.f;
        S.box_scale[a] = ok ? 8.f / (hs.hi[a] - hs.lo[a]) : 0.f;
    }
    const DevScene v = scene_view(S, descs[0]);
    S.tlas_root = v.tlas_root;
    S.sky_mode = v.sky_mode;
    S.sky_size = v.sky_size;
    for (int c = 0; c < 3; ++c) S.sky_color[c] = v.sky_color[c];
    S.num_lights = v.num_lights;
    S.light_total = v.light_total;
    ctx->bvh_nodes = static_cast<uint32_t>(hs.nodes.size());
    ctx->bvh_bytes = hs.nodes.size() * sizeof(WideNode) + hs.tris.size() * sizeof(float4);
    ctx->has_scene = true;
    ctx->dirty = true;
    return SPK_OK;
}

// SceneRenderProxy::UpdateBVH's `tlas_ = std::make_unique<TLAS>(primitives_); tlas_->Build()`
// (SceneRenderProxy.cpp:292-296) for a single-scene context whose BLASes are resident: rebuilds the instance
// records, the TLAS and the emissive-triangle light table on the host from the kept instance list and mesh
// positions, and uploads them (the TLAS into the nodes behind the BLASes).
spk_status rebuild_top(spk_ctx *ctx) {
    DynScene &dy = ctx->dyn;
    const uint32_t n = static_cast<uint32_t>(dy.instances.size());
    std::vector<BuildBox> boxes;
    float abs_x = 0.f;
    float lo[3] = {std::numeric_limits<float>::max(), std::numeric_limits<float>::max(),
                   std::numeric_limits<float>::max()};
    float hi[3] = {-lo[0], -lo[1], -lo[2]};
    instance_records(dy.instances.data(), n, dy.blas, dy.mats, dy.insts, boxes, abs_x, lo, hi);
    std::vector<WideNode> tlas;
    std::vector<uint32_t> items;
    if (n > 0) {
        const WideBvh wide = build_wide(boxes, ctx->tuning, host_threads());
        for (WideNode w : wide.nodes) {
            w.child_base += dy.tlas_root;
            tlas.push_back(w);
        }
        items = wide.items;
    }
    std::vector<spk_mesh> views(dy.positions.size());
    for (size_t m = 0; m < views.size(); ++m) {
        views[m] = spk_mesh{};
        views[m].positions = dy.positions[m].data();
        views[m].indices = dy.indices[m].data();
        views[m].num_vertices = static_cast<uint32_t>(dy.positions[m].size() / 3);
        views[m].num_faces = static_cast<uint32_t>(dy.indices[m].size() / 3);
    }
    std::vector<DevLight> lights;
    std::vector<float> cdf;
    float total = 0.f;
    light_table(dy.instances.data(), n, views.data(), dy.mats, dy.insts, lights, cdf, total);

    cudaError_t e;
    const size_t need = static_cast<size_t>(dy.tlas_root) + tlas.size();
    if (need > dy.node_capacity) {  // grow: keep the BLAS nodes, double the TLAS room
        const size_t cap = static_cast<size_t>(dy.tlas_root) + 2 * std::max<size_t>(tlas.size(), 1);
        DevBuf<uint4> grown;
        if ((e = cudaMalloc(&grown.ptr, cap * 5 * sizeof(uint4))) != cudaSuccess) return cuda_fail(ctx, e, "TLAS nodes");
        grown.count = cap * 5;
        if (dy.tlas_root &&
            (e = cudaMemcpyAsync(grown.ptr, ctx->nodes.ptr, dy.tlas_root * 5ull * sizeof(uint4), cudaMemcpyDeviceToDevice,
                                 ctx->stream)) != cudaSuccess) {
            grown.reset();
            return cuda_fail(ctx, e, "TLAS nodes");
        }
        cudaStreamSynchronize(ctx->stream);
        ctx->nodes.reset();
        ctx->nodes = grown;
        dy.node_capacity = static_cast<uint32_t>(cap);
    }
    dy.desc.tlas_root = n > 0 ? dy.tlas_root : kInvalid;
    dy.desc.num_lights = static_cast<uint32_t>(lights.size());
    dy.desc.light_total = total;
    if ((!tlas.empty() && (e = cudaMemcpyAsync(ctx->nodes.ptr + 5ull * dy.tlas_root, tlas.data(),
                                               tlas.size() * sizeof(WideNode), cudaMemcpyHostToDevice, ctx->stream)) !=
                              cudaSuccess) ||
        (e = upload(ctx->tlas_items, items.data(), items.size(), ctx->stream)) != cudaSuccess ||
        (e = upload(ctx->instances, dy.insts.data(), dy.insts.size(), ctx->stream)) != cudaSuccess ||
        (e = upload(ctx->lights, lights.data(), lights.size(), ctx->stream)) != cudaSuccess ||
        (e = upload(ctx->light_cdf, cdf.data(), cdf.size(), ctx->stream)) != cudaSuccess ||
        (e = upload(ctx->scene_descs, &dy.desc, 1, ctx->stream)) != cudaSuccess) {
        ctx->has_scene = false;
        return cuda_fail(ctx, e, "scene update");
    }
    DevScene &S = ctx->scene;
    S.nodes = ctx->nodes.ptr;
    S.tlas_items = ctx->tlas_items.ptr;
    S.instances = ctx->instances.ptr;
    S.lights = ctx->lights.ptr;
    S.light_cdf = ctx->light_cdf.ptr;
    S.descs = ctx->scene_descs.ptr;
    S.tlas_root = dy.desc.tlas_root;
    S.num_lights = dy.desc.num_lights;
    S.light_total = total;
    S.scene_abs_x = abs_x;
    for (int a = 0; a < 3; ++a) {
        const bool ok = hi[a] > lo[a];
        S.box_lo[a] = ok ? lo[a] : 0.f;
        S.box_scale[a] = ok ? 8.f / (hi[a] - lo[a]) : 0.f;
    }
    ctx->bvh_nodes = static_cast<uint32_t>(need);
    ctx->dirty = true;  // any primitive change clears the accumulation (SceneRenderProxy.cpp:198-202)
    return SPK_OK;
}

spk_status require_dynamic(spk_ctx *ctx) {
    if (!ctx) return SPK_ERR_INVALID_ARGUMENT;
    if (!ctx->has_scene || !ctx->dyn.valid)
        return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "incremental updates need a scene set by spk_set_scene");
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    return SPK_OK;
}

}  // namespace

extern "C" {

uint32_t spk_abi_version(void) { return SPK_ABI_VERSION; }

spk_status spk_create(int32_t device, spk_ctx **out_ctx) {
    if (!out_ctx) return SPK_ERR_INVALID_ARGUMENT;
    *out_ctx = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return SPK_ERR_CUDA;
    if (device < 0 || device >= count) return SPK_ERR_INVALID_ARGUMENT;
    auto *ctx = new (std::nothrow) spk_ctx();
    if (!ctx) return SPK_ERR_OUT_OF_MEMORY;
    ctx->device = device;
    if ((e = cudaSetDevice(device)) != cudaSuccess ||
        (e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreate(&ctx->ev_start)) != cudaSuccess || (e = cudaEventCreate(&ctx->ev_stop)) != cudaSuccess ||
        (e = cudaMalloc(&ctx->counters, sizeof(Counters))) != cudaSuccess ||
        (e = cudaMemset(ctx->counters, 0, sizeof(Counters))) != cudaSuccess) {
        spk_destroy(ctx);
        return SPK_ERR_CUDA;
    }
    *out_ctx = ctx;
    return SPK_OK;
}

spk_status spk_destroy(spk_ctx *ctx) {
    if (!ctx) return SPK_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    ctx->nodes.reset();
    ctx->tris.reset();
    ctx->tlas_items.reset();
    ctx->instances.reset();
    ctx->verts.reset();
    ctx->faces.reset();
    ctx->materials.reset();
    ctx->sky.reset();
    ctx->lights.reset();
    ctx->light_cdf.reset();
    ctx->scene_descs.reset();
    ctx->textures.reset();
    ctx->texels.reset();
    ctx->gcolor.reset();
    ctx->gnormal.reset();
    ctx->guide_nd.reset();
    ctx->guide_albedo.reset();
    ctx->rgba8_tables.reset();
    ctx->rgba8.reset();
    ctx->fb_half.reset();
    ctx->fb.reset();
    ctx->out.reset();
    wavefront_free(ctx->wf);
    wavefront_free(ctx->wf_batch);
    ctx->batch_reqs.reset();
    ctx->batch_hdr.reset();
    ctx->batch_img.reset();
    chunk_graph_free(ctx->chunk_graph);
    if (ctx->counters) cudaFree(ctx->counters);
    for (cudaEvent_t ev : ctx->event_pool) cudaEventDestroy(ev);
    if (ctx->ev_start) cudaEventDestroy(ctx->ev_start);
    if (ctx->ev_stop) cudaEventDestroy(ctx->ev_stop);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return SPK_OK;
}

const char *spk_last_error(const spk_ctx *ctx) { return ctx ? ctx->error.c_str() : "null context"; }

spk_status spk_set_scene(spk_ctx *ctx, const spk_mesh *meshes, uint32_t num_meshes, const spk_instance *instances,
                         uint32_t num_instances, const spk_material *materials, uint32_t num_materials,
                         const spk_sky *sky) try {
    if (!ctx) return SPK_ERR_INVALID_ARGUMENT;
    const spk_scene_desc d{meshes, num_meshes, instances, num_instances, materials, num_materials, sky,
                           nullptr, 0, nullptr};
    return spk_set_scenes(ctx, &d, 1);
} catch (const std::bad_alloc &) {
    return fail(ctx, SPK_ERR_OUT_OF_MEMORY, "host memory exhausted");
} catch (const std::exception &ex) {
    return fail(ctx, SPK_ERR_INTERNAL, "%s", ex.what());
}

spk_status spk_set_scenes(spk_ctx *ctx, const spk_scene_desc *scenes, uint32_t num_scenes) try {
    NvtxRange range("spk_set_scenes");
    if (!ctx) return SPK_ERR_INVALID_ARGUMENT;
    if (!scenes || num_scenes == 0) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "no scenes");
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    ctx->dyn = DynScene{};
    ctx->blas_reused = 0;
    HostScene all;
    std::vector<DevSceneDesc> descs(num_scenes);
    for (uint32_t k = 0; k < num_scenes; ++k) {
        const spk_scene_desc &d = scenes[k];
        HostScene hs;
        const spk_status st = build_host_scene(ctx, d.meshes, d.num_meshes, d.instances, d.num_instances,
                                               d.materials, d.num_materials, d.sky, d.textures, d.num_textures,
                                               d.maps, hs);
        if (st != SPK_OK) {
            if (num_scenes > 1) ctx->error = "scene " + std::to_string(k) + ": " + ctx->error;
            return st;
        }
        if (num_scenes == 1) {
            descs[0] = DevSceneDesc{hs.tlas_root, hs.sky_mode, hs.sky_size, {hs.sky_color[0], hs.sky_color[1],
                                    hs.sky_color[2]}, 0u, 0u, static_cast<uint32_t>(hs.lights.size()), hs.light_total};
            // A wide TLAS over n instances has at most max(1, n) nodes: reserve that much behind the BLASes.
            const uint32_t blas_nodes = hs.tlas_root == kInvalid ? static_cast<uint32_t>(hs.nodes.size()) : hs.tlas_root;
            const size_t capacity = static_cast<size_t>(blas_nodes) +
                                    std::max<size_t>(hs.nodes.size() - blas_nodes, std::max(1u, d.num_instances));
            const spk_status up = upload_scene(ctx, hs, descs, capacity);
            if (up != SPK_OK) return up;
            DynScene &dy = ctx->dyn;
            dy.instances.assign(d.instances, d.instances + d.num_instances);
            dy.positions.resize(d.num_meshes);
            dy.indices.resize(d.num_meshes);
            for (uint32_t m = 0; m < d.num_meshes; ++m) {
                const spk_mesh &mesh = d.meshes[m];
                const size_t np = mesh.positions ? 3ull * mesh.num_vertices : 0;
                const size_t nx = mesh.indices ? 3ull * mesh.num_faces : 0;
                dy.positions[m].resize(np);
                dy.indices[m].resize(nx);
                parallel_for(np, [&](uint64_t lo, uint64_t hi) {
                    std::memcpy(dy.positions[m].data() + lo, mesh.positions + lo, (hi - lo) * sizeof(float));
                });
                parallel_for(nx, [&](uint64_t lo, uint64_t hi) {
                    std::memcpy(dy.indices[m].data() + lo, mesh.indices + lo, (hi - lo) * sizeof(uint32_t));
                });
            }
            dy.blas = std::move(hs.blas);
            dy.mats = std::move(hs.mats);
            dy.insts = std::move(hs.insts);
            dy.desc = descs[0];
            dy.tlas_root = blas_nodes;
            dy.built_with = ctx->tuning;
            dy.node_capacity = static_cast<uint32_t>(capacity);
            dy.valid = true;
            return SPK_OK;
        }
        append_scene(all, hs, descs[k]);
    }
    return upload_scene(ctx, all, descs);
} catch (const std::bad_alloc &) {
    return fail(ctx, SPK_ERR_OUT_OF_MEMORY, "host memory exhausted");
} catch (const std::exception &ex) {
    return fail(ctx, SPK_ERR_INTERNAL, "%s", ex.what());
}

spk_status spk_set_instances(spk_ctx *ctx, const spk_instance *instances, uint32_t num_instances) try {
    NvtxRange range("spk_set_instances");
    spk_status st = require_dynamic(ctx);
    if (st != SPK_OK) return st;
    if (num_instances && !instances) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "null instance array");
    DynScene &dy = ctx->dyn;
    for (uint32_t k = 0; k < num_instances; ++k) {
        const spk_instance &in = instances[k];
        if (in.type != SPK_PRIM_MESH && in.type != SPK_PRIM_SPHERE)
            return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "instance %u: bad type", k);
        if (in.type == SPK_PRIM_MESH && in.mesh_id >= dy.blas.size())
            return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "instance %u: mesh_id out of range", k);
        if (in.material_id >= dy.mats.size())
            return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "instance %u: material_id out of range", k);
    }
    dy.instances.assign(instances, instances + num_instances);
    return rebuild_top(ctx);
} catch (const std::bad_alloc &) {
    return fail(ctx, SPK_ERR_OUT_OF_MEMORY, "host memory exhausted");
} catch (const std::exception &ex) {
    return fail(ctx, SPK_ERR_INTERNAL, "%s", ex.what());
}

spk_status spk_set_instance_transforms(spk_ctx *ctx, uint32_t first, uint32_t count, const float *transforms,
                                       const float *inv_transforms) try {
    NvtxRange range("spk_set_instance_transforms");
    spk_status st = require_dynamic(ctx);
    if (st != SPK_OK) return st;
    DynScene &dy = ctx->dyn;
    if (count && (!transforms || !inv_transforms)) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "null transforms");
    if (static_cast<uint64_t>(first) + count > dy.instances.size())
        return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "instances %u..%u out of range (%zu instances)", first,
                    first + count, dy.instances.size());
    for (uint32_t k = 0; k < count; ++k) {
        std::memcpy(dy.instances[first + k].transform, transforms + 12ull * k, 12 * sizeof(float));
        std::memcpy(dy.instances[first + k].inv_transform, inv_transforms + 12ull * k, 12 * sizeof(float));
    }
    return rebuild_top(ctx);
} catch (const std::bad_alloc &) {
    return fail(ctx, SPK_ERR_OUT_OF_MEMORY, "host memory exhausted");
} catch (const std::exception &ex) {
    return fail(ctx, SPK_ERR_INTERNAL, "%s", ex.what());
}

spk_status spk_update_mesh(spk_ctx *ctx, uint32_t mesh_id, uint32_t num_vertices, const float *positions,
                           const float *normals, const float *tangents) try {
    NvtxRange range("spk_update_mesh");
    spk_status st = require_dynamic(ctx);
    if (st != SPK_OK) return st;
    DynScene &dy = ctx->dyn;
    if (mesh_id >= dy.blas.size()) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "mesh_id %u out of range", mesh_id);
    std::vector<float> &pos = dy.positions[mesh_id];
    if (num_vertices != pos.size() / 3)
        return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "mesh %u: %u vertices given, the mesh has %zu", mesh_id,
                    num_vertices, pos.size() / 3);
    if (num_vertices && !positions) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "null positions");
    const MeshBlas &b = dy.blas[mesh_id];
    const uint32_t num_faces = static_cast<uint32_t>(dy.indices[mesh_id].size() / 3);
    cudaError_t e;
    const size_t nv3 = 3ull * num_vertices;
    // The host copy (bounds, light table) and the device copy (refit) of the new positions.
    if (nv3 && (e = cudaMemcpy(pos.data(), positions, nv3 * sizeof(float), cudaMemcpyDefault)) != cudaSuccess)
        return cuda_fail(ctx, e, "positions");
    if (ctx->dyn_pos.count < nv3 && (e = alloc(ctx->dyn_pos, nv3)) != cudaSuccess) return cuda_fail(ctx, e, "positions");
    if (nv3 && (e = cudaMemcpyAsync(ctx->dyn_pos.ptr, pos.data(), nv3 * sizeof(float), cudaMemcpyHostToDevice,
                                    ctx->stream)) != cudaSuccess)
        return cuda_fail(ctx, e, "positions");
    if (normals || tangents) {
        const size_t na = (normals ? nv3 : 0) + (tangents ? 4ull * num_vertices : 0);
        if (ctx->dyn_attr.count < na && (e = alloc(ctx->dyn_attr, na)) != cudaSuccess)
            return cuda_fail(ctx, e, "vertex attributes");
        float *dn = normals ? ctx->dyn_attr.ptr : nullptr;
        float *dt = tangents ? ctx->dyn_attr.ptr + (normals ? nv3 : 0) : nullptr;
        if ((normals && (e = cudaMemcpyAsync(dn, normals, nv3 * sizeof(float), cudaMemcpyDefault, ctx->stream)) !=
                            cudaSuccess) ||
            (tangents && (e = cudaMemcpyAsync(dt, tangents, 4ull * num_vertices * sizeof(float), cudaMemcpyDefault,
                                              ctx->stream)) != cudaSuccess) ||
            (e = launch_update_vertices(ctx->verts.ptr, b.vert_base, num_vertices, dn, dt, ctx->stream)) != cudaSuccess)
            return cuda_fail(ctx, e, "vertex attributes");
    }
    if (b.root != kInvalid) {
        if (ctx->dyn_boxes.count < 6ull * b.node_count && (e = alloc(ctx->dyn_boxes, 6ull * b.node_count)) != cudaSuccess)
            return cuda_fail(ctx, e, "refit scratch");
        BlasRefit r{};
        r.nodes = ctx->nodes.ptr;
        r.boxes = ctx->dyn_boxes.ptr;
        r.tris = ctx->tris.ptr;
        r.faces = ctx->faces.ptr + b.face_base;
        r.positions = ctx->dyn_pos.ptr;
        r.root = b.root;
        r.node_count = b.node_count;
        r.tri_first = b.tri_first;
        r.tri_count = b.tri_count;
        r.num_faces = num_faces;
        r.num_vertices = num_vertices;
        if ((e = launch_refit_triangles(r, ctx->stream)) != cudaSuccess) return cuda_fail(ctx, e, "refit");
        for (size_t l = b.levels.size() - 1; l-- > 0;)
            if ((e = launch_refit_nodes(r, b.levels[l], b.levels[l + 1], ctx->stream)) != cudaSuccess)
                return cuda_fail(ctx, e, "refit");
    }
    // The mesh's local box over its faces' vertices, as the BLAS build takes it.
    MeshBlas &mb = dy.blas[mesh_id];
    for (int a = 0; a < 3; ++a) {
        mb.bounds[a] = std::numeric_limits<double>::max();
        mb.bounds[3 + a] = -std::numeric_limits<double>::max();
    }
    for (uint32_t i : dy.indices[mesh_id])
        for (int a = 0; a < 3; ++a) {
            mb.bounds[a] = std::min(mb.bounds[a], static_cast<double>(pos[3ull * i + a]));
            mb.bounds[3 + a] = std::max(mb.bounds[3 + a], static_cast<double>(pos[3ull * i + a]));
        }
    st = rebuild_top(ctx);
    if (st != SPK_OK) return st;
    if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return cuda_fail(ctx, e, "refit");
    return SPK_OK;
} catch (const std::bad_alloc &) {
    return fail(ctx, SPK_ERR_OUT_OF_MEMORY, "host memory exhausted");
} catch (const std::exception &ex) {
    return fail(ctx, SPK_ERR_INTERNAL, "%s", ex.what());
}

spk_status spk_read_bvh_nodes(spk_ctx *ctx, void *nodes, uint64_t capacity, uint64_t *count) try {
    if (!ctx || !count) return SPK_ERR_INVALID_ARGUMENT;
    if (!ctx->has_scene) return fail(ctx, SPK_ERR_NOT_READY, "no scene");
    *count = ctx->bvh_nodes;
    if (!nodes) return SPK_OK;
    const uint64_t n = std::min<uint64_t>(capacity, ctx->bvh_nodes);
    cudaSetDevice(ctx->device);
    cudaError_t e = cudaMemcpyAsync(nodes, ctx->nodes.ptr, n * sizeof(WideNode), cudaMemcpyDefault, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? SPK_OK : cuda_fail(ctx, e, "read nodes");
} catch (const std::bad_alloc &) {
    return fail(ctx, SPK_ERR_OUT_OF_MEMORY, "host memory exhausted");
} catch (const std::exception &ex) {
    return fail(ctx, SPK_ERR_INTERNAL, "%s", ex.what());
}

spk_status spk_get_config(const spk_ctx *ctx, spk_config *out) {
    if (!ctx || !out) return SPK_ERR_INVALID_ARGUMENT;
    if (!ctx->has_config) return SPK_ERR_NOT_READY;
    *out = ctx->cfg;
    return SPK_OK;
}

spk_status spk_set_camera(spk_ctx *ctx, const spk_camera *camera) {
    if (!ctx || !camera) return SPK_ERR_INVALID_ARGUMENT;
    static_assert(sizeof(DevCamera) == sizeof(spk_camera), "camera layout");
    std::memcpy(&ctx->cam, camera, sizeof(DevCamera));
    ctx->has_camera = true;
    ctx->dirty = true;
    return SPK_OK;
}

spk_status spk_camera_from_look(const float position[3], const float target[3], const float world_up[3],
                                float vertical_fov_rad, float focus_distance, float aperture_radius, float exposure,
                                uint32_t width, uint32_t height, spk_camera *out) {
    if (!position || !target || !world_up || !out || width == 0 || height == 0 || !(focus_distance > 0.f))
        return SPK_ERR_INVALID_ARGUMENT;
    double f[3], r[3], u[3];
    for (int k = 0; k < 3; ++k) f[k] = static_cast<double>(target[k]) - position[k];
    double n = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    if (!(n > 0)) return SPK_ERR_INVALID_ARGUMENT;
    for (double &x : f) x /= n;
    r[0] = f[1] * world_up[2] - f[2] * world_up[1];
    r[1] = f[2] * world_up[0] - f[0] * world_up[2];
    r[2] = f[0] * world_up[1] - f[1] * world_up[0];
    n = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    if (!(n > 0)) return SPK_ERR_INVALID_ARGUMENT;
    for (double &x : r) x /= n;
    u[0] = r[1] * f[2] - r[2] * f[1];
    u[1] = r[2] * f[0] - r[0] * f[2];
    u[2] = r[0] * f[1] - r[1] * f[0];
    spk_camera c{};
    for (int k = 0; k < 3; ++k) {
        c.position[k] = position[k];
        c.front[k] = static_cast<float>(f[k]);
        c.right[k] = static_cast<float>(r[k]);
        c.up[k] = static_cast<float>(u[k]);
    }
    // CameraRenderProxy::Update: h = tan(fov / 2); height = 2 h focus; width = aspect * height.
    const volatile float h = std::tan(vertical_fov_rad / 2.f);
    const volatile float fh = 2.f * h * focus_distance;
    const volatile float aspect = static_cast<float>(width) / static_cast<float>(height);
    const volatile float fw = aspect * fh;
    for (int k = 0; k < 3; ++k) {
        c.max_u[k] = c.right[k] * fw;
        c.max_v[k] = c.up[k] * fh;
        const volatile float a = c.position[k] + c.front[k] * focus_distance;
        const volatile float b = a - c.max_u[k] * .5f;
        c.lower_left[k] = b - c.max_v[k] * .5f;
    }
    c.aperture_radius = aperture_radius;
    c.exposure = exposure;
    c.far_plane = 1000.f;
    *out = c;
    return SPK_OK;
}

spk_status spk_set_config(spk_ctx *ctx, const spk_config *config) try {
    if (!ctx || !config) return SPK_ERR_INVALID_ARGUMENT;
    if (config->width < 2 || config->height < 2)
        return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "resolution must be at least 2x2");
    if (static_cast<uint64_t>(config->width) * config->height > (1ull << 31))
        return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "resolution too large");
    if (config->rng > SPK_RNG_XOSHIRO256SS) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "unknown rng policy");
    if (config->debug_mode != SPK_DEBUG_COLOR) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "only debug_mode 0 (color)");
    if (config->kernel > SPK_KERNEL_WAVEFRONT) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "unknown kernel schedule");
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    const size_t n = static_cast<size_t>(config->width) * config->height;
    cudaError_t e;
    if ((e = alloc(ctx->gcolor, n)) != cudaSuccess || (e = alloc(ctx->gnormal, n)) != cudaSuccess ||
        (e = alloc(ctx->fb, n)) != cudaSuccess || (e = alloc(ctx->out, n)) != cudaSuccess) {
        ctx->has_config = false;
        return cuda_fail(ctx, e, "frame buffer allocation");
    }
    if ((e = cudaMemsetAsync(ctx->gnormal.ptr, 0, n * sizeof(float4), ctx->stream)) != cudaSuccess ||
        (e = cudaMemsetAsync(ctx->fb.ptr, 0, n * sizeof(float4), ctx->stream)) != cudaSuccess) {
        return cuda_fail(ctx, e, "frame buffer clear");
    }
    if (ctx->wf.capacity < n && (e = wavefront_alloc(ctx->wf, static_cast<uint32_t>(n))) != cudaSuccess) {
        ctx->has_config = false;
        return cuda_fail(ctx, e, "path state allocation");
    }
    ctx->cfg = *config;
    // sub_pixel_count_ = lround(sqrt(float(spp))); actual spp = its square (CPURenderer.cpp:102-104)
    const auto sub = static_cast<unsigned>(std::lround(std::sqrt(static_cast<float>(config->spp))));
    ctx->spp_eff = sub * sub;
    ctx->has_config = true;
    ctx->dirty = true;
    return SPK_OK;
} catch (const std::bad_alloc &) {
    return fail(ctx, SPK_ERR_OUT_OF_MEMORY, "host memory exhausted");
} catch (const std::exception &ex) {
    return fail(ctx, SPK_ERR_INTERNAL, "%s", ex.what());
}

static WfTuning wf_tuning(const spk_ctx *ctx) {
    WfTuning t;
    t.extend_blocks_per_sm = ctx->tuning.extend_blocks_per_sm;
    t.shade_blocks_per_sm = ctx->tuning.shade_blocks_per_sm;
    t.material_sort = ctx->tuning.material_sort != 0;
    t.ray_sort = ctx->tuning.ray_sort != 0;
    t.slots_per_pixel = ctx->tuning.path_slots_per_pixel;
    t.shadow_stage = ctx->tuning.shadow_stage != 0;
    t.packets = ctx->tuning.primary_packets;
    return t;
}

static spk_status render_impl(spk_ctx *ctx, uint32_t num_frames) {
    FrameBuffers fbuf{ctx->gcolor.ptr, ctx->gnormal.ptr, ctx->fb.ptr, ctx->out.ptr, ctx->cfg.width, ctx->cfg.height};
    cudaError_t e;
    const bool wavefront = ctx->cfg.kernel != SPK_KERNEL_MEGAKERNEL;
    const bool count = (ctx->instrumentation & SPK_INSTR_COUNT_TRAFFIC) != 0;
    const size_t launches_per_frame = wavefront ? ctx->cfg.bounce : 1;
    if ((e = prepare_events(ctx, static_cast<size_t>(num_frames) * launches_per_frame + 16)) != cudaSuccess)
        return cuda_fail(ctx, e, "event pool");
    if (ctx->accum_target) {
        // The last frames went into a caller's buffer (spk_render_noalloc): fb holds none of them, so the
        // accumulation starts over here.
        ctx->dirty = true;
        ctx->accum_target = nullptr;
    }
    ctx->noalloc_counters = nullptr;
    ctx->launches_in_call = 0;
    if ((e = cudaMemsetAsync(ctx->counters, 0, sizeof(Counters), ctx->stream)) != cudaSuccess)
        return cuda_fail(ctx, e, "counter reset");
    if ((e = cudaEventRecord(ctx->ev_start, ctx->stream)) != cudaSuccess) return cuda_fail(ctx, e, "event");
    if (wavefront && ctx->tuning.multi_frame && num_frames > 0) {
        // All frames in one regenerating wavefront: run the per-frame bookkeeping ahead on the host and hand
        // the kernels each frame's weight and seed base (the spatial fill, when on, runs per frame in the
        // resolve over that frame's samples and first-hit normals).
        ctx->frame_weights.resize(num_frames);
        ctx->frame_seeds.resize(num_frames);
        bool clear = false;
        for (uint32_t f = 0; f < num_frames; ++f) {
            if (ctx->dirty) {
                ctx->cumulated = 0;
                ctx->pending = 0;
            }
            ctx->cumulated = std::min(ctx->cfg.max_spp, ctx->cumulated + ctx->pending);
            ctx->pending = 0;
            if (ctx->dirty) {
                clear = true;
                ctx->dirty = false;
                ctx->dispatched = ctx->cfg.sample_offset;
            }
            ctx->frame_seeds[f] = ctx->dispatched;
            ctx->frame_weights[f] =
                static_cast<float>(ctx->cumulated) / static_cast<float>(ctx->cumulated + ctx->spp_eff);
            ctx->dispatched += ctx->spp_eff;
            ctx->pending += ctx->spp_eff;
        }
        if (clear &&
            (e = cudaMemsetAsync(ctx->fb.ptr, 0, ctx->fb.count * sizeof(float4), ctx->stream)) != cudaSuccess)
            return cuda_fail(ctx, e, "frame buffer clear");
        RenderParams p{0u, ctx->cfg.bounce, ctx->cfg.rng, ctx->cfg.seed, ctx->cfg.spatial_denoise, ctx->cfg.enable_nee};
        uint32_t launches = 0;
        ctx->chunk_graph.enabled = ctx->tuning.cuda_graph != 0;
        const uint32_t replays0 = ctx->chunk_graph.replays;
        // Path slots for the multi-frame schedule: pixels x path_slots_per_pixel, no more than the frames of
        // one pass can use and at most kMaxPathSlots (about 20 GB of path state); grown on demand and kept.
        const uint64_t npix = static_cast<uint64_t>(ctx->cfg.width) * ctx->cfg.height;
        const uint64_t per_pixel = std::min<uint64_t>({ctx->tuning.path_slots_per_pixel, num_frames, kFramesPerPass});
        const uint64_t slots = std::max<uint64_t>(npix, std::min<uint64_t>(npix * per_pixel, kMaxPathSlots));
        if (ctx->wf.capacity < slots && (e = wavefront_alloc(ctx->wf, static_cast<uint32_t>(slots))) != cudaSuccess)
            return cuda_fail(ctx, e, "path state allocation");
        e = launch_render_multiframe(ctx->scene, ctx->cam, fbuf, p, num_frames, ctx->frame_weights.data(),
                                     ctx->frame_seeds.data(), count, ctx->counters, ctx->wf, ctx->num_sms,
                                     ctx->stream, &launches, &ctx->launch_events, wf_tuning(ctx), &ctx->chunk_graph);
        if (e != cudaSuccess) {
            const std::string what = std::string("multi-frame wavefront (") + wavefront_error_site() + ")";
            return cuda_fail(ctx, e, what.c_str());
        }
        ctx->launches_in_call = launches;
        if ((e = cudaEventRecord(ctx->ev_stop, ctx->stream)) != cudaSuccess) return cuda_fail(ctx, e, "event");
        ctx->last = spk_stats{};
        ctx->last.paths = static_cast<uint64_t>(num_frames) * ctx->cfg.width * ctx->cfg.height;
        ctx->last.graph_replays = ctx->chunk_graph.replays - replays0;
        ctx->stats_pending = true;
        return SPK_OK;
    }
    for (uint32_t f = 0; f < num_frames; ++f) {
        // CameraRenderProxy::Update (CameraRenderProxy.cpp:66-75)
        if (ctx->dirty) {
            ctx->cumulated = 0;
            ctx->pending = 0;
        }
        ctx->cumulated = std::min(ctx->cfg.max_spp, ctx->cumulated + ctx->pending);
        ctx->pending = 0;
        // CPURenderer::Render: clear on dirty (CPURenderer.cpp:128-137)
        if (ctx->dirty) {
            if ((e = cudaMemsetAsync(ctx->fb.ptr, 0, ctx->fb.count * sizeof(float4), ctx->stream)) != cudaSuccess)
                return cuda_fail(ctx, e, "frame buffer clear");
            ctx->dirty = false;
            ctx->dispatched = ctx->cfg.sample_offset;
        }
        RenderParams p{ctx->dispatched, ctx->cfg.bounce, ctx->cfg.rng, ctx->cfg.seed, ctx->cfg.spatial_denoise,
                       ctx->cfg.enable_nee};
        uint32_t launches = 0;
        if (wavefront) {
            e = launch_render_wavefront(ctx->scene, ctx->cam, fbuf, p, count, ctx->counters, ctx->wf, ctx->num_sms,
                                        ctx->stream, &launches, &ctx->launch_events, wf_tuning(ctx));
        } else {
            e = launch_render_mega(ctx->scene, ctx->cam, fbuf, p, count, ctx->counters, ctx->stream,
                                   &ctx->launch_events);
            launches = 1;
        }
        if (e != cudaSuccess) return cuda_fail(ctx, e, "base pass launch");
        ctx->launches_in_call += launches;
        // DenoisePass weight: cumulated / (cumulated + actual spp) (CPURenderer.cpp:530-532)
        const float mavg = static_cast<float>(ctx->cumulated) / static_cast<float>(ctx->cumulated + ctx->spp_eff);
        if ((e = launch_resolve(fbuf, mavg, ctx->cam.exposure, ctx->cfg.spatial_denoise, ctx->stream)) != cudaSuccess)
            return cuda_fail(ctx, e, "resolve launch");
        ctx->launches_in_call += 1;
        ctx->dispatched += ctx->spp_eff;
        ctx->pending += ctx->spp_eff;
    }
    if ((e = cudaEventRecord(ctx->ev_stop, ctx->stream)) != cudaSuccess) return cuda_fail(ctx, e, "event");
    ctx->last = spk_stats{};
    ctx->last.paths = static_cast<uint64_t>(num_frames) * ctx->cfg.width * ctx->cfg.height;
    ctx->stats_pending = true;
    return SPK_OK;
}

spk_status spk_render(spk_ctx *ctx, uint32_t num_frames) try {
    NvtxRange range("spk_render");
    if (!ctx) return SPK_ERR_INVALID_ARGUMENT;
    if (!ctx->has_scene || !ctx->has_config || !ctx->has_camera)
        return fail(ctx, SPK_ERR_NOT_READY, "render needs spk_set_scene, spk_set_config and spk_set_camera first");
    cudaSetDevice(ctx->device);
    return render_impl(ctx, num_frames);
} catch (const std::bad_alloc &) {
    return fail(ctx, SPK_ERR_OUT_OF_MEMORY, "host memory exhausted");
} catch (const std::exception &ex) {
    return fail(ctx, SPK_ERR_INTERNAL, "%s", ex.what());
}

spk_status spk_read_framebuffer(spk_ctx *ctx, float *hdr_rgba, uint16_t *rgba16f) {
    if (!ctx) return SPK_ERR_INVALID_ARGUMENT;
    if (!ctx->has_config) return fail(ctx, SPK_ERR_NOT_READY, "no frame buffer");
    if (const spk_status st = require_own_buffers(ctx)) return st;
    cudaSetDevice(ctx->device);
    cudaError_t e;
    if (hdr_rgba &&
        (e = cudaMemcpyAsync(hdr_rgba, ctx->fb.ptr, ctx->fb.count * sizeof(float4), cudaMemcpyDefault,
                             ctx->stream)) != cudaSuccess)
        return cuda_fail(ctx, e, "frame buffer read");
    if (rgba16f &&
        (e = cudaMemcpyAsync(rgba16f, ctx->out.ptr, ctx->out.count * sizeof(ushort4), cudaMemcpyDefault,
                             ctx->stream)) != cudaSuccess)
        return cuda_fail(ctx, e, "output image read");
    if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return cuda_fail(ctx, e, "synchronize");
    return SPK_OK;
}

// Render checkpoint: a header (magic, version, the spk_config, the sample bookkeeping), then the frame
// buffer (width * height float4) and the output image (width * height half4).
namespace {
struct CheckpointHeader {
    char magic[8];
    uint32_t version;
    uint32_t reserved;
    spk_config config;
    uint32_t cumulated, pending, dispatched, dirty;
};
constexpr char kCheckpointMagic[8] = {'S', 'P', 'K', 'C', 'K', 'P', 'T', '1'};

uint64_t checkpoint_bytes(const spk_ctx *ctx) {
    const uint64_t n = static_cast<uint64_t>(ctx->cfg.width) * ctx->cfg.height;
    return sizeof(CheckpointHeader) + n * (sizeof(float4) + sizeof(ushort4));
}
}  // namespace

spk_status spk_checkpoint_size(const spk_ctx *ctx, uint64_t *bytes) {
    if (!ctx || !bytes) return SPK_ERR_INVALID_ARGUMENT;
    if (!ctx->has_config) return SPK_ERR_NOT_READY;
    *bytes = checkpoint_bytes(ctx);
    return SPK_OK;
}

spk_status spk_save_checkpoint(spk_ctx *ctx, void *buffer, uint64_t size) {
    if (!ctx || !buffer) return SPK_ERR_INVALID_ARGUMENT;
    if (!ctx->has_config) return fail(ctx, SPK_ERR_NOT_READY, "no frame buffer");
    if (size < checkpoint_bytes(ctx)) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "checkpoint buffer too small");
    if (const spk_status st = require_own_buffers(ctx)) return st;
    cudaSetDevice(ctx->device);
    CheckpointHeader h{};
    std::memcpy(h.magic, kCheckpointMagic, 8);
    h.version = 1;
    h.config = ctx->cfg;
    h.cumulated = ctx->cumulated;
    h.pending = ctx->pending;
    h.dispatched = ctx->dispatched;
    h.dirty = ctx->dirty ? 1u : 0u;
    auto *out = static_cast<uint8_t *>(buffer);
    std::memcpy(out, &h, sizeof(h));
    const uint64_t n = static_cast<uint64_t>(ctx->cfg.width) * ctx->cfg.height;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(out + sizeof(h), ctx->fb.ptr, n * sizeof(float4), cudaMemcpyDefault, ctx->stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(out + sizeof(h) + n * sizeof(float4), ctx->out.ptr, n * sizeof(ushort4), cudaMemcpyDefault,
                             ctx->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess)
        return cuda_fail(ctx, e, "checkpoint read");
    return SPK_OK;
}

spk_status spk_load_checkpoint(spk_ctx *ctx, const void *buffer, uint64_t size) {
    if (!ctx || !buffer) return SPK_ERR_INVALID_ARGUMENT;
    if (!ctx->has_config) return fail(ctx, SPK_ERR_NOT_READY, "set the checkpoint's config first");
    CheckpointHeader h{};
    if (size < sizeof(h)) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "checkpoint truncated");
    std::memcpy(&h, buffer, sizeof(h));
    if (std::memcmp(h.magic, kCheckpointMagic, 8) != 0 || h.version != 1)
        return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "not a render checkpoint of this version");
    if (std::memcmp(&h.config, &ctx->cfg, sizeof(spk_config)) != 0)
        return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "checkpoint config differs from the context's");
    if (size < checkpoint_bytes(ctx)) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "checkpoint truncated");
    cudaSetDevice(ctx->device);
    const uint64_t n = static_cast<uint64_t>(ctx->cfg.width) * ctx->cfg.height;
    const auto *in = static_cast<const uint8_t *>(buffer);
    cudaError_t e;
    if ((e = cudaMemcpyAsync(ctx->fb.ptr, in + sizeof(h), n * sizeof(float4), cudaMemcpyDefault, ctx->stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(ctx->out.ptr, in + sizeof(h) + n * sizeof(float4), n * sizeof(ushort4), cudaMemcpyDefault,
                             ctx->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess)
        return cuda_fail(ctx, e, "checkpoint write");
    ctx->cumulated = h.cumulated;
    ctx->pending = h.pending;
    ctx->dispatched = h.dispatched;
    ctx->dirty = h.dirty != 0;  // the accumulation continues from the saved state, not from a cleared one
    ctx->accum_target = nullptr;
    return SPK_OK;
}

// BVH blob: header {magic, version, mesh count, knobs[4]}, per mesh {faces, vertices, hash, node count,
// item count}, then per mesh its nodes (80 B, child and item bases relative to the mesh's BLAS) and items.
namespace {
struct BvhBlobHeader {
    char magic[8];
    uint32_t version, num_meshes;
    uint32_t knobs[4];
};
struct BvhBlobMesh {
    uint32_t num_faces, num_vertices;
    uint64_t hash;
    uint32_t node_count, item_count;
};
constexpr char kBvhMagic[8] = {'S', 'P', 'K', 'B', 'V', 'H', '0', '1'};
}  // namespace

spk_status spk_bvh_blob_size(spk_ctx *ctx, uint64_t *bytes) {
    if (!ctx || !bytes) return SPK_ERR_INVALID_ARGUMENT;
    if (!ctx->has_scene || !ctx->dyn.valid)
        return fail(ctx, SPK_ERR_NOT_READY, "BVH blobs are saved from a scene set by spk_set_scene");
    uint64_t n = sizeof(BvhBlobHeader);
    for (const MeshBlas &b : ctx->dyn.blas)
        n += sizeof(BvhBlobMesh) + static_cast<uint64_t>(b.node_count) * sizeof(WideNode) + 4ull * b.tri_count;
    *bytes = n;
    return SPK_OK;
}

spk_status spk_save_bvh(spk_ctx *ctx, void *blob, uint64_t size) try {
    uint64_t need = 0;
    spk_status st = spk_bvh_blob_size(ctx, &need);
    if (st != SPK_OK) return st;
    if (!blob || size < need) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "BVH blob buffer too small");
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    const DynScene &dy = ctx->dyn;
    auto *out = static_cast<uint8_t *>(blob);
    BvhBlobHeader h{};
    std::memcpy(h.magic, kBvhMagic, 8);
    h.version = 1;
    h.num_meshes = static_cast<uint32_t>(dy.blas.size());
    const uint32_t knobs[4] = {dy.built_with.bvh_width, dy.built_with.bvh_leaf_size, dy.built_with.bvh_collapse,
                               dy.built_with.bvh_builder};
    std::memcpy(h.knobs, knobs, sizeof(knobs));
    std::memcpy(out, &h, sizeof(h));
    uint8_t *meta = out + sizeof(h);
    uint8_t *data = meta + dy.blas.size() * sizeof(BvhBlobMesh);
    for (size_t k = 0; k < dy.blas.size(); ++k) {
        const MeshBlas &b = dy.blas[k];
        BvhBlobMesh mm{};
        mm.num_faces = static_cast<uint32_t>(dy.indices[k].size() / 3);
        mm.num_vertices = static_cast<uint32_t>(dy.positions[k].size() / 3);
        mm.hash = geometry_hash(dy.positions[k].data(), mm.num_vertices, dy.indices[k].data(), mm.num_faces);
        mm.node_count = b.root == kInvalid ? 0 : b.node_count;
        mm.item_count = b.root == kInvalid ? 0 : b.tri_count;
        std::memcpy(meta + k * sizeof(BvhBlobMesh), &mm, sizeof(mm));
        if (mm.node_count) {
            std::vector<WideNode> nodes(mm.node_count);
            std::vector<float4> tris(3ull * mm.item_count);
            cudaError_t e;
            if ((e = cudaMemcpy(nodes.data(), ctx->nodes.ptr + 5ull * b.root, nodes.size() * sizeof(WideNode),
                                cudaMemcpyDeviceToHost)) != cudaSuccess ||
                (e = cudaMemcpy(tris.data(), ctx->tris.ptr + 3ull * b.tri_first, tris.size() * sizeof(float4),
                                cudaMemcpyDeviceToHost)) != cudaSuccess)
                return cuda_fail(ctx, e, "BVH read");
            for (WideNode &w : nodes) {
                w.child_base -= b.root;
                w.item_base -= b.tri_first;
            }
            std::memcpy(data, nodes.data(), nodes.size() * sizeof(WideNode));
            data += nodes.size() * sizeof(WideNode);
            for (uint32_t i = 0; i < mm.item_count; ++i) {
                uint32_t face;
                std::memcpy(&face, &tris[3ull * i + 2].y, 4);
                std::memcpy(data + 4ull * i, &face, 4);
            }
            data += 4ull * mm.item_count;
        }
    }
    return SPK_OK;
} catch (const std::bad_alloc &) {
    return fail(ctx, SPK_ERR_OUT_OF_MEMORY, "host memory exhausted");
}

spk_status spk_set_bvh(spk_ctx *ctx, const void *blob, uint64_t size) try {
    if (!ctx) return SPK_ERR_INVALID_ARGUMENT;
    ctx->bvh_cache.clear();
    if (!blob || size == 0) return SPK_OK;
    const auto *in = static_cast<const uint8_t *>(blob);
    BvhBlobHeader h{};
    if (size < sizeof(h)) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "BVH blob truncated");
    std::memcpy(&h, in, sizeof(h));
    if (std::memcmp(h.magic, kBvhMagic, 8) != 0 || h.version != 1)
        return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "not a BVH blob of this version");
    uint64_t pos = sizeof(h) + static_cast<uint64_t>(h.num_meshes) * sizeof(BvhBlobMesh);
    if (pos > size) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "BVH blob truncated");
    std::vector<CachedBlas> cache(h.num_meshes);
    for (uint32_t k = 0; k < h.num_meshes; ++k) {
        BvhBlobMesh mm{};
        std::memcpy(&mm, in + sizeof(h) + k * sizeof(BvhBlobMesh), sizeof(mm));
        const uint64_t bytes = static_cast<uint64_t>(mm.node_count) * sizeof(WideNode) + 4ull * mm.item_count;
        if (pos + bytes > size || mm.item_count > mm.num_faces)
            return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "BVH blob: mesh %u does not fit", k);
        CachedBlas &c = cache[k];
        c.num_faces = mm.num_faces;
        c.num_vertices = mm.num_vertices;
        c.hash = mm.hash;
        c.bvh.nodes.resize(mm.node_count);
        c.bvh.items.resize(mm.item_count);
        std::memcpy(c.bvh.nodes.data(), in + pos, c.bvh.nodes.size() * sizeof(WideNode));
        std::memcpy(c.bvh.items.data(), in + pos + c.bvh.nodes.size() * sizeof(WideNode), 4ull * mm.item_count);
        for (const WideNode &w : c.bvh.nodes)  // every reference stays inside this BLAS
            if (w.child_base > mm.node_count || w.item_base > mm.item_count)
                return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "BVH blob: mesh %u has an out-of-range node", k);
        for (uint32_t f : c.bvh.items)
            if (f >= mm.num_faces) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "BVH blob: mesh %u has a bad item", k);
        pos += bytes;
    }
    std::memcpy(ctx->bvh_cache_knobs, h.knobs, sizeof(h.knobs));
    ctx->bvh_cache = std::move(cache);
    return SPK_OK;
} catch (const std::bad_alloc &) {
    return fail(ctx, SPK_ERR_OUT_OF_MEMORY, "host memory exhausted");
}

void spk_debug_fail_allocation(uint32_t nth) { fault_arm_allocation(nth); }

spk_status spk_debug_walk_budget(spk_ctx *ctx, uint32_t steps) {
    if (!ctx) return SPK_ERR_INVALID_ARGUMENT;
    ctx->scene.walk_budget = steps;
    return SPK_OK;
}

spk_status spk_read_rgba8(spk_ctx *ctx, uint8_t *rgba8) try {
    if (!ctx || !rgba8) return SPK_ERR_INVALID_ARGUMENT;
    if (!ctx->has_config) return fail(ctx, SPK_ERR_NOT_READY, "no frame buffer");
    if (const spk_status st = require_own_buffers(ctx)) return st;
    cudaSetDevice(ctx->device);
    cudaError_t e;
    if (!ctx->rgba8_tables.ptr) {
        std::vector<uint8_t> tab(2 * 65536);
        std::memcpy(tab.data(), rgba8_table(true), 65536);
        std::memcpy(tab.data() + 65536, rgba8_table(false), 65536);
        if ((e = upload(ctx->rgba8_tables, tab.data(), tab.size(), ctx->stream)) != cudaSuccess)
            return cuda_fail(ctx, e, "conversion tables");
    }
    const uint64_t n = ctx->out.count;
    if (ctx->rgba8.count != n && (e = alloc(ctx->rgba8, n)) != cudaSuccess) return cuda_fail(ctx, e, "RGBA8 image");
    if ((e = launch_rgba16f_to_rgba8(ctx->out.ptr, n, ctx->rgba8_tables.ptr, ctx->rgba8.ptr, ctx->stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(rgba8, ctx->rgba8.ptr, n * sizeof(uchar4), cudaMemcpyDefault, ctx->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess)
        return cuda_fail(ctx, e, "RGBA8 conversion");
    return SPK_OK;
} catch (const std::bad_alloc &) {
    return fail(ctx, SPK_ERR_OUT_OF_MEMORY, "host memory exhausted");
} catch (const std::exception &ex) {
    return fail(ctx, SPK_ERR_INTERNAL, "%s", ex.what());
}

spk_status spk_save_image(spk_ctx *ctx, const char *path, uint32_t format) try {
    NvtxRange range("spk_save_image");
    if (!ctx || !path || !*path) return SPK_ERR_INVALID_ARGUMENT;
    if (!ctx->has_config) return fail(ctx, SPK_ERR_NOT_READY, "no frame buffer");
    if (format > SPK_IMAGE_EXR) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "unknown image format %u", format);
    if (const spk_status st = require_own_buffers(ctx)) return st;
    const uint32_t w = ctx->cfg.width, h = ctx->cfg.height;
    const uint64_t n = static_cast<uint64_t>(w) * h;
    std::vector<uint8_t> bytes;
    cudaError_t e;
    if (format == SPK_IMAGE_PNG) {
        std::vector<uint8_t> px(4 * n);
        const spk_status st = spk_read_rgba8(ctx, px.data());
        if (st != SPK_OK) return st;
        bytes = encode_png(px.data(), w, h);
    } else if (format == SPK_IMAGE_HDR) {
        std::vector<float> fb(4 * n), top(4 * n);
        if ((e = cudaMemcpyAsync(fb.data(), ctx->fb.ptr, n * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream)) !=
                cudaSuccess ||
            (e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess)
            return cuda_fail(ctx, e, "frame buffer read");
        for (uint32_t y = 0; y < h; ++y)  // frame buffer rows run bottom up
            std::memcpy(&top[4ull * y * w], &fb[4ull * (h - 1 - y) * w], 4ull * w * sizeof(float));
        bytes = encode_hdr(top.data(), w, h);
    } else {
        if (ctx->fb_half.count != n && (e = alloc(ctx->fb_half, n)) != cudaSuccess)
            return cuda_fail(ctx, e, "half image");
        std::vector<uint16_t> px(4 * n);
        if ((e = launch_fb_to_half(ctx->fb.ptr, w, h, ctx->fb_half.ptr, ctx->stream)) != cudaSuccess ||
            (e = cudaMemcpyAsync(px.data(), ctx->fb_half.ptr, n * sizeof(ushort4), cudaMemcpyDeviceToHost,
                                 ctx->stream)) != cudaSuccess ||
            (e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess)
            return cuda_fail(ctx, e, "half image");
        bytes = encode_exr(px.data(), w, h);
    }
    std::string err;
    if (!write_file(path, bytes, err)) return fail(ctx, SPK_ERR_IO, "%s", err.c_str());
    return SPK_OK;
} catch (const std::bad_alloc &) {
    return fail(ctx, SPK_ERR_OUT_OF_MEMORY, "host memory exhausted");
} catch (const std::exception &ex) {
    return fail(ctx, SPK_ERR_INTERNAL, "%s", ex.what());
}

spk_status spk_write_png(const char *path, const uint8_t *rgba8, uint32_t width, uint32_t height) try {
    if (!path || !rgba8 || width == 0 || height == 0) return SPK_ERR_INVALID_ARGUMENT;
    std::string err;
    return write_file(path, encode_png(rgba8, width, height), err) ? SPK_OK : SPK_ERR_IO;
} catch (const std::bad_alloc &) {
    return SPK_ERR_OUT_OF_MEMORY;
} catch (const std::exception &ex) {
    (void)ex;
    return SPK_ERR_INTERNAL;
}

spk_status spk_write_hdr(const char *path, const float *rgba, uint32_t width, uint32_t height) try {
    if (!path || !rgba || width == 0 || height == 0) return SPK_ERR_INVALID_ARGUMENT;
    std::string err;
    return write_file(path, encode_hdr(rgba, width, height), err) ? SPK_OK : SPK_ERR_IO;
} catch (const std::bad_alloc &) {
    return SPK_ERR_OUT_OF_MEMORY;
} catch (const std::exception &ex) {
    (void)ex;
    return SPK_ERR_INTERNAL;
}

spk_status spk_write_exr(const char *path, const uint16_t *rgba16f, uint32_t width, uint32_t height) try {
    if (!path || !rgba16f || width == 0 || height == 0) return SPK_ERR_INVALID_ARGUMENT;
    std::string err;
    return write_file(path, encode_exr(rgba16f, width, height), err) ? SPK_OK : SPK_ERR_IO;
} catch (const std::bad_alloc &) {
    return SPK_ERR_OUT_OF_MEMORY;
} catch (const std::exception &ex) {
    (void)ex;
    return SPK_ERR_INTERNAL;
}

spk_status spk_convert_rgba8(const uint16_t *rgba16f, uint64_t pixels, uint8_t *rgba8) try {
    if (pixels && (!rgba16f || !rgba8)) return SPK_ERR_INVALID_ARGUMENT;
    rgba16f_to_rgba8(rgba16f, pixels, rgba8);
    return SPK_OK;
} catch (const std::bad_alloc &) {
    return SPK_ERR_OUT_OF_MEMORY;
} catch (const std::exception &ex) {
    (void)ex;
    return SPK_ERR_INTERNAL;
}

spk_status spk_framebuffer_device(spk_ctx *ctx, void **hdr_rgba, void **rgba16f) {
    if (!ctx) return SPK_ERR_INVALID_ARGUMENT;
    if (!ctx->has_config) return fail(ctx, SPK_ERR_NOT_READY, "no frame buffer");
    if (hdr_rgba) *hdr_rgba = ctx->fb.ptr;
    if (rgba16f) *rgba16f = ctx->out.ptr;
    return SPK_OK;
}

spk_status spk_sample_counts(const spk_ctx *ctx, uint32_t *cumulated, uint32_t *dispatched) {
    if (!ctx) return SPK_ERR_INVALID_ARGUMENT;
    if (cumulated) *cumulated = ctx->cumulated;
    if (dispatched) *dispatched = ctx->dispatched;
    return SPK_OK;
}

int32_t spk_is_converged(const spk_ctx *ctx) {
    return ctx && ctx->has_config && ctx->cumulated >= ctx->cfg.max_spp ? 1 : 0;
}

static spk_status trace_impl(spk_ctx *ctx, const void *d_rays, uint64_t num_rays, void *d_hits, int32_t any_hit) {
    cudaError_t e;
    if ((e = prepare_events(ctx, 1)) != cudaSuccess) return cuda_fail(ctx, e, "event pool");
    if ((e = cudaMemsetAsync(ctx->counters, 0, sizeof(Counters), ctx->stream)) != cudaSuccess)
        return cuda_fail(ctx, e, "counter reset");
    cudaEventRecord(ctx->ev_start, ctx->stream);
    e = launch_trace(ctx->scene, static_cast<const float *>(d_rays), num_rays, d_hits,
                     any_hit ? kTraceAnyRef : kTraceClosest, (ctx->instrumentation & SPK_INSTR_COUNT_TRAFFIC) != 0,
                     ctx->counters, ctx->num_sms, ctx->stream, &ctx->launch_events);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "trace launch");
    cudaEventRecord(ctx->ev_stop, ctx->stream);
    ctx->launches_in_call = 1;
    ctx->last = spk_stats{};
    ctx->noalloc_counters = nullptr;
    ctx->stats_pending = true;
    return SPK_OK;
}

spk_status spk_trace_device(spk_ctx *ctx, const void *d_rays, uint64_t num_rays, void *d_hits, int32_t any_hit) {
    if (!ctx || (num_rays && (!d_rays || !d_hits))) return SPK_ERR_INVALID_ARGUMENT;
    if (!ctx->has_scene) return fail(ctx, SPK_ERR_NOT_READY, "trace needs spk_set_scene first");
    cudaSetDevice(ctx->device);
    return trace_impl(ctx, d_rays, num_rays, d_hits, any_hit);
}

spk_status spk_trace(spk_ctx *ctx, const spk_ray *rays, uint64_t num_rays, spk_hit *hits, int32_t any_hit) try {
    NvtxRange range("spk_trace");
    if (!ctx || (num_rays && (!rays || !hits))) return SPK_ERR_INVALID_ARGUMENT;
    if (!ctx->has_scene) return fail(ctx, SPK_ERR_NOT_READY, "trace needs spk_set_scene first");
    cudaSetDevice(ctx->device);
    if (num_rays == 0) return SPK_OK;
    void *d_rays = nullptr, *d_hits = nullptr;
    cudaError_t e;
    if ((e = cudaMalloc(&d_rays, num_rays * sizeof(spk_ray))) != cudaSuccess) return cuda_fail(ctx, e, "ray buffer");
    if ((e = cudaMalloc(&d_hits, num_rays * sizeof(spk_hit))) != cudaSuccess) {
        cudaFree(d_rays);
        return cuda_fail(ctx, e, "hit buffer");
    }
    spk_status st = SPK_OK;
    if ((e = cudaMemcpyAsync(d_rays, rays, num_rays * sizeof(spk_ray), cudaMemcpyHostToDevice, ctx->stream)) !=
        cudaSuccess) {
        st = cuda_fail(ctx, e, "ray upload");
    } else if ((st = trace_impl(ctx, d_rays, num_rays, d_hits, any_hit)) == SPK_OK) {
        if ((e = cudaMemcpyAsync(hits, d_hits, num_rays * sizeof(spk_hit), cudaMemcpyDeviceToHost, ctx->stream)) !=
                cudaSuccess ||
            (e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) {
            st = cuda_fail(ctx, e, "hit download");
        }
    }
    cudaStreamSynchronize(ctx->stream);
    cudaFree(d_rays);
    cudaFree(d_hits);
    return st;
} catch (const std::bad_alloc &) {
    return fail(ctx, SPK_ERR_OUT_OF_MEMORY, "host memory exhausted");
} catch (const std::exception &ex) {
    return fail(ctx, SPK_ERR_INTERNAL, "%s", ex.what());
}

spk_status spk_synchronize(spk_ctx *ctx) {
    if (!ctx) return SPK_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    const cudaError_t e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? SPK_OK : cuda_fail(ctx, e, "synchronize");
}

spk_status spk_get_stats(spk_ctx *ctx, spk_stats *out) {
    if (!ctx || !out) return SPK_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (ctx->stats_pending) {
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "synchronize");
        Counters c{};
        const Counters *src = ctx->noalloc_counters ? ctx->noalloc_counters : ctx->counters;
        if ((e = cudaMemcpy(&c, src, sizeof(Counters), cudaMemcpyDeviceToHost)) != cudaSuccess)
            return cuda_fail(ctx, e, "counter read");
        ctx->last.extension_rays = c.extension_rays;
        ctx->last.shadow_rays = c.shadow_rays;
        ctx->last.error_flags = c.error_flags;
        ctx->last.node_visits = c.node_visits;
        ctx->last.triangle_tests = c.tri_tests;
        ctx->stats_pending = false;
        if (ctx->noalloc_counters) {  // no events are recorded by spk_render_noalloc: counters only
            ctx->last.kernel_launches = ctx->launches_in_call;
            ctx->last.bvh_nodes = ctx->bvh_nodes;
            ctx->last.bvh_bytes = ctx->bvh_bytes;
            *out = ctx->last;
            out->blas_reused = ctx->blas_reused;
            return SPK_OK;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop);
        ctx->last.device_ms = ms;
        float tms = 0.f;
        const LaunchEvents &le = ctx->launch_events;
        for (int k = 0; k < le.used; ++k) {
            float x = 0.f;
            cudaEventElapsedTime(&x, le.pairs[2 * k], le.pairs[2 * k + 1]);
            tms += x;
        }
        ctx->last.trace_kernel_ms = tms + le.graph_ms;
        ctx->last.trace_launches = static_cast<uint32_t>(le.used + le.graph_launches);
        ctx->last.kernel_launches = ctx->launches_in_call;
        ctx->stats_pending = false;
    }
    ctx->last.bvh_nodes = ctx->bvh_nodes;
    ctx->last.bvh_bytes = ctx->bvh_bytes;
    *out = ctx->last;
    out->blas_reused = ctx->blas_reused;
    return SPK_OK;
}

spk_status spk_render_guides(spk_ctx *ctx) try {
    NvtxRange range("spk_render_guides");
    if (!ctx) return SPK_ERR_INVALID_ARGUMENT;
    if (!ctx->has_scene || !ctx->has_config || !ctx->has_camera)
        return fail(ctx, SPK_ERR_NOT_READY, "guides need spk_set_scene, spk_set_config and spk_set_camera first");
    cudaSetDevice(ctx->device);
    const size_t n = static_cast<size_t>(ctx->cfg.width) * ctx->cfg.height;
    cudaError_t e;
    if (ctx->guide_nd.count != n) {
        ctx->guide_nd.reset();
        ctx->guide_albedo.reset();
        if ((e = cudaMalloc(reinterpret_cast<void **>(&ctx->guide_nd.ptr), n * sizeof(float4))) != cudaSuccess ||
            (e = cudaMalloc(reinterpret_cast<void **>(&ctx->guide_albedo.ptr), n * sizeof(float4))) != cudaSuccess)
            return cuda_fail(ctx, e, "guide buffers");
        ctx->guide_nd.count = ctx->guide_albedo.count = n;
    }
    if ((e = launch_guides(ctx->scene, ctx->cam, ctx->cfg.width, ctx->cfg.height, ctx->guide_nd.ptr,
                           ctx->guide_albedo.ptr, ctx->counters, ctx->stream)) != cudaSuccess)
        return cuda_fail(ctx, e, "guides launch");
    return SPK_OK;
} catch (const std::bad_alloc &) {
    return fail(ctx, SPK_ERR_OUT_OF_MEMORY, "host memory exhausted");
} catch (const std::exception &ex) {
    return fail(ctx, SPK_ERR_INTERNAL, "%s", ex.what());
}

spk_status spk_guides_device(spk_ctx *ctx, void **normal_depth, void **albedo) {
    if (!ctx) return SPK_ERR_INVALID_ARGUMENT;
    if (!ctx->guide_nd.ptr) return fail(ctx, SPK_ERR_NOT_READY, "no guides: call spk_render_guides first");
    if (normal_depth) *normal_depth = ctx->guide_nd.ptr;
    if (albedo) *albedo = ctx->guide_albedo.ptr;
    return SPK_OK;
}

spk_status spk_read_guides(spk_ctx *ctx, float *normal_depth, float *albedo) {
    if (!ctx) return SPK_ERR_INVALID_ARGUMENT;
    if (!ctx->guide_nd.ptr) return fail(ctx, SPK_ERR_NOT_READY, "no guides: call spk_render_guides first");
    cudaSetDevice(ctx->device);
    cudaError_t e;
    const size_t bytes = ctx->guide_nd.count * sizeof(float4);
    if ((normal_depth && (e = cudaMemcpyAsync(normal_depth, ctx->guide_nd.ptr, bytes, cudaMemcpyDefault,
                                              ctx->stream)) != cudaSuccess) ||
        (albedo && (e = cudaMemcpyAsync(albedo, ctx->guide_albedo.ptr, bytes, cudaMemcpyDefault, ctx->stream)) !=
                       cudaSuccess))
        return cuda_fail(ctx, e, "guide read");
    if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return cuda_fail(ctx, e, "synchronize");
    return SPK_OK;
}

spk_status spk_render_batch(spk_ctx *ctx, const spk_request *requests, uint32_t num_requests, uint32_t rng,
                            uint32_t enable_nee) try {
    NvtxRange range("spk_render_batch");
    if (!ctx) return SPK_ERR_INVALID_ARGUMENT;
    if (!ctx->has_scene) return fail(ctx, SPK_ERR_NOT_READY, "batch needs spk_set_scenes first");
    if (!requests || num_requests == 0) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "no requests");
    if (rng > SPK_RNG_XOSHIRO256SS) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "unknown rng %u", rng);
    cudaSetDevice(ctx->device);
    std::vector<DevRequest> reqs(num_requests);
    unsigned long long items = 0, pixels = 0;
    for (uint32_t r = 0; r < num_requests; ++r) {
        const spk_request &q = requests[r];
        if (q.scene >= ctx->scene.num_scenes)
            return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "request %u: scene %u of %u", r, q.scene, ctx->scene.num_scenes);
        if (q.width < 2 || q.height < 2 || q.spp == 0 || q.bounce == 0)
            return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "request %u: needs width, height >= 2 and spp, bounce >= 1", r);
        DevRequest &d = reqs[r];
        std::memset(&d, 0, sizeof(d));
        std::memcpy(&d.cam, &q.camera, sizeof(DevCamera));
        d.scene = q.scene;
        d.width = q.width;
        d.height = q.height;
        d.npix = q.width * q.height;
        d.spp = q.spp;
        d.bounce = q.bounce;
        d.seed = q.seed;
        d.item_base = items;
        d.pixel_base = pixels;
        items += static_cast<unsigned long long>(d.npix) * q.spp;
        pixels += d.npix;
    }
    if (items >= 0xFFFFFFFFull)
        return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "batch of %llu sample items: split it below 2^32", items);
    const uint32_t slots = static_cast<uint32_t>(
        std::min<unsigned long long>(items, ctx->tuning.batch_slots ? ctx->tuning.batch_slots : kMaxPathSlots));
    // Groups of consecutive whole requests, each one wavefront, and their first-pass queue layout (batch_plan.h).
    std::vector<BatchGroup> groups;
    {
        std::vector<uint64_t> req_items(num_requests);
        std::vector<uint32_t> req_spp(num_requests), queue_base(num_requests);
        for (uint32_t r = 0; r < num_requests; ++r) {
            req_items[r] = 1ull * reqs[r].npix * reqs[r].spp;
            req_spp[r] = reqs[r].spp;
        }
        const bool pk = ctx->tuning.primary_packets != 0;
        for (const BatchPlanGroup &g : plan_batch(req_items.data(), req_spp.data(), num_requests, slots,
                                                  kPacketMinSamples, kPacket2MinSamples, queue_base.data()))
            groups.push_back(BatchGroup{g.item_lo, g.item_hi, pk ? g.packet_items : 0ull, pk ? g.packet2_items : 0ull});
        for (uint32_t r = 0; r < num_requests; ++r) reqs[r].queue_base = queue_base[r];
    }
    cudaError_t e;
    WavefrontState &s = ctx->wf_batch;
    if (s.capacity < slots && (e = wavefront_alloc(s, slots)) != cudaSuccess) return cuda_fail(ctx, e, "batch slots");
    if (s.sample_capacity < items) {
        if (s.samples) cudaFree(s.samples);
        s.samples = nullptr;
        s.sample_capacity = 0;
        if ((e = cudaMalloc(reinterpret_cast<void **>(&s.samples), items * sizeof(float4))) != cudaSuccess)
            return cuda_fail(ctx, e, "batch sample buffer");
        s.sample_capacity = items;
    }
    if ((e = upload(ctx->batch_reqs, reqs.data(), reqs.size(), ctx->stream)) != cudaSuccess)
        return cuda_fail(ctx, e, "batch requests");
    if (ctx->batch_hdr.count < pixels) {
        ctx->batch_hdr.reset();
        ctx->batch_img.reset();
        if ((e = cudaMalloc(reinterpret_cast<void **>(&ctx->batch_hdr.ptr), pixels * sizeof(float4))) != cudaSuccess ||
            (e = cudaMalloc(reinterpret_cast<void **>(&ctx->batch_img.ptr), pixels * sizeof(ushort4))) != cudaSuccess)
            return cuda_fail(ctx, e, "batch outputs");
        ctx->batch_hdr.count = ctx->batch_img.count = pixels;
    }
    BatchParams b{};
    b.reqs = ctx->batch_reqs.ptr;
    b.num_reqs = num_requests;
    b.rng = rng;
    b.enable_nee = enable_nee ? 1u : 0u;
    b.total_items = items;
    b.total_pixels = pixels;
    b.item_lo = 0;
    b.item_hi = items;
    b.out_hdr = ctx->batch_hdr.ptr;
    b.out_image = ctx->batch_img.ptr;
    const bool count = (ctx->instrumentation & SPK_INSTR_COUNT_TRAFFIC) != 0;
    if ((e = prepare_events(ctx, 16)) != cudaSuccess) return cuda_fail(ctx, e, "event pool");
    if ((e = cudaMemsetAsync(ctx->counters, 0, sizeof(Counters), ctx->stream)) != cudaSuccess)
        return cuda_fail(ctx, e, "counter reset");
    if ((e = cudaEventRecord(ctx->ev_start, ctx->stream)) != cudaSuccess) return cuda_fail(ctx, e, "event");
    uint32_t launches = 0;
    ctx->launch_events.capacity = 0;  // per-launch traversal timing is not recorded for batches
    WfTuning bt = wf_tuning(ctx);
    bt.batch_slots = slots;  // the state may be larger (it only grows): use the requested number of paths
    e = launch_render_batch(ctx->scene, b, groups, count, ctx->counters, s, ctx->num_sms, ctx->stream, &launches,
                            nullptr, bt);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "batch wavefront");
    if ((e = cudaEventRecord(ctx->ev_stop, ctx->stream)) != cudaSuccess) return cuda_fail(ctx, e, "event");
    ctx->batch_host = reqs;
    ctx->launches_in_call = launches;
    ctx->last = spk_stats{};
    ctx->last.paths = items;
    ctx->noalloc_counters = nullptr;
    ctx->stats_pending = true;
    if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return cuda_fail(ctx, e, "synchronize");
    return SPK_OK;
} catch (const std::bad_alloc &) {
    return fail(ctx, SPK_ERR_OUT_OF_MEMORY, "host memory exhausted");
} catch (const std::exception &ex) {
    return fail(ctx, SPK_ERR_INTERNAL, "%s", ex.what());
}

spk_status spk_read_batch(spk_ctx *ctx, uint32_t index, float *hdr_rgba, uint16_t *rgba16f) try {
    if (!ctx) return SPK_ERR_INVALID_ARGUMENT;
    if (index >= ctx->batch_host.size()) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "no request %u in the last batch", index);
    cudaSetDevice(ctx->device);
    const DevRequest &r = ctx->batch_host[index];
    cudaError_t e;
    if (hdr_rgba && (e = cudaMemcpyAsync(hdr_rgba, ctx->batch_hdr.ptr + r.pixel_base, r.npix * sizeof(float4),
                                         cudaMemcpyDefault, ctx->stream)) != cudaSuccess)
        return cuda_fail(ctx, e, "batch read");
    if (rgba16f && (e = cudaMemcpyAsync(rgba16f, ctx->batch_img.ptr + r.pixel_base, r.npix * sizeof(ushort4),
                                        cudaMemcpyDefault, ctx->stream)) != cudaSuccess)
        return cuda_fail(ctx, e, "batch read");
    if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return cuda_fail(ctx, e, "synchronize");
    return SPK_OK;
} catch (const std::bad_alloc &) {
    return fail(ctx, SPK_ERR_OUT_OF_MEMORY, "host memory exhausted");
} catch (const std::exception &ex) {
    return fail(ctx, SPK_ERR_INTERNAL, "%s", ex.what());
}

void spk_tuning_defaults(spk_tuning *out) {
    if (!out) return;
    *out = spk_tuning{};
    out->cuda_graph = 1;
    out->material_sort = 0;
    out->bvh_width = 8;
    out->bvh_leaf_size = 3;
    out->extend_blocks_per_sm = 0;
    out->shade_blocks_per_sm = 8;
    out->bvh_collapse = 0;
    out->bvh_builder = 0;
    out->path_slots_per_pixel = 64;
    out->shadow_stage = 1;
    out->multi_frame = 1;
    out->primary_packets = 1;
}

spk_status spk_set_tuning(spk_ctx *ctx, const spk_tuning *t) {
    if (!ctx || !t) return SPK_ERR_INVALID_ARGUMENT;
    if (t->cuda_graph > 1 || t->material_sort > 1)
        return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "cuda_graph and material_sort take 0 or 1");
    if (t->bvh_width < 2 || t->bvh_width > 8) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "bvh_width must be 2..8");
    if (t->bvh_leaf_size < 1 || t->bvh_leaf_size > 3)
        return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "bvh_leaf_size must be 1..3");
    if (t->extend_blocks_per_sm > 32 || t->shade_blocks_per_sm < 1 || t->shade_blocks_per_sm > 32)
        return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "blocks per SM out of range");
    if (t->ray_sort > 1 || t->bvh_collapse > 1)
        return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "ray_sort and bvh_collapse take 0 or 1");
    if (t->bvh_builder > 2) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "bvh_builder takes 0, 1 or 2");
    if (t->path_slots_per_pixel < 1 || t->path_slots_per_pixel > 64)
        return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "path_slots_per_pixel must be 1..64");
    if (t->shadow_stage > 1 || t->multi_frame > 1 || t->primary_packets > 1)
        return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "shadow_stage, multi_frame and primary_packets take 0 or 1");
    ctx->tuning = *t;
    return SPK_OK;
}

spk_status spk_get_tuning(const spk_ctx *ctx, spk_tuning *out) {
    if (!ctx || !out) return SPK_ERR_INVALID_ARGUMENT;
    *out = ctx->tuning;
    return SPK_OK;
}

spk_status spk_set_instrumentation(spk_ctx *ctx, uint32_t flags) {
    if (!ctx) return SPK_ERR_INVALID_ARGUMENT;
    if (flags & ~static_cast<uint32_t>(SPK_INSTR_COUNT_TRAFFIC))
        return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "unknown instrumentation flags 0x%x", flags);
    ctx->instrumentation = flags;
    return SPK_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------------------
// spk_render_noalloc: the one-kernel render into caller-owned buffers, with its scratch (the per-frame
// G-buffer and the counters) in a static device array instead of context allocations, for callers that
// must not allocate while rendering.
// ------------------------------------------------------------------------------------------------
namespace {

constexpr size_t kNoallocGbufferBytes = static_cast<size_t>(SPK_NOALLOC_MAX_PIXELS) * 2 * sizeof(float4);
constexpr size_t kNoallocCounterBytes = 256;
static_assert(sizeof(Counters) <= kNoallocCounterBytes, "counters fit their slot");

// G-buffer colour (max pixels x float4), G-buffer normal (max pixels x float4), then the counters.
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocGbufferBytes + kNoallocCounterBytes];

constexpr int kNoallocMaxDevices = 64;
std::mutex g_noalloc_mutex;
struct NoallocAddress {
    unsigned long long context_id = 0;  // the CUDA context the address belongs to (0: none looked up)
    void *address = nullptr;
};
NoallocAddress g_noalloc_address[kNoallocMaxDevices];

using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);

// The current CUDA context's unique id (cuCtxGetId, through the driver entry point: no libcuda link
// dependency). A device's primary context that was torn down (cudaDeviceReset) and created again gets a
// new id, and its module -- with g_noalloc_scratch -- is loaded again at another address.
cudaError_t current_context_id(unsigned long long *id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr, *q = nullptr;
        cudaDriverEntryPointQueryResult r1, r2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &r1) == cudaSuccess &&
            r1 == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &q, 12000, cudaEnableDefault, &r2) == cudaSuccess &&
            r2 == cudaDriverEntryPointSuccess) {
            get_current = reinterpret_cast<CtxGetCurrentFn>(p);
            get_id = reinterpret_cast<CtxGetIdFn>(q);
        }
    });
    if (!get_current || !get_id) return cudaErrorNotSupported;
    CUcontext c = nullptr;
    if (get_current(&c) != CUDA_SUCCESS || !c || get_id(c, id) != CUDA_SUCCESS) return cudaErrorDeviceUninitialized;
    return cudaSuccess;
}

// Device address of g_noalloc_scratch on `device` (current, its context initialised), looked up once per
// device and context. The host-side name of the array is only a stand-in and must never be handed to a
// kernel.
cudaError_t noalloc_scratch(int device, unsigned char **out) {
    if (device < 0 || device >= kNoallocMaxDevices) return cudaErrorInvalidDevice;
    unsigned long long id = 0;
    cudaError_t e = current_context_id(&id);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    NoallocAddress &slot = g_noalloc_address[device];
    if (slot.context_id != id || !slot.address) {
        void *p = nullptr;
        if ((e = cudaGetSymbolAddress(&p, g_noalloc_scratch)) != cudaSuccess) return e;
        slot.address = p;
        slot.context_id = id;
    }
    *out = static_cast<unsigned char *>(slot.address);
    return cudaSuccess;
}

}  // namespace

extern "C" spk_status spk_render_noalloc(spk_ctx *ctx, uint32_t num_frames, void *d_hdr_rgba, void *d_rgba16f) try {
    if (!ctx) return SPK_ERR_INVALID_ARGUMENT;
    if (!d_hdr_rgba || !d_rgba16f) return fail(ctx, SPK_ERR_INVALID_ARGUMENT, "null output buffer");
    if (!ctx->has_scene || !ctx->has_config || !ctx->has_camera)
        return fail(ctx, SPK_ERR_NOT_READY, "render needs spk_set_scene, spk_set_config and spk_set_camera first");
    const uint64_t npix = static_cast<uint64_t>(ctx->cfg.width) * ctx->cfg.height;
    if (npix > SPK_NOALLOC_MAX_PIXELS)
        return fail(ctx, SPK_ERR_INVALID_ARGUMENT,
                    "spk_render_noalloc supports at most %u pixels (512 x 512); the config has %llu", SPK_NOALLOC_MAX_PIXELS,
                    static_cast<unsigned long long>(npix));
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "set device");
    unsigned char *scratch = nullptr;
    if ((e = noalloc_scratch(ctx->device, &scratch)) != cudaSuccess) return cuda_fail(ctx, e, "scratch address");
    float4 *gcolor = reinterpret_cast<float4 *>(scratch);
    float4 *gnormal = gcolor + SPK_NOALLOC_MAX_PIXELS;
    auto *counters = reinterpret_cast<Counters *>(scratch + kNoallocGbufferBytes);
    FrameBuffers fbuf{gcolor, gnormal, static_cast<float4 *>(d_hdr_rgba), static_cast<ushort4 *>(d_rgba16f),
                      ctx->cfg.width, ctx->cfg.height};
    // The sample bookkeeping belongs to one frame buffer: frames accumulated so far in another one (the
    // context's own, or another caller buffer) are not in this one, so it starts over.
    if (ctx->accum_target != d_hdr_rgba) {
        ctx->dirty = true;
        ctx->accum_target = d_hdr_rgba;
    }
    // The array keeps the previous call's contents; only the counters must start at zero (the G-buffer is
    // fully written by every frame before it is read).
    if ((e = cudaMemsetAsync(counters, 0, sizeof(Counters), ctx->stream)) != cudaSuccess)
        return cuda_fail(ctx, e, "counter reset");
    ctx->noalloc_counters = counters;
    ctx->launches_in_call = 0;
    ctx->last = spk_stats{};
    ctx->last.paths = static_cast<uint64_t>(num_frames) * npix;
    ctx->stats_pending = true;
    for (uint32_t f = 0; f < num_frames; ++f) {
        // The same per-frame bookkeeping as spk_render (CameraRenderProxy.cpp:66-75, CPURenderer.cpp:128-137).
        if (ctx->dirty) {
            ctx->cumulated = 0;
            ctx->pending = 0;
        }
        ctx->cumulated = std::min(ctx->cfg.max_spp, ctx->cumulated + ctx->pending);
        ctx->pending = 0;
        if (ctx->dirty) {
            if ((e = cudaMemsetAsync(d_hdr_rgba, 0, npix * sizeof(float4), ctx->stream)) != cudaSuccess)
                return cuda_fail(ctx, e, "frame buffer clear");
            ctx->dirty = false;
            ctx->dispatched = ctx->cfg.sample_offset;
        }
        const RenderParams p{ctx->dispatched, ctx->cfg.bounce, ctx->cfg.rng, ctx->cfg.seed, ctx->cfg.spatial_denoise,
                             ctx->cfg.enable_nee};
        if ((e = launch_render_mega(ctx->scene, ctx->cam, fbuf, p, false, counters, ctx->stream, nullptr)) !=
            cudaSuccess)
            return cuda_fail(ctx, e, "base pass launch");
        const float mavg = static_cast<float>(ctx->cumulated) / static_cast<float>(ctx->cumulated + ctx->spp_eff);
        if ((e = launch_resolve(fbuf, mavg, ctx->cam.exposure, ctx->cfg.spatial_denoise, ctx->stream)) != cudaSuccess)
            return cuda_fail(ctx, e, "resolve launch");
        ctx->launches_in_call += 2;
        ctx->dispatched += ctx->spp_eff;
        ctx->pending += ctx->spp_eff;
    }
    return SPK_OK;
} catch (const std::bad_alloc &) {
    return fail(ctx, SPK_ERR_OUT_OF_MEMORY, "host memory exhausted");
} catch (const std::exception &ex) {
    return fail(ctx, SPK_ERR_INTERNAL, "%s", ex.what());
}
