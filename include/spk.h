/*
 * spk.h -- C ABI of the GB300 path tracer.
 *
 * This is the drop-in boundary for Sparkle's `cpu` pipeline. Sparkle has no C ABI: its boundary is the
 * C++ virtual `Renderer` (libraries/include/renderer/renderer/Renderer.h:28-108) instantiated as
 * `CPURenderer` (libraries/source/renderer/renderer/CPURenderer.cpp) for `RenderConfig::Pipeline::Cpu`,
 * reading the render-thread scene through `SceneRenderProxy` (libraries/include/renderer/proxy/
 * SceneRenderProxy.h:46-121). Each entry point below names the reference interface it replaces.
 *
 * Conventions
 *  - Every call returns spk_status (0 = ok) and never aborts; the text of the last error of a context is
 *    returned by spk_last_error().
 *  - Plain pointers and sizes only. Host pointers are copied in or out before the call returns; the
 *    *_device entry points take device pointers that stay owned by the caller.
 *  - A context owns all device memory it allocates. One context is used by one thread at a time (the
 *    reference renders on its render thread only, Renderer.cpp:20); several contexts may coexist.
 *  - Coordinate system, units and constants are the reference's: Z up, Y front, X right
 *    (libraries/include/core/math/Types.h:45-47).
 */
#ifndef SPK_H_
#define SPK_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPK_ABI_VERSION 4u

typedef int32_t spk_status;
enum {
    SPK_OK = 0,
    SPK_ERR_INVALID_ARGUMENT = 1,
    SPK_ERR_CUDA = 2,
    SPK_ERR_OUT_OF_MEMORY = 3,
    SPK_ERR_NOT_READY = 4,      /* e.g. render before set_scene / set_config */
    SPK_ERR_DEVICE_LIMIT = 5,   /* a device-side bound (traversal stack, iteration budget) was exceeded */
    SPK_ERR_INTERNAL = 6,
    SPK_ERR_IO = 7,             /* a file could not be written */
};

typedef struct spk_ctx spk_ctx;

/* ------------------------------------------------------------------------------------------------ */
/* Scene description (render-thread proxies, copied in by spk_set_scene)                             */
/* ------------------------------------------------------------------------------------------------ */

/* A triangle mesh as held by `Mesh` (libraries/include/io/Mesh.h:7-141): per-vertex SoA attributes and a
 * triangle index list. normals are required (Mesh::Validate, Mesh.h:136-140); tangents may be NULL
 * (Mesh::GetTangent then returns (1,0,0,1), Mesh.h:104-118); uvs may be NULL (zero, Mesh.h:120-134). */
typedef struct spk_mesh {
    const float *positions; /* [num_vertices][3] */
    const float *normals;   /* [num_vertices][3] */
    const float *tangents;  /* [num_vertices][4] or NULL */
    const float *uvs;       /* [num_vertices][2] or NULL */
    const uint32_t *indices; /* [num_faces][3] */
    uint32_t num_vertices;
    uint32_t num_faces;
} spk_mesh;

enum { SPK_PRIM_MESH = 0, SPK_PRIM_SPHERE = 1 };

/* One `PrimitiveRenderProxy` (libraries/include/renderer/proxy/PrimitiveRenderProxy.h:14-78): a mesh
 * instance (`MeshRenderProxy`) or an analytic sphere (`SphereRenderProxy`, SphereRenderProxy.h:9-42).
 * `transform` is the affine matrix M (row-major 3x4: linear part | translation) of the proxy's
 * `Transform`; `inv_transform` is the inverse the reference keeps beside it (Transform.h:141-142) and uses
 * to move world rays into local space (MeshRenderProxy.cpp:99-100). Both are given by the caller so that
 * every consumer uses the same bits. A sphere's centre is the translation column; `radius` is its scaled
 * radius (SphereRenderProxy::SetRadius, SphereRenderProxy.h:32-35). */
typedef struct spk_instance {
    uint32_t type;        /* SPK_PRIM_MESH / SPK_PRIM_SPHERE */
    uint32_t mesh_id;     /* index into the mesh array (mesh instances) */
    uint32_t material_id; /* index into the material array */
    float radius;         /* spheres only */
    float transform[12];     /* row-major 3x4 */
    float inv_transform[12]; /* row-major 3x4 */
} spk_instance;

enum { SPK_MAT_PBR = 0, SPK_MAT_DIELECTRIC = 1 };

/* A material render proxy: `PbrMaterialRenderProxy` (PbrMaterialRenderProxy.h:10-52) or
 * `DieletricMaterialRenderProxy` (DialetricMaterialRenderProxy.h:10-39), constant-valued
 * (`MaterialResource`, libraries/include/io/Material.h:7-20). The reference's Lambertian and Metal
 * materials are PBR with fixed metallic/roughness (LambertianMaterial.h:8-15, MetalMaterial.h:8-15). */
typedef struct spk_material {
    uint32_t type; /* SPK_MAT_PBR / SPK_MAT_DIELECTRIC */
    float base_color[3];
    float emissive[3];
    float metallic;
    float roughness;
    float eta;
} spk_material;

enum { SPK_SKY_NONE = 0, SPK_SKY_GRADIENT = 1, SPK_SKY_CUBE = 2 };

/* `SkyRenderProxy::Evaluate` input (SkyRenderProxy.cpp:50-64): no sky (misses add nothing), the
 * white-to-colour gradient on d.z, or an RGBA float cube map sampled per face bilinearly with wrap
 * (Image2DCube::Sample, libraries/source/io/Image.cpp:298-357). Faces are +X,-X,+Y,-Y,+Z,-Z, each
 * cube_size x cube_size texels, row-major, 4 floats per texel. */
typedef struct spk_sky {
    uint32_t mode;
    float color[3];
    uint32_t cube_size;
    const float *cube_rgba; /* [6][cube_size][cube_size][4] or NULL */
} spk_sky;

/* ------------------------------------------------------------------------------------------------ */
/* Camera and render configuration                                                                   */
/* ------------------------------------------------------------------------------------------------ */

/* `CameraRenderProxy` posture + focus plane + attribute (CameraRenderProxy.h:30-57), i.e. the values
 * SetupViewRay reads (CPURenderer.cpp:220-238). spk_camera_from_look() derives them the way
 * CameraRenderProxy::Update/OnTransformDirty do (CameraRenderProxy.cpp:10-76, 118-128). */
typedef struct spk_camera {
    float position[3];
    float right[3];
    float up[3];
    float front[3];
    float lower_left[3];
    float max_u[3];
    float max_v[3];
    float aperture_radius;
    float exposure;
    float far_plane;
} spk_camera;

enum { SPK_RNG_XOSHIRO128P = 0, SPK_RNG_XOSHIRO256SS = 1 };
enum { SPK_DEBUG_COLOR = 0 };
enum { SPK_KERNEL_AUTO = 0, SPK_KERNEL_MEGAKERNEL = 1, SPK_KERNEL_WAVEFRONT = 2 };

/* The subset of `RenderConfig` (libraries/include/renderer/RenderConfig.h:28-123) the cpu pipeline reads,
 * with the cvar names of RenderConfig.cpp:13-47 as field names. `rng` selects the per-pixel generator:
 * the reference's Xoshiro128+ reseeded with j*W+i+frame_seed*W*H (Sampler.h:16-40,
 * CPURenderer.cpp:436-444), or xoshiro256** seeded from (seed, pixel index, frame). `enable_nee` turns on
 * next-event estimation (not part of the reference cpu pipeline). `kernel` selects the device
 * schedule; both schedules compute identical results. `sample_offset` (0 in the reference) is the sample
 * count a clear resets dispatched_sample_count_ to: the seed base of the first frame after it. Replica r of
 * several that each render F frames of one view sets it to r * F * spp_eff, so the replicas together draw
 * exactly the samples one renderer draws in N * F frames, under either generator. */
typedef struct spk_config {
    uint32_t width;
    uint32_t height;
    uint32_t spp;     /* `spp` cvar: per-frame sample weight (CPURenderer.cpp:102-105) */
    uint32_t max_spp; /* `max_spp` cvar: accumulation cap (CameraRenderProxy.cpp:66-75) */
    uint32_t bounce;  /* `bounce` cvar: max path segments (CPURenderer.cpp:257-259) */
    uint32_t spatial_denoise; /* `spatial_denoise` cvar (CPURenderer.cpp:452-526) */
    uint32_t enable_nee;
    uint32_t rng;
    uint32_t seed;
    uint32_t debug_mode;
    uint32_t kernel;
    uint32_t sample_offset;
} spk_config;

/* ------------------------------------------------------------------------------------------------ */
/* Ray casting (ray-set parity)                                                                      */
/* ------------------------------------------------------------------------------------------------ */

/* A ray as `Ray` holds it (libraries/include/core/math/Ray.h:8-65): origin and unit direction. */
typedef struct spk_ray {
    float origin[3];
    float direction[3];
} spk_ray;

#define SPK_INVALID_ID 0xFFFFFFFFu

/* The closest-hit candidate `IntersectionCandidate` (Intersection.h:90-103) after the scene walk:
 * world-space t (Ray::InverseAt, Ray.h:43-47), barycentrics u,v of the winning triangle, the scene
 * primitive index (the caller's instance index, not the TLAS-reordered slot) and the original face index.
 * Misses have prim == SPK_INVALID_ID. Spheres report face == SPK_INVALID_ID and u = v = 0. For any-hit
 * queries only `prim` != SPK_INVALID_ID is meaningful. */
typedef struct spk_hit {
    float t;
    float u;
    float v;
    uint32_t prim;
    uint32_t face;
} spk_hit;

/* Counters of the last spk_render / spk_trace call. */
typedef struct spk_stats {
    uint64_t extension_rays; /* closest-hit segments traced */
    uint64_t shadow_rays;    /* any-hit segments traced (NEE) */
    uint64_t paths;          /* camera paths started */
    float device_ms;         /* device time of the call, CUDA events on the context stream */
    float trace_kernel_ms;   /* device time of the traversal kernels alone */
    uint32_t trace_launches; /* launches of the traversal kernels */
    uint32_t kernel_launches; /* all kernel launches of the call */
    uint32_t error_flags;    /* device-side error bits (stack overflow, iteration budget) */
    uint32_t bvh_nodes;      /* wide nodes resident for the scene */
    uint64_t bvh_bytes;      /* bytes of wide nodes + triangle records resident */
    uint64_t node_visits;    /* wide nodes visited (only with SPK_INSTR_COUNT_TRAFFIC) */
    uint64_t triangle_tests; /* ray-triangle tests run (only with SPK_INSTR_COUNT_TRAFFIC) */
    uint32_t graph_replays;  /* CUDA graph launches of the multi-frame iteration chunk (spk_tuning.cuda_graph) */
    uint32_t blas_reused;    /* BLASes the last spk_set_scene took from a spk_set_bvh blob instead of building */
} spk_stats;

enum { SPK_INSTR_NONE = 0, SPK_INSTR_COUNT_TRAFFIC = 1 };

/* Performance knobs (no reference counterpart: the reference's cpu pipeline has none). None of them changes
 * a result: closest hits are resolved with a tie-break independent of the tree's shape and every sample
 * draws its random numbers from its own (pixel, sample) seed, so any setting renders the same bits.
 * spk_tuning_defaults() fills the defaults; sparkle_gb300.autotune searches them per scene. */
typedef struct spk_tuning {
    uint32_t cuda_graph;           /* 1: replay each multi-frame iteration chunk as one CUDA graph (default 1) */
    uint32_t material_sort;        /* 1: group each shade queue by material class before shading (default 0) */
    uint32_t bvh_width;            /* children per wide node, 2..8 (default 8); used by the next spk_set_scene */
    uint32_t bvh_leaf_size;        /* items per BVH leaf, 1..3 (default 3); used by the next spk_set_scene */
    uint32_t extend_blocks_per_sm; /* traversal CTAs per SM, 0 = the occupancy maximum (default 0) */
    uint32_t shade_blocks_per_sm;  /* shading CTAs per SM, 1..32 (default 8) */
    uint32_t batch_slots;          /* path slots (queue capacity) of spk_render_batch, 0 = min(items, 2^27); also the
                                      largest group of requests rendered as one wavefront */
    uint32_t ray_sort;             /* 1: order each extend queue by ray (direction octant, origin cell) (default 0) */
    uint32_t bvh_collapse;         /* 8-wide collapse: 0 greedy largest-area (default), 1 SAH-optimal; next spk_set_scene */
    uint32_t bvh_builder;          /* BLAS builder: 0 host binned SAH (default), 1 device LBVH (Karras radix tree over
                                      Morton order), 2 device PLOC clustering over Morton order; 1 and 2 use the greedy
                                      collapse (bvh_collapse ignored) and take milliseconds where the host takes seconds */
    uint32_t path_slots_per_pixel; /* multi-frame schedule: paths in flight per pixel, 1..64 (default 64: every sample
                                      of a 64-frame call at once, at most 2^27 paths, ~144 B of state each). More paths
                                      per extend launch spread each launch's tail (its last, longest walks) over more
                                      rays; spk_render(1) uses one path per pixel whatever the setting */
    uint32_t shadow_stage;         /* wavefront NEE: 1 (default) queues the light and sky occlusion rays of each
                                      light-sampling vertex for a persistent any-hit stage with lane refill, then adds
                                      their radiance in order; 0 walks them inline in the shade kernel, one per thread */
    uint32_t multi_frame;          /* wavefront: 1 (default) renders all frames of a call in one regenerating wavefront
                                      (16 B per sample of the call, 32 B with the spatial fill, in device memory);
                                      0 renders frame by frame (one path per pixel, no per-sample buffers) */
    uint32_t primary_packets;      /* wavefront: 1 (default) walks the primary rays of a multi-frame pass of >= 8 frames
                                      (of batch requests of >= 8 spp) in packets of 32 consecutive samples (64 from 32
                                      frames), a pixel's samples side by side, each node tested once for the packet; 0
                                      walks every ray on its own. Fewer samples per pixel are walked on their own
                                      either way */
} spk_tuning;

/* ------------------------------------------------------------------------------------------------ */
/* Entry points                                                                                      */
/* ------------------------------------------------------------------------------------------------ */

/* ABI version of the loaded library (SPK_ABI_VERSION). */
uint32_t spk_abi_version(void);

/* Replaces Renderer::CreateRenderer(Pipeline::Cpu, ...) (Renderer.cpp:17-52) + CPURenderer's constructor
 * (CPURenderer.cpp:22-28). Selects CUDA device `device` and creates the context stream. */
spk_status spk_create(int32_t device, spk_ctx **out_ctx);

/* Releases every device allocation of the context. */
spk_status spk_destroy(spk_ctx *ctx);

/* Text of the last error on this context ("" if none). Valid until the next call on the context. */
const char *spk_last_error(const spk_ctx *ctx);

/* Replaces SceneRenderProxy::UpdateBVH (SceneRenderProxy.cpp:269-297): builds every BLAS
 * (MeshRenderProxy::BuildBVH, MeshRenderProxy.cpp:310-314) and the TLAS (SceneRenderProxy.cpp:31-69) on
 * the host, flattens them into compressed 8-wide nodes and uploads them with the shading attributes.
 * Marks the accumulation dirty, as any primitive change does. */
spk_status spk_set_scene(spk_ctx *ctx, const spk_mesh *meshes, uint32_t num_meshes,
                         const spk_instance *instances, uint32_t num_instances,
                         const spk_material *materials, uint32_t num_materials, const spk_sky *sky);

/* A texture as `Image2D` holds it (libraries/include/io/Image.h:112-150): width x height RGBA texels, row
 * y = v * height, as floats (8-bit formats divided by 255, ColorToVec, Utilities.h:377-380). `srgb` marks an
 * sRGB format, decoded after the bilinear filter (the "pseudo srgb decode" of Image2D::Sample). */
typedef struct spk_texture {
    uint32_t width;
    uint32_t height;
    uint32_t srgb;
    const float *rgba; /* [height][width][4] */
} spk_texture;

/* Texture maps of one material (MaterialResource's *_texture fields, io/Material.h:16-19): indices into the
 * scene's texture array, or -1 for none. With a map the material reads texture x factor (base colour,
 * emissive), texture.z x metallic, texture.y x roughness, and the normal map perturbs the shading normal in
 * the vertex tangent frame (MaterialRenderProxy.h:117-160, MeshRenderProxy.cpp:341-358). */
typedef struct spk_material_maps {
    int32_t base_color;
    int32_t metallic_roughness;
    int32_t emissive;
    int32_t normal;
} spk_material_maps;

/* One scene of a multi-scene context: the arguments of spk_set_scene, plus optional textures (`maps` has
 * num_materials entries, or is NULL for untextured materials). */
typedef struct spk_scene_desc {
    const spk_mesh *meshes;
    uint32_t num_meshes;
    const spk_instance *instances;
    uint32_t num_instances;
    const spk_material *materials;
    uint32_t num_materials;
    const spk_sky *sky;
    const spk_texture *textures;
    uint32_t num_textures;
    const spk_material_maps *maps;
} spk_scene_desc;

/* No reference counterpart (the reference renders one scene). Makes several scenes resident at once, for
 * spk_render_batch: each is built exactly as spk_set_scene builds one, then all share the device arrays.
 * spk_render / spk_trace / spk_render_guides see scene 0. spk_set_scene(...) is
 * spk_set_scenes(&one, 1). */
spk_status spk_set_scenes(spk_ctx *ctx, const spk_scene_desc *scenes, uint32_t num_scenes);

/* Incremental scene changes on a context whose scene came from spk_set_scene (one scene). Each replaces
 * SceneRenderProxy::UpdateBVH for one kind of PrimitiveChangeType (SceneRenderProxy.cpp:269-297): every
 * BLAS stays resident, the TLAS, the instance records and the emissive-triangle light table are rebuilt
 * (on the host: the TLAS is as small as the instance list), and the accumulation is marked dirty. The
 * result of any sequence of updates equals spk_set_scene with the updated arguments.
 *
 * spk_set_instances: New / Remove / Move (index swap) -- the whole instance list, over the resident
 * meshes and materials. */
spk_status spk_set_instances(spk_ctx *ctx, const spk_instance *instances, uint32_t num_instances);

/* Update (PrimitiveRenderProxy::IsTransformDirty, SceneRenderProxy.cpp:213-226): new transforms and inverse
 * transforms (row-major 3x4 each, 12 floats per instance) for instances first .. first + count - 1. */
spk_status spk_set_instance_transforms(spk_ctx *ctx, uint32_t first, uint32_t count, const float *transforms,
                                       const float *inv_transforms);

/* No reference counterpart (Sparkle builds a BLAS once per mesh): new vertex positions (and optionally
 * normals [n][3] and tangents [n][4]) for mesh `mesh_id`, same vertex count and faces. The device rewrites
 * the mesh's triangle records and refits its BLAS level by level, re-quantising every child box as the
 * host builder does; then the TLAS is rebuilt. Host or device pointers. */
spk_status spk_update_mesh(spk_ctx *ctx, uint32_t mesh_id, uint32_t num_vertices, const float *positions,
                           const float *normals, const float *tangents);

/* The resident BVH node array (80-byte compressed 8-wide nodes: every BLAS, then the TLAS): sets *count to
 * its length and copies min(capacity, *count) nodes into `nodes` (host or device) when it is not NULL. */
spk_status spk_read_bvh_nodes(spk_ctx *ctx, void *nodes, uint64_t capacity, uint64_t *count);

/* Replaces CameraRenderProxy::OnTransformDirty/UpdateAttribute (CameraRenderProxy.cpp:118-128): a new
 * camera marks pixels dirty, so the next frame clears the accumulation (CPURenderer.cpp:128-137). */
spk_status spk_set_camera(spk_ctx *ctx, const spk_camera *camera);

/* Derives an spk_camera from a look-at posture the way CameraRenderProxy::Update (vertical fov, focus
 * distance, aspect ratio; CameraRenderProxy.cpp:21-34) and OnTransformDirty (:113-136) do. */
spk_status spk_camera_from_look(const float position[3], const float target[3], const float world_up[3],
                                float vertical_fov_rad, float focus_distance, float aperture_radius,
                                float exposure, uint32_t width, uint32_t height, spk_camera *out);

/* Replaces CPURenderer::InitRenderResources (CPURenderer.cpp:38-105): sizes the frame buffer, G-buffer
 * and output image for `width` x `height` and derives the per-frame sample count round(sqrt(spp))^2. */
spk_status spk_set_config(spk_ctx *ctx, const spk_config *config);

/* The context's current spk_config (SPK_ERR_NOT_READY before spk_set_config). */
spk_status spk_get_config(const spk_ctx *ctx, spk_config *out);

/* Replaces `num_frames` calls of CPURenderer::Render (CPURenderer.cpp:119-208) on a static scene: per frame
 * the clear (if dirty), BasePass (:419-450), DenoisePass (:506-552) and ToneMappingPass (:565-576), with
 * the camera's cumulated-sample bookkeeping between frames (CameraRenderProxy.cpp:66-75). Asynchronous
 * with respect to the host: results are visible to spk_read_framebuffer / spk_synchronize. */
spk_status spk_render(spk_ctx *ctx, uint32_t num_frames);

/* Copies the accumulated HDR frame buffer (`frame_buffer_`, H rows of W float4, row j = image row j from
 * the bottom as the reference indexes it) and/or the tonemapped RGBA16F output image (`output_image_`,
 * already flipped: row 0 is the top row, CPURenderer.cpp:573). Either pointer may be NULL; each may be host
 * memory or device memory of the context's GPU (the copy direction follows from the pointer). */
spk_status spk_read_framebuffer(spk_ctx *ctx, float *hdr_rgba, uint16_t *rgba16f);

/* Device pointers of the context's frame buffer (float4 x W*H) and output image (half4 x W*H), valid
 * until the next spk_set_config / spk_destroy. */
spk_status spk_framebuffer_device(spk_ctx *ctx, void **hdr_rgba, void **rgba16f);

/* Camera accumulation counters: samples already folded into the frame buffer (capped at max_spp), and
 * the number of samples dispatched since the last clear (the per-frame seed base). Mirrors
 * CameraRenderProxy::GetCumulatedSampleCount and CPURenderer::dispatched_sample_count_. */
spk_status spk_sample_counts(const spk_ctx *ctx, uint32_t *cumulated, uint32_t *dispatched);

/* Replaces CPURenderer::IsReadyForAutoScreenshot (CPURenderer.cpp:32-36): cumulated >= max_spp. */
int32_t spk_is_converged(const spk_ctx *ctx);

/* Replaces SceneRenderProxy::Intersect<AnyHit> (SceneRenderProxy.cpp:299-309) over a host ray set:
 * closest hit (any_hit = 0) or any hit (any_hit = 1) per ray. `hits` receives num_rays records. */
spk_status spk_trace(spk_ctx *ctx, const spk_ray *rays, uint64_t num_rays, spk_hit *hits, int32_t any_hit);

/* Same query on device-resident rays/hits (arrays of spk_ray / spk_hit in device memory). */
spk_status spk_trace_device(spk_ctx *ctx, const void *d_rays, uint64_t num_rays, void *d_hits, int32_t any_hit);

/* Waits for all work queued on the context stream. */
spk_status spk_synchronize(spk_ctx *ctx);

/* Counters of the last spk_render / spk_trace / spk_trace_device call (waits for it to finish). */
spk_status spk_get_stats(spk_ctx *ctx, spk_stats *out);

/* Measurement hook with no reference counterpart (the reference's only instrumentation is Tracy scopes,
 * libraries/include/core/Profiler.h:9-28): SPK_INSTR_COUNT_TRAFFIC switches the traversal kernels to
 * variants that also count visited nodes and tested triangles (slower; results are unchanged). */
spk_status spk_set_instrumentation(spk_ctx *ctx, uint32_t flags);

/* Default performance knobs. */
void spk_tuning_defaults(spk_tuning *out);

/* Sets / reads the context's performance knobs (see spk_tuning). Rejects out-of-range values with
 * SPK_ERR_INVALID_ARGUMENT and leaves the previous setting in place. */
spk_status spk_set_tuning(spk_ctx *ctx, const spk_tuning *tuning);
spk_status spk_get_tuning(const spk_ctx *ctx, spk_tuning *out);

/* Primary-hit guides for the learned denoiser (spk_denoise.h), the G-buffer the reference's GPU pipeline
 * writes for its denoiser (WritePrimaryHitGBuffer, ray_trace.cs.slang:282-351): one pixel-centre ray per
 * pixel from the camera position (no jitter, no lens); on a hit (t <= 1000) the unit world normal and
 * the linear depth along normalize(cross(max_v, max_u)) (`normal_depth`, float4) and the base colour with
 * 2 for an emissive surface else 1 (`albedo`, float4); zeros on a miss. Rows are ordered like the frame
 * buffer. spk_render_guides is asynchronous; the buffers live until the next spk_set_config. */
spk_status spk_render_guides(spk_ctx *ctx);
spk_status spk_guides_device(spk_ctx *ctx, void **normal_depth, void **albedo);
spk_status spk_read_guides(spk_ctx *ctx, float *normal_depth, float *albedo); /* host or device pointers */

/* One render request of a batch: `scene` (index of spk_set_scenes), an image of width x height, `spp`
 * frames of one sample per pixel (like `spp` spk_render calls at spp = 1 from a cleared accumulation),
 * path depth `bounce`, per-pixel seed `seed`, and its camera. */
typedef struct spk_request {
    uint32_t scene;
    uint32_t width;
    uint32_t height;
    uint32_t spp;
    uint32_t bounce;
    uint32_t seed;
    spk_camera camera;
} spk_request;

/* No reference counterpart. Renders the requests in groups of consecutive whole requests of at most the
 * path slots' sample items (spk_tuning.batch_slots; a larger request alone), each group one regenerating
 * wavefront: the sample items (request, frame, pixel) of its requests are handed to path slots from one
 * counter, so requests of uneven resolution, sample count, depth and scene keep the GPU full together, and a
 * group that fits starts all its samples at once. `rng` and `enable_nee` apply to the whole batch. Each request's frame buffer and tonemapped image are bit-identical to spk_set_config
 * ({width, height, spp = 1, max_spp >= spp, bounce, spatial_denoise = 0, enable_nee, rng, seed}) +
 * spk_set_camera + spk_render(spp) on its scene. Waits for completion; spk_get_stats reports the batch. */
spk_status spk_render_batch(spk_ctx *ctx, const spk_request *requests, uint32_t num_requests, uint32_t rng,
                            uint32_t enable_nee);

/* Copies request `index` of the last batch out (host or device pointers; either may be NULL): its
 * accumulated HDR frame buffer (height rows of width float4, bottom row first) and its tonemapped RGBA16F
 * image (top row first). */
spk_status spk_read_batch(spk_ctx *ctx, uint32_t index, float *hdr_rgba, uint16_t *rgba16f);

/* Largest width * height spk_render_noalloc accepts (512 x 512). */
#define SPK_NOALLOC_MAX_PIXELS (512u * 512u)

/* No counterpart in the reference. Renders `num_frames` frames exactly like spk_render does with the
 * one-kernel schedule (SPK_KERNEL_MEGAKERNEL) -- same scene, camera, config, seeds and sample
 * bookkeeping, bit-identical results -- but without allocating anything: no cudaMalloc, no cudaFree, no
 * event creation. It is meant for callers that cannot allocate device memory while they render: a frame
 * loop that must not stall on the allocator or contend for its lock mid-frame, code that runs while a
 * stream is being captured (allocation is not allowed there), or a host whose device memory is already
 * carved up by its own pool. Set-up still allocates once (spk_create, spk_set_scene, spk_set_config,
 * spk_set_camera must have been called); render time does not.
 *
 * The caller owns the outputs: `d_hdr_rgba` (width*height float4, device memory) is the accumulated frame
 * buffer and is read and written; `d_rgba16f` (width*height half4, device memory) receives the tonemapped
 * image. The context's sample bookkeeping follows one frame buffer at a time: a call whose `d_hdr_rgba`
 * differs from the previous call's (or that follows spk_render) clears it and starts the accumulation
 * over, as a dirty context does; and after such calls spk_render starts over in the context's own buffer,
 * while spk_read_framebuffer, spk_read_rgba8, spk_save_image and spk_save_checkpoint return
 * SPK_ERR_NOT_READY (the context's own buffer holds none of those frames) until spk_render or
 * spk_load_checkpoint runs.
 *
 * The per-frame G-buffer and the counters live in one file-scope device array sized for
 * SPK_NOALLOC_MAX_PIXELS pixels (8 MB plus 256 bytes, held by every GPU that loads the library until the
 * process exits); larger configs return SPK_ERR_INVALID_ARGUMENT. The first call on a device, and the
 * first after that device's context was torn down and created again (cudaDeviceReset), looks up the
 * array's device address (cudaGetSymbolAddress), so make that call before capturing any stream. Every
 * call on a device shares the one array and it keeps the last call's contents (the counters are cleared
 * by each call): calls that overlap on the GPU (two contexts, two streams) race on it and must be
 * serialised by the caller. Asynchronous like spk_render. spk_get_stats after it waits for the stream and
 * reports the call's counters -- rays, paths, launches and spk_stats.error_flags (walk stack bound and
 * iteration budget) -- read from the shared array, so read them before another context's call on the
 * same device; it records no events, so device_ms and trace_kernel_ms are 0. */
spk_status spk_render_noalloc(spk_ctx *ctx, uint32_t num_frames, void *d_hdr_rgba, void *d_rgba16f);

/* ------------------------------------------------------------------------------------------------ */
/* Checkpoint / resume and test hooks                                                               */
/* ------------------------------------------------------------------------------------------------ */

/* No reference counterpart (SessionManager, include/application/SessionManager.h:12-29, keeps the camera
 * and the config only): a render checkpoint holds the accumulation state -- the frame buffer, the output
 * image and CameraRenderProxy / CPURenderer's sample bookkeeping -- so that a long render stops and
 * resumes bit for bit. spk_checkpoint_size gives its byte size for the context's config;
 * spk_save_checkpoint writes it (host or device buffer of at least that size); spk_load_checkpoint
 * restores it into a context with the same spk_config (scene and camera set as at the save, before the
 * load: setting them afterwards restarts the accumulation, as any change does). */
spk_status spk_checkpoint_size(const spk_ctx *ctx, uint64_t *bytes);
spk_status spk_save_checkpoint(spk_ctx *ctx, void *buffer, uint64_t size);
spk_status spk_load_checkpoint(spk_ctx *ctx, const void *buffer, uint64_t size);

/* The acceleration structure of a single-scene context as a blob: every mesh's BLAS (flattened 8-wide
 * nodes and leaf order) tagged with its face / vertex counts, a hash of its positions and indices and the
 * BVH knobs it was built with. spk_set_bvh hands such a blob to a context (host memory, copied): its next
 * spk_set_scene takes each mesh's BLAS from the blob when that mesh and the knobs match, and builds the
 * others; spk_stats.blas_reused counts the reused ones; spk_set_bvh(ctx, NULL, 0) drops the blob. A scene
 * reloaded this way skips the BLAS builds (seconds for large meshes) and gets the same nodes. */
spk_status spk_bvh_blob_size(spk_ctx *ctx, uint64_t *bytes);
spk_status spk_save_bvh(spk_ctx *ctx, void *blob, uint64_t size);
spk_status spk_set_bvh(spk_ctx *ctx, const void *blob, uint64_t size);

/* Test hooks for failure handling, no GPU fault involved. spk_debug_fail_allocation(n): the nth device
 * allocation the library makes from now on fails as out of memory, once (0 disarms); the entry point
 * that made it returns SPK_ERR_OUT_OF_MEMORY and its context stays usable. spk_debug_walk_budget(ctx, n):
 * every ray walk of the context may take at most n node steps (0 = the default 2^20); a walk that runs out
 * ends and sets the iteration-budget bit of spk_stats.error_flags. */
void spk_debug_fail_allocation(uint32_t nth);
spk_status spk_debug_walk_budget(spk_ctx *ctx, uint32_t steps);

/* ------------------------------------------------------------------------------------------------ */
/* Image output (the reference's screenshot flow)                                                   */
/* ------------------------------------------------------------------------------------------------ */

enum { SPK_IMAGE_PNG = 0, SPK_IMAGE_HDR = 1, SPK_IMAGE_EXR = 2 };

/* Image2D::CreateFromRawPixels of the RGBA16F output (ConvertPixelsToRGBA8, libraries/source/io/Image.cpp:
 * 30-67): every colour channel clamped to [0, 1], raised to 0.45 (utilities::LinearToSrgb) and stored as
 * lround(x * 255); alpha without the power. Converted on the device; `rgba8` (width*height*4 bytes, rows
 * top first) is a host or device pointer. */
spk_status spk_read_rgba8(spk_ctx *ctx, uint8_t *rgba8);

/* Renderer::RequestSaveScreenshot + ReadbackFinalOutputIfRequested + Image2D::WriteToFile
 * (libraries/source/renderer/renderer/Renderer.cpp:94-181, Image.cpp:221-275) without the UI: writes
 * `path` as SPK_IMAGE_PNG (the spk_read_rgba8 image, 8-bit RGBA), SPK_IMAGE_HDR (Radiance RGBE of the
 * linear frame buffer, as WriteToFile writes HDR images) or SPK_IMAGE_EXR (the linear frame buffer as
 * half RGBA, uncompressed scanlines). The path is used as given. */
spk_status spk_save_image(spk_ctx *ctx, const char *path, uint32_t format);

/* The encoders on caller images (rows top first): RGBA8 to PNG, float RGBA to Radiance HDR, RGBA16F to
 * OpenEXR; and the RGBA16F -> RGBA8 conversion of spk_read_rgba8 on the host. */
spk_status spk_write_png(const char *path, const uint8_t *rgba8, uint32_t width, uint32_t height);
spk_status spk_write_hdr(const char *path, const float *rgba, uint32_t width, uint32_t height);
spk_status spk_write_exr(const char *path, const uint16_t *rgba16f, uint32_t width, uint32_t height);
spk_status spk_convert_rgba8(const uint16_t *rgba16f, uint64_t pixels, uint8_t *rgba8);

/* SkyLight::SetSkyMap's cube cook (SkyLightCookJob::Execute, scene/component/light/SkyLight.cpp:83-113) on
 * device `device`: the cube_size x cube_size faces (+X, -X, +Y, -Y, +Z, -Z) of the SPK_SKY_CUBE sky the
 * reference samples on a miss, from a width x height equirectangular sky map (RGBA floats as Image2D holds
 * them; `srgb` for an sRGB format, decoded after the filter): each texel centre's direction mapped by
 * CartesianToEquirectangular, the map sampled bilinearly with wrap, rounded to half (RGBAFloat16) with
 * alpha 1. `cube_rgba` receives 6 * cube_size^2 * 4 floats (host or device). The reference cooks 1024. */
spk_status spk_sky_from_equirect(int32_t device, const float *rgba, uint32_t width, uint32_t height, uint32_t srgb,
                                 uint32_t cube_size, float *cube_rgba);

/* ------------------------------------------------------------------------------------------------ */
/* Image evaluation                                                                                   */
/* ------------------------------------------------------------------------------------------------ */

/* The reference's rendering-test score (tests/rendering/render_test_support.py:43-59: mean FLIP of a
 * screenshot against a ground-truth PNG, both read as RGB / 255, LDR-FLIP with sRGB inputs and default
 * parameters) on device `device`: the published LDR-FLIP (Andersson et al. 2020) of two width x height RGB
 * float images in [0, 1] (sRGB-encoded, 3 floats per pixel, host or device pointers).
 * `pixels_per_degree` is the viewing condition (67.02 = 0.7 m from a 0.7 m wide 3840-pixel screen, FLIP's
 * default). Writes the per-pixel error to `error_map` (width*height floats, host or device) when it is
 * not NULL and the mean to *mean_error. */
spk_status spk_flip(int32_t device, const float *reference_rgb, const float *test_rgb, uint32_t width,
                    uint32_t height, float pixels_per_degree, float *error_map, double *mean_error);

/* relMSE = mean over the `count` values of (x - ref)^2 / (ref^2 + eps) (the metric of the denoiser
 * benchmark, eps = 0.01), on device `device`; host or device pointers. */
spk_status spk_relmse(int32_t device, const float *x, const float *reference, uint64_t count, float eps,
                      double *out);

#ifdef __cplusplus
}
#endif

#endif /* SPK_H_ */
