/*
 * oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * C API of the CPU oracle: a plain C++ restatement of Sparkle's CPU path tracer (the `cpu` pipeline:
 * libraries/source/renderer/renderer/CPURenderer.cpp, SceneRenderProxy.cpp, MeshRenderProxy.cpp,
 * SphereRenderProxy.cpp, libraries/include/core/math/{Sampler,Utilities,Ray,Intersection}.h,
 * libraries/include/scene/material/BxDF.h and the material proxies). It is the checker the GPU path is
 * compared against and the CPU baseline that bench.py times; nothing in the product links it.
 *
 * PARITY UNPINNED against upstream: the reference cannot be built here (its bvh, Xoshiro-cpp and Eigen
 * submodules are empty) and its tests hold no golden vectors for this path, so this restatement is
 * pinned by its own committed fixtures and by an independent Python restatement on small cases.
 *
 * The scene input uses the POD structs of include/spk.h (the data format only).
 */
#ifndef SPK_ORACLE_H_
#define SPK_ORACLE_H_

#include "spk.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_scene or_scene;
typedef struct or_renderer or_renderer;

enum { OR_TRAVERSAL_FAITHFUL = 0, OR_TRAVERSAL_PRUNED = 1 };

/* Builds every BLAS and the TLAS (binned SAH BVH2, restating SceneRenderProxy::UpdateBVH). */
or_scene *or_scene_create(const spk_mesh *meshes, uint32_t num_meshes, const spk_instance *instances,
                          uint32_t num_instances, const spk_material *materials, uint32_t num_materials,
                          const spk_sky *sky);
void or_scene_destroy(or_scene *scene);

/* SceneRenderProxy::Intersect<AnyHit> over a ray set; returns the number of traversal-stack overflows. */
uint64_t or_trace(const or_scene *scene, const spk_ray *rays, uint64_t num_rays, spk_hit *hits, int32_t any_hit,
                  int32_t traversal, int32_t num_threads);

/* Brute-force closest hit over every triangle and sphere (tree-independent check of or_trace). */
void or_trace_brute(const or_scene *scene, const spk_ray *rays, uint64_t num_rays, spk_hit *hits,
                    int32_t num_threads);

/* CPURenderer with the cpu pipeline's passes; frames are rendered exactly as Render() does. */
or_renderer *or_renderer_create(const or_scene *scene, const spk_config *config, const spk_camera *camera);
void or_renderer_destroy(or_renderer *r);
/* Renders `num_frames` frames; rows [row_begin, row_end) only when row_end > row_begin (timing samples;
 * the other rows are left untouched and the accumulation bookkeeping still advances). */
void or_render(or_renderer *r, uint32_t num_frames, int32_t traversal, int32_t num_threads, uint32_t row_begin,
               uint32_t row_end);
/* As or_render over rows row_begin, row_begin + row_step, ... below row_end (timing samples spread over
 * the image). */
void or_render_rows(or_renderer *r, uint32_t num_frames, int32_t traversal, int32_t num_threads, uint32_t row_begin,
                    uint32_t row_end, uint32_t row_step);
void or_read_framebuffer(const or_renderer *r, float *hdr_rgba, uint16_t *rgba16f);
/* Per-pixel G-buffer of the last frame: color (rgb, valid flag) and first-hit world normal. */
void or_read_gbuffer(const or_renderer *r, float *color_rgba, float *world_normal);
void or_guides(const or_renderer *r, float *normal_depth, float *albedo_hit);
void or_scene_set_textures(or_scene *sc, const spk_texture *textures, uint32_t num_textures,
                           const spk_material_maps *maps);
void or_counts(const or_renderer *r, uint64_t *extension_rays, uint64_t *shadow_rays, uint64_t *paths);
void or_sample_counts(const or_renderer *r, uint32_t *cumulated, uint32_t *dispatched);

/* Hooks for unit tests of the restated pieces. */
void or_rng_fill(int32_t kind, uint64_t seed, uint32_t n, uint32_t *out_u32, float *out_unit);
uint32_t or_float_to_half(float f);
/* One PbrMaterialRenderProxy / DieletricMaterialRenderProxy::SampleSurface draw with a Xoshiro128+ seeded
 * from `seed`: out[0..2] throughput, out[3..5] world w_i, out[6] = number of RandomUnit() draws. */
void or_sample_surface(const spk_material *m, const float ray_dir[3], const float normal[3], const float tangent[3],
                       uint32_t seed, float out[7]);

#ifdef __cplusplus
}
#endif

#endif
