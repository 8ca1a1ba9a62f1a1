// device_scene.cuh -- layout of the resident scene in device memory.
//
//  nodes     : WideNode[]   80 B each, BLAS nodes of every mesh followed by the TLAS nodes
//  tris      : float4[3*T]  48 B per triangle in BLAS leaf order: {p0.xyz, e1.x} {e1.yz, e2.xy}
//                           {e2.z, face id, -, -}; p0/e1/e2 are BLAS::Triangle (MeshRenderProxy.cpp:78-92)
//  tlas_items: uint32[]     instance index per TLAS leaf slot (TLAS::Build's prim_ids reorder)
//  instances : DevInstance[] caller order
//  verts     : float4[3*V]  48 B per vertex {n.xyz, t.x} {t.yzw, uv.x} {uv.y, -, -, -}
//  faces     : uint4[F]     vertex indices of each face (w unused), per-mesh ranges
//  materials : DevMaterial[]
//  sky cube  : float4[6*N*N]
#pragma once

#include <cstdint>

#include "spk_math.cuh"

namespace spk {

struct alignas(16) DevInstance {
    float m[12];     // transform rows
    float minv[12];  // inverse transform rows
    uint32_t type;   // SPK_PRIM_MESH / SPK_PRIM_SPHERE
    uint32_t blas_root;
    uint32_t material;
    float radius;
    uint32_t vert_base;  // first vertex of the mesh in `verts`
    uint32_t face_base;  // first face of the mesh in `faces`
    uint32_t normal_map;  // the material's normal-map texture (kInvalid for none), read with the instance
    uint32_t light_base;  // first entry of this instance's triangles in `lights`, kInvalid if it does not emit
};
static_assert(sizeof(DevInstance) == 128, "DevInstance is 128 bytes");

// A texture in the shared texel array (Image2D, io/Image.h:112-150).
struct DevTexture {
    uint32_t offset;  // first texel in `texels`
    uint32_t width, height;
    uint32_t srgb;
};

struct alignas(16) DevMaterial {
    float base[3];
    uint32_t type;
    float emissive[3];
    uint32_t is_emissive;  // ||emissive|| > Eps, evaluated once on the host exactly as SamplePixel does
    float metallic, roughness, eta, pad;
    // texture maps (indices into DevScene::textures, kInvalid for none): base colour, metallic-roughness,
    // emissive, normal
    uint32_t tex_base, tex_mr, tex_emissive, tex_normal;
};
static_assert(sizeof(DevMaterial) == 64, "DevMaterial is 64 bytes");

// An emissive triangle in world space for next-event estimation (64 B).
struct alignas(16) DevLight {
    float p0[3], e1[3], e2[3], ng[3], emission[3];
    float area;
};
static_assert(sizeof(DevLight) == 64, "DevLight is 64 bytes");

// One scene of a context holding several (spk_set_scenes): its TLAS root in the shared node array, its
// sky, and its slice of the shared light table. Instance light_base indices are relative to the slice.
struct DevSceneDesc {
    uint32_t tlas_root;
    uint32_t sky_mode, sky_size;
    float sky_color[3];
    uint32_t sky_offset;   // first texel of the scene's cube in sky_cube
    uint32_t light_base;   // first entry of the scene's lights / light_cdf
    uint32_t num_lights;
    float light_total;
};

struct DevScene {
    const DevLight *lights;   // emissive triangles of mesh instances, instance then face order
    const float *light_cdf;   // running sum of light areas
    uint32_t num_lights;
    float light_total;        // total emissive area
    const uint4 *nodes;
    const float4 *tris;
    const uint32_t *tlas_items;
    const DevInstance *instances;
    const float4 *verts;
    const uint4 *faces;
    const DevMaterial *materials;
    const float4 *sky_cube;
    uint32_t tlas_root;  // kInvalid for an empty scene
    uint32_t sky_mode;
    uint32_t sky_size;
    float sky_color[3];
    float scene_abs_x;  // max |x| over world bounds; bounds the x-only world-t error used for pruning
    const DevTexture *textures;  // all scenes' textures
    const float4 *texels;        // their texels, texture after texture
    const DevSceneDesc *descs;  // every scene of the context (the fields above are scene 0's)
    uint32_t num_scenes;
    float box_lo[3];     // world bounds of all scenes (ray sort cells)
    float box_scale[3];  // 8 / extent per axis (0 for a flat axis)
    uint32_t walk_budget;  // node steps a walk may take before it reports kErrIterationBudget; 0 = 2^20
};

// The DevScene of scene `k` of a multi-scene context: scene 0's record with the TLAS root, sky and light
// table of scene k. Everything else (nodes, triangles, instances, materials) is shared.
__host__ __device__ inline DevScene scene_view(const DevScene &S, const DevSceneDesc &d) {
    DevScene v = S;
    v.tlas_root = d.tlas_root;
    v.sky_mode = d.sky_mode;
    v.sky_size = d.sky_size;
    v.sky_color[0] = d.sky_color[0];
    v.sky_color[1] = d.sky_color[1];
    v.sky_color[2] = d.sky_color[2];
    v.sky_cube = S.sky_cube + d.sky_offset;
    v.lights = S.lights + d.light_base;
    v.light_cdf = S.light_cdf + d.light_base;
    v.num_lights = d.num_lights;
    v.light_total = d.light_total;
    return v;
}

}  // namespace spk
