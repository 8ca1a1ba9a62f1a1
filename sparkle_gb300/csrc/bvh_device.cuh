// bvh_device.cuh -- BVH work on the device: refitting a mesh's BLAS after its vertices move, and building one.
//
// Sparkle builds a mesh's BLAS once, in local space, when the primitive is created and rebuilds the TLAS on
// every primitive change (SceneRenderProxy.cpp:269-297, MeshRenderProxy.cpp:52-92). A deforming mesh (same
// faces, new vertex positions) keeps its tree here: the triangle records are rewritten from the new
// positions and the 8-wide nodes are refitted level by level, deepest first, each child box re-quantised
// exactly as the host builder quantises it (so a refit with unchanged positions reproduces the nodes bit
// for bit). Traversal results never depend on the tree's shape, only its conservativeness.
//
// It also builds a mesh's BLAS on the device (spk_tuning.bvh_builder = 1) in place of the host's binned SAH
// build: a linear BVH (Karras, "Maximizing Parallelism in the Construction of BVHs, Octrees, and k-d Trees",
// HPG 2012) over 63-bit Morton codes of the triangle centroids, sorted by a stable LSD radix sort (face index
// breaks ties), boxes propagated bottom-up with one atomic counter per node, then collapsed into 8-wide nodes
// breadth first, one launch per level, with the host collapse's rules (open the largest-area inner child
// until 8, subtrees of <= leaf-size triangles become leaves, octant slot order, the same quantisation).
// Every step is deterministic: the same mesh gives the same nodes. spk_tuning.bvh_builder = 2 replaces the
// radix tree by PLOC clustering (Meister and Bittner 2018) over the same Morton order.
#pragma once

#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "bvh_builder.h"

namespace spk {

struct BlasRefit {
    uint4 *nodes;           // the scene's node array (80 B = 5 x uint4 per node)
    float *boxes;           // scratch: 6 floats (lo, hi) per node of this BLAS, relative to `root`
    float4 *tris;           // the scene's triangle records (3 x float4 each)
    const uint4 *faces;     // the mesh's faces (vertex indices, mesh-local)
    const float *positions; // the mesh's new vertex positions (3 floats each, device)
    uint32_t root;          // first node of the BLAS
    uint32_t node_count;    // nodes of the BLAS
    uint32_t tri_first;     // first triangle record of the BLAS
    uint32_t tri_count;
    uint32_t num_faces, num_vertices;  // bounds of `faces` and `positions`
};

// Rewrites the BLAS's triangle records (p0, e1 = p1 - p0, e2 = p2 - p0; BLAS::Triangle::Set,
// MeshRenderProxy.cpp:80-86) from the new positions.
cudaError_t launch_refit_triangles(const BlasRefit &r, cudaStream_t stream);

// Refits the nodes root + [first, last): one depth of the breadth-first node order the builders emit,
// launched deepest depth first so that every inner child is refitted before its parent.
cudaError_t launch_refit_nodes(const BlasRefit &r, uint32_t first, uint32_t last, cudaStream_t stream);

// Writes new normals (and, when given, tangents xyzw) into the vertex records verts[3*(vert_base + v)].
cudaError_t launch_update_vertices(float4 *verts, uint32_t vert_base, uint32_t num_vertices, const float *normals,
                                   const float *tangents, cudaStream_t stream);

// Builds the 8-wide BLAS of one mesh on the device, from the Karras radix tree of the Morton-sorted faces
// or, with `clustered`, from a PLOC agglomerative clustering of them (tighter trees, a few more rounds). positions [num_vertices][3] and indices [num_faces][3]
// are host arrays (indices already checked against num_vertices). `out` receives the nodes (node 0 the
// root, children after their parent depth by depth) and the leaf items (face indices) as the host builder
// returns them; `levels` the first node of each depth, then the node count. `max_children` 2..8,
// `max_leaf` 1..3.
cudaError_t build_wide_device(const float *positions, uint32_t num_vertices, const uint32_t *indices,
                              uint32_t num_faces, int max_children, int max_leaf, bool clustered, cudaStream_t stream,
                              WideBvh &out, std::vector<uint32_t> &levels);

}  // namespace spk
