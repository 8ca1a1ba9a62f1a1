// bvh_builder.h -- host BVH construction for the device traversal.
//
// Stands in for SceneRenderProxy/MeshRenderProxy's use of bvh v2's DefaultBuilder (SceneRenderProxy.cpp:55-57,
// MeshRenderProxy.cpp:62-64): a binned-SAH binary BVH is built on the host, then collapsed into 8-wide nodes
// whose child boxes are quantised to 8 bits relative to the node box (80 bytes per node, read on the device
// as five 128-bit loads). Child slots are ordered by octant so that a ray visits hit children roughly near
// to far by visiting permuted slot indices in ascending order. Leaves hold at most 3 items (triangles for a
// BLAS, instances for the TLAS); an 8-wide node addresses at most 24 leaf items through one 24-bit mask.
#pragma once

#include <cstdint>
#include <vector>

namespace spk {

struct BuildBox {
    float lo[3], hi[3];
};

struct Bvh2Node {
    float lo[3], hi[3];
    uint32_t first;  // inner: left child index (right = first + 1); leaf: first item in `items`
    uint32_t count;  // 0 for inner nodes
};

struct Bvh2 {
    std::vector<Bvh2Node> nodes;
    std::vector<uint32_t> items;
};

// Binned SAH (32 bins, traversal cost 1 : item cost 1), at most `max_leaf` items per leaf.
Bvh2 build_bvh2(const std::vector<BuildBox> &boxes, uint32_t max_leaf, int num_threads);

// 80-byte quantised 8-wide node. Layout (bytes): p[3] f32 @0, biased exponents ex,ey,ez @12, imask @15,
// child_base @16, item_base @20, meta[8] @24, qlo_x @32, qlo_y @40, qlo_z @48, qhi_x @56, qhi_y @64,
// qhi_z @72. meta per slot: 0 = empty; inner = 0x20 | (24 + slot); leaf = (unary count << 5) | offset.
struct alignas(16) WideNode {
    float p[3];
    uint8_t e[3];
    uint8_t imask;
    uint32_t child_base;
    uint32_t item_base;
    uint8_t meta[8];
    uint8_t qlo[3][8];
    uint8_t qhi[3][8];
};
static_assert(sizeof(WideNode) == 80, "wide node must be 80 bytes");

struct WideBvh {
    std::vector<WideNode> nodes;  // node 0 is the root
    std::vector<uint32_t> items;  // leaf items in leaf order (wide leaves address item_base + offset)
};

// Collapses a binary BVH (leaves of <= 3 items) into 8-wide quantised nodes.
// `max_children` (2..8) caps the children opened per wide node; fewer children give smaller effective
// fan-out (more, emptier nodes) in the same 80-byte record.
WideBvh collapse_wide(const Bvh2 &bvh, int max_children = 8);

// SAH-optimal collapse (the dynamic program of Ylitie, Karras and Laine, "Efficient Incoherent Ray
// Traversal on GPUs Through Compressed Wide BVHs", HPG 2017): for every binary node and every k <= 8 the
// cheapest way to represent its subtree as at most k roots, each root a leaf of <= `max_leaf` items or a
// wide node; cost = half area x (1 per wide node, 0.3 per item). Best on a binary BVH with one item per leaf,
// so that the program also chooses the leaf sizes.
WideBvh collapse_wide_sah(const Bvh2 &bvh, int max_children = 8, int max_leaf = 3);

}  // namespace spk
