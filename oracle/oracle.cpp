// oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of Sparkle's `cpu` path-tracing pipeline, used as the checker of the GPU path (tests/,
// __graft_entry__.smoke) and as the timed CPU baseline of bench.py. Nothing in the product links it.
// Every function cites the reference lines it restates (paths relative to the Sparkle tree; a bare file
// name lives under libraries/). PARITY UNPINNED against upstream: the reference does not build here
// (thirdparty/bvh, Xoshiro-cpp and Eigen are empty submodules) and its tests hold no golden vectors for
// this path. What pins this file instead: an independent numpy / pure-Python restatement of the same
// reference lines (tests/test_oracle.py) and the committed golden streams, hits and images it must keep
// reproducing (tests/golden/).
//
// Floating-point conventions (compiled with -ffp-contract=off, no -ffast-math):
//  * Eigen 3.x evaluates a fixed-size 3-term reduction (dot, squaredNorm, a row of a 3x3 product) as
//    x0 + (x1 + x2) (its unrolled redux splits the range in halves); dot3/sum3 below follow that order.
//  * Eigen's normalized() divides each component by sqrt(squaredNorm) when squaredNorm > 0.
//  * bvh v2's box test uses fast_mul_add; this file uses std::fma (the FP_FAST_FMAF form taken on
//    aarch64 hosts) so the box test is the same on every host.
//  * std::min/std::max/std::clamp keep their operand-order NaN behaviour (written out as ternaries).

#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

// ------------------------------------------------------------------------------------------------
// Vector math (libraries/include/core/math/Types.h, Utilities.h) in Eigen's evaluation order
// ------------------------------------------------------------------------------------------------
struct V3 {
    float x, y, z;
};
struct V4 {
    float x, y, z, w;
};

constexpr float kEps = 1e-6f;        // Types.h:54 Eps
constexpr float kTolerance = 1e-4f;  // Types.h:55 Tolerance
constexpr float kPi = 3.14159265358979323846f;  // std::numbers::pi_v<float> (Types.h:51)
constexpr float kInvSqrt3 = 0.577350269189625764509f;  // std::numbers::inv_sqrt3_v<float> (Types.h:56)
constexpr float kInvPi = 0.318309886183790671538f;     // std::numbers::inv_pi_v<float> (Types.h:52)
constexpr float kOutputLimit = 6.f;  // CameraRenderProxy.h:16

inline V3 mk(float x, float y, float z) { return {x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 cmul(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline float sum3(float a, float b, float c) { return a + (b + c); }
inline float dot3(V3 a, V3 b) { return sum3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float sqnorm(V3 a) { return dot3(a, a); }
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline V3 normalized(V3 a) {
    const float z = sqnorm(a);
    if (z > 0.f) {
        const float s = std::sqrt(z);
        return {a.x / s, a.y / s, a.z / s};
    }
    return a;
}
inline float min_std(float a, float b) { return (b < a) ? b : a; }  // std::min(a, b)
inline float max_std(float a, float b) { return (a < b) ? b : a; }  // std::max(a, b)
inline V3 load3(const float *p) { return {p[0], p[1], p[2]}; }
// RenderPixel's clamp min(c, OutputLimit) (CPURenderer.cpp:408) with one deliberate deviation: a non-finite
// component becomes 0 instead of entering the running mean as NaN for good. NaN samples come from Refract
// (Utilities.h:213-220, no total-internal-reflection guard) when RandomUnit() returns exactly 1.0 or when
// FrDielectric's `sin_t >= 1` test and Refract's sin^2 round differently at the critical angle.
inline float clamp_sample(float c) { return (c - c == 0.f) ? min_std(c, kOutputLimit) : 0.f; }

// Affine transform rows (3x4, row-major). TransformPoint = t + L*p (Eigen's transform_right_product_impl:
// res = translation; res += linear * p), TransformDirection = L*d (Transform.h:95-103).
struct Affine {
    float m[12];
};
inline V3 xform_point(const Affine &a, V3 p) {
    const float *m = a.m;
    return {m[3] + sum3(m[0] * p.x, m[1] * p.y, m[2] * p.z), m[7] + sum3(m[4] * p.x, m[5] * p.y, m[6] * p.z),
            m[11] + sum3(m[8] * p.x, m[9] * p.y, m[10] * p.z)};
}
inline V3 xform_dir(const Affine &a, V3 d) {
    const float *m = a.m;
    return {sum3(m[0] * d.x, m[1] * d.y, m[2] * d.z), sum3(m[4] * d.x, m[5] * d.y, m[6] * d.z),
            sum3(m[8] * d.x, m[9] * d.y, m[10] * d.z)};
}

// ------------------------------------------------------------------------------------------------
// RNG: Sampler.h:16-53. Xoshiro128+ (Blackman & Vigna, public-domain reference algorithm) seeded through
// SplitMix64 the way Xoshiro-cpp's 32-bit generators are documented to be (each state word is the low 32
// bits of one SplitMix64 output; unverifiable here, the library is absent). xoshiro256** is the second
// policy (same authors); its state is four SplitMix64 outputs.
// ------------------------------------------------------------------------------------------------
inline uint64_t splitmix64_next(uint64_t &s) {
    s += 0x9E3779B97F4A7C15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline uint32_t rotl32(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }
inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

struct Rng {
    int kind = SPK_RNG_XOSHIRO128P;
    uint32_t s32[4] = {0, 0, 0, 0};
    uint64_t s64[4] = {0, 0, 0, 0};
    uint32_t draws = 0;

    void seed128(uint64_t seed) {
        kind = SPK_RNG_XOSHIRO128P;
        uint64_t sm = seed;
        for (auto &w : s32) w = static_cast<uint32_t>(splitmix64_next(sm));
    }
    void seed256(uint64_t seed) {
        kind = SPK_RNG_XOSHIRO256SS;
        uint64_t sm = seed;
        for (auto &w : s64) w = splitmix64_next(sm);
    }
    uint32_t next_u32() {
        if (kind == SPK_RNG_XOSHIRO128P) {
            const uint32_t result = s32[0] + s32[3];
            const uint32_t t = s32[1] << 9;
            s32[2] ^= s32[0];
            s32[3] ^= s32[1];
            s32[1] ^= s32[2];
            s32[0] ^= s32[3];
            s32[2] ^= t;
            s32[3] = rotl32(s32[3], 11);
            return result;
        }
        const uint64_t result = rotl64(s64[1] * 5, 7) * 9;
        const uint64_t t = s64[1] << 17;
        s64[2] ^= s64[0];
        s64[3] ^= s64[1];
        s64[1] ^= s64[2];
        s64[0] ^= s64[3];
        s64[2] ^= t;
        s64[3] = rotl64(s64[3], 45);
        return static_cast<uint32_t>(result >> 32);
    }
    // RandomUnit: float(u32) / float(UINT32_MAX); float(4294967295u) rounds to 2^32 (Sampler.h:32-41).
    float unit() {
        ++draws;
        return static_cast<float>(next_u32()) / static_cast<float>(std::numeric_limits<uint32_t>::max());
    }
};

// Per-pixel seeding. Reference policy: ReseedCurrentThread(j*W + i + frame_seed*W*H) in 32-bit unsigned
// arithmetic (CPURenderer.cpp:442-443, Sampler.h:27-30). xoshiro256** policy: SplitMix64 state
// (seed << 40) ^ (64-bit sample index frame_seed*W*H + j*W + i), no wrap.
inline void seed_pixel(Rng &rng, int kind, uint32_t seed, uint32_t i, uint32_t j, uint32_t w, uint32_t h,
                       uint32_t frame_seed) {
    if (kind == SPK_RNG_XOSHIRO128P) {
        const uint32_t s = j * w + i + frame_seed * w * h;
        rng.seed128(static_cast<uint64_t>(s));
    } else {
        const uint64_t idx = static_cast<uint64_t>(frame_seed) * w * h + static_cast<uint64_t>(j) * w + i;
        rng.seed256((static_cast<uint64_t>(seed) << 40) ^ idx);
    }
    rng.draws = 0;
}

// UnitDisk (Sampler.h:43-53): r = sqrt(u1), theta = (u2 * 2) * Pi.
inline void unit_disk(Rng &rng, float &x, float &y) {
    const float rand = rng.unit();
    const float theta = rng.unit() * 2.0f * kPi;
    const float r = std::sqrt(rand);
    x = r * std::cos(theta);
    y = r * std::sin(theta);
}

// ------------------------------------------------------------------------------------------------
// BVH2: binned-SAH top-down builder standing in for bvh v2's DefaultBuilder (absent) and bvh v2's
// Bvh::intersect traversal (near-first, explicit stack, root box never tested, non-robust slab test).
// ------------------------------------------------------------------------------------------------
struct Node2 {
    float b[6];  // min_x, max_x, min_y, max_y, min_z, max_z (bvh::v2::Node bounds order)
    uint32_t first;  // leaf: first index into prim_ids; inner: left child (right = first + 1)
    uint32_t count;  // > 0 for leaves
};
struct Bvh2 {
    std::vector<Node2> nodes;
    std::vector<uint32_t> prim_ids;
};

struct Box {
    float lo[3], hi[3];
};
inline Box empty_box() {
    Box b;
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = std::numeric_limits<float>::max();
        b.hi[k] = -std::numeric_limits<float>::max();
    }
    return b;
}
inline void grow(Box &b, const Box &o) {
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = std::min(b.lo[k], o.lo[k]);
        b.hi[k] = std::max(b.hi[k], o.hi[k]);
    }
}
inline float half_area(const Box &b) {
    const float dx = std::max(0.f, b.hi[0] - b.lo[0]), dy = std::max(0.f, b.hi[1] - b.lo[1]),
                dz = std::max(0.f, b.hi[2] - b.lo[2]);
    return dx * dy + dy * dz + dz * dx;
}

Bvh2 build_bvh2(const std::vector<Box> &boxes, const std::vector<V3> &centers) {
    constexpr int kBins = 16;
    constexpr uint32_t kMaxLeaf = 4;
    Bvh2 bvh;
    const uint32_t n = static_cast<uint32_t>(boxes.size());
    if (n == 0) return bvh;
    bvh.prim_ids.resize(n);
    for (uint32_t i = 0; i < n; ++i) bvh.prim_ids[i] = i;
    bvh.nodes.reserve(2 * n);
    bvh.nodes.push_back({});
    struct Task {
        uint32_t node, begin, end;
    };
    std::vector<Task> work{{0, 0, n}};
    while (!work.empty()) {
        const Task t = work.back();
        work.pop_back();
        Box nb = empty_box(), cb = empty_box();
        for (uint32_t i = t.begin; i < t.end; ++i) {
            const uint32_t p = bvh.prim_ids[i];
            grow(nb, boxes[p]);
            const Box c{{centers[p].x, centers[p].y, centers[p].z}, {centers[p].x, centers[p].y, centers[p].z}};
            grow(cb, c);
        }
        Node2 &node = bvh.nodes[t.node];
        for (int k = 0; k < 3; ++k) {
            node.b[2 * k] = nb.lo[k];
            node.b[2 * k + 1] = nb.hi[k];
        }
        const uint32_t count = t.end - t.begin;
        auto make_leaf = [&]() {
            node.first = t.begin;
            node.count = count;
        };
        if (count == 1) {
            make_leaf();
            continue;
        }
        // SAH over centroid bins on every axis (traversal cost 1, intersection cost 1).
        float best_cost = std::numeric_limits<float>::max();
        int best_axis = -1, best_split = -1;
        for (int axis = 0; axis < 3; ++axis) {
            const float lo = cb.lo[axis], ext = cb.hi[axis] - cb.lo[axis];
            if (!(ext > 0.f)) continue;
            Box bin_box[kBins];
            uint32_t bin_cnt[kBins] = {};
            for (auto &bb : bin_box) bb = empty_box();
            const float scale = kBins / ext;
            for (uint32_t i = t.begin; i < t.end; ++i) {
                const uint32_t p = bvh.prim_ids[i];
                const float c = axis == 0 ? centers[p].x : axis == 1 ? centers[p].y : centers[p].z;
                int bi = static_cast<int>((c - lo) * scale);
                bi = std::min(std::max(bi, 0), kBins - 1);
                bin_cnt[bi]++;
                grow(bin_box[bi], boxes[p]);
            }
            float right_area[kBins];
            uint32_t right_cnt[kBins];
            Box acc = empty_box();
            uint32_t cnt = 0;
            for (int b = kBins - 1; b > 0; --b) {
                grow(acc, bin_box[b]);
                cnt += bin_cnt[b];
                right_area[b] = half_area(acc);
                right_cnt[b] = cnt;
            }
            acc = empty_box();
            cnt = 0;
            for (int b = 0; b < kBins - 1; ++b) {
                grow(acc, bin_box[b]);
                cnt += bin_cnt[b];
                if (cnt == 0 || right_cnt[b + 1] == 0) continue;
                const float cost = half_area(acc) * cnt + right_area[b + 1] * right_cnt[b + 1];
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = axis;
                    best_split = b;
                }
            }
        }
        const float leaf_cost = half_area(nb) * count;
        const float split_cost = half_area(nb) + best_cost;
        uint32_t mid;
        if (best_axis < 0) {
            if (count <= kMaxLeaf) {
                make_leaf();
                continue;
            }
            mid = t.begin + count / 2;  // coincident centroids: split by index
        } else {
            if (count <= kMaxLeaf && leaf_cost <= split_cost) {
                make_leaf();
                continue;
            }
            const float lo = cb.lo[best_axis], scale = kBins / (cb.hi[best_axis] - cb.lo[best_axis]);
            auto it = std::partition(bvh.prim_ids.begin() + t.begin, bvh.prim_ids.begin() + t.end, [&](uint32_t p) {
                const float c = best_axis == 0 ? centers[p].x : best_axis == 1 ? centers[p].y : centers[p].z;
                int bi = static_cast<int>((c - lo) * scale);
                bi = std::min(std::max(bi, 0), kBins - 1);
                return bi <= best_split;
            });
            mid = static_cast<uint32_t>(it - bvh.prim_ids.begin());
            if (mid == t.begin || mid == t.end) mid = t.begin + count / 2;
        }
        const uint32_t left = static_cast<uint32_t>(bvh.nodes.size());
        bvh.nodes[t.node].first = left;
        bvh.nodes[t.node].count = 0;
        bvh.nodes.push_back({});
        bvh.nodes.push_back({});
        work.push_back({left + 1, mid, t.end});
        work.push_back({left, t.begin, mid});
    }
    return bvh;
}

// bvh v2 utils: safe_inverse, robust_min/robust_max (return the right operand when the left is NaN).
inline float safe_inverse(float x) {
    return std::fabs(x) <= std::numeric_limits<float>::epsilon()
               ? std::copysign(std::numeric_limits<float>::max(), x)
               : 1.f / x;
}
inline float robust_min(float a, float b) { return a < b ? a : b; }
inline float robust_max(float a, float b) { return a > b ? a : b; }

struct TravRay {
    float org[3], inv[3], inv_org[3];
    int oct[3];
    float tmin, tmax;
};
inline TravRay make_trav_ray(V3 o, V3 d) {
    TravRay r;
    const float org[3] = {o.x, o.y, o.z}, dir[3] = {d.x, d.y, d.z};
    for (int k = 0; k < 3; ++k) {
        r.org[k] = org[k];
        r.inv[k] = safe_inverse(dir[k]);
        r.inv_org[k] = -r.inv[k] * org[k];
        r.oct[k] = std::signbit(dir[k]) ? 1 : 0;
    }
    r.tmin = 0.f;  // bvh::v2::Ray defaults: tmin = 0, tmax = max float
    r.tmax = std::numeric_limits<float>::max();
    return r;
}
// Node::intersect_fast + make_intersection_result.
inline void box_interval(const Node2 &n, const TravRay &r, float &t0, float &t1) {
    t0 = r.tmin;
    t1 = r.tmax;
    for (int k = 0; k < 3; ++k) {
        const float near_b = n.b[2 * k + r.oct[k]], far_b = n.b[2 * k + 1 - r.oct[k]];
        const float tn = std::fma(near_b, r.inv[k], r.inv_org[k]);
        const float tf = std::fma(far_b, r.inv[k], r.inv_org[k]);
        t0 = robust_max(tn, t0);
        t1 = robust_min(tf, t1);
    }
}

constexpr int kStack = 64;  // bvh v2 SmallStack<..., 32> in the reference; 64 here, overflow is counted

// Bvh::intersect<AnyHit, false>. `leaf(begin, end)` returns whether something was hit so far; the
// pruned traversal lets the leaf lower `r.tmax` (the faithful one never does).
template <bool AnyHit, class Leaf>
void traverse(const Bvh2 &bvh, TravRay &r, Leaf &&leaf, uint64_t &overflows) {
    if (bvh.nodes.empty()) return;
    uint32_t stack[kStack];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        uint32_t top = stack[--sp];
        bool dead = false;
        while (bvh.nodes[top].count == 0) {
            const uint32_t li = bvh.nodes[top].first, ri = li + 1;
            float l0, l1, r0, r1;
            box_interval(bvh.nodes[li], r, l0, l1);
            box_interval(bvh.nodes[ri], r, r0, r1);
            const bool hit_l = l0 <= l1, hit_r = r0 <= r1;
            if (hit_l) {
                uint32_t near_i = li;
                if (hit_r) {
                    uint32_t far_i = ri;
                    if (!AnyHit && l0 > r0) std::swap(near_i, far_i);
                    if (sp < kStack) {
                        stack[sp++] = far_i;
                    } else {
                        ++overflows;
                    }
                }
                top = near_i;
            } else if (hit_r) {
                top = ri;
            } else {
                dead = true;
                break;
            }
        }
        if (dead) continue;
        const bool was_hit = leaf(bvh.nodes[top].first, bvh.nodes[top].first + bvh.nodes[top].count);
        if (AnyHit && was_hit) return;
    }
}

// ------------------------------------------------------------------------------------------------
// Scene: meshes with BLAS (MeshRenderProxy.cpp:24-199), instances, TLAS (SceneRenderProxy.cpp:24-131)
// ------------------------------------------------------------------------------------------------
struct Tri {
    V3 p0, e1, e2;  // BLAS::Triangle::Set (MeshRenderProxy.cpp:80-86); n is never read by the test
};
struct MeshData {
    std::vector<V3> pos, nrm;
    std::vector<V4> tan;
    std::vector<float> uv;  // 2 per vertex, empty if none
    std::vector<uint32_t> idx;
    bool has_tan = false, has_uv = false;
    std::vector<Tri> tris;
    Bvh2 bvh;
    V3 bound_center, bound_half;
};
struct Inst {
    spk_instance desc;
    Affine M, Minv;
    Box world_box;
};
struct Candidate {  // IntersectionCandidate (Intersection.h:90-103)
    float t = std::numeric_limits<float>::max();
    float u = 0.f, v = 0.f;
    uint32_t face = SPK_INVALID_ID;
    int32_t slot = -1;  // TLAS slot of the winning primitive
};
struct Hit {  // Intersection (Intersection.h:9-88) after GetIntersection
    bool hit = false;
    float t = 0.f;
    V3 location, normal, tangent;
    float uv[2] = {0.f, 0.f};
    uint32_t prim = SPK_INVALID_ID;
};

}  // namespace

struct or_scene {
    std::vector<MeshData> meshes;
    std::vector<Inst> insts;          // caller order
    std::vector<uint32_t> tlas_slot;  // TLAS slot -> caller instance index (prim_ids reorder)
    Bvh2 tlas;
    std::vector<spk_material> materials;
    spk_sky sky{};
    std::vector<float> cube;
    float scene_abs_x = 0.f;  // max |x| of any world box, bounds the x-quirk error of world t
    // Next-event estimation: emissive triangles in world space, their area CDF, and per-instance first
    // light index (SPK_INVALID_ID when the instance does not emit).
    struct Light {
        V3 p0, e1, e2, ng, emission;
        float area;
    };
    std::vector<Light> lights;
    std::vector<float> light_cdf;
    float light_total = 0.f;
    std::vector<uint32_t> inst_light_base;
    // Textures (Image2D) and per-material maps (MaterialResource's *_texture fields); empty when untextured.
    struct Tex {
        uint32_t w, h, srgb;
        std::vector<V4> px;
    };
    std::vector<Tex> textures;
    std::vector<spk_material_maps> maps;
};

namespace {

// Möller–Trumbore in local space + world t via Ray::InverseAt (MeshRenderProxy.cpp:128-194, Ray.h:38-47).
template <bool AnyHit>
inline bool intersect_triangle(const Tri &tri, V3 wo, V3 wd, V3 lo, V3 ld, const Affine &M, Candidate &cand,
                               uint32_t face) {
    const V3 h = cross(ld, tri.e2);
    const float a = dot3(tri.e1, h);
    if (std::abs(a) < kEps) return false;
    const V3 s = lo - tri.p0;
    const float f = 1.f / a;
    const float u = f * dot3(s, h);
    if (u < 0.f || u > 1.f) return false;
    const V3 q = cross(s, tri.e1);
    const float v = f * dot3(ld, q);
    if (v < 0.f || u + v > 1.f) return false;
    const float t = f * dot3(tri.e2, q);
    if (t > kEps) {
        if (AnyHit) return true;
        const V3 local_p = lo + ld * t;
        const V3 world_p = xform_point(M, local_p);
        const float world_t = (world_p.x - wo.x) / wd.x;
        if (world_t > 0 && world_t < cand.t) {
            cand.t = world_t;
            cand.u = u;
            cand.v = v;
            cand.face = face;
            return true;
        }
    }
    return false;
}

// SphereRenderProxy::IntersectInternal (SphereRenderProxy.cpp:5-38).
template <bool AnyHit>
inline bool intersect_sphere(const Inst &in, V3 o, V3 d, Candidate &cand) {
    const V3 center = mk(in.desc.transform[3], in.desc.transform[7], in.desc.transform[11]);
    const V3 co = o - center;
    const float a = 1.f;
    const float half_b = dot3(d, co);
    const float c = sqnorm(co) - in.desc.radius * in.desc.radius;
    const float disc = half_b * half_b - a * c;
    if (disc < 0) return false;
    if (AnyHit) return true;
    const float sq = std::sqrt(disc);
    const float t = (-half_b + (c >= 0 ? -sq : sq)) / a;
    if (t > 0 && t < cand.t) {
        cand.t = t;
        return true;
    }
    return false;
}

// Conservative bound on |world_t - t| from the x-only Ray::InverseAt quirk; used by the pruned walk only.
inline float pruning_limit(const or_scene &sc, V3 o, V3 d, float best) {
    if (!(best < std::numeric_limits<float>::max())) return std::numeric_limits<float>::max();
    const float ax = std::fabs(d.x);
    const float slack = ax > 0.f ? (std::fabs(o.x) + sc.scene_abs_x) * 0x1p-18f / ax : std::numeric_limits<float>::max();
    const float lim = best * (1.f + 0x1p-14f) + slack;
    return std::isfinite(lim) ? lim : std::numeric_limits<float>::max();
}

// MeshRenderProxy BLAS walk (MeshRenderProxy.cpp:94-126).
template <bool AnyHit>
bool intersect_mesh(const or_scene &sc, const Inst &in, V3 o, V3 d, Candidate &cand, bool pruned,
                    uint64_t &overflows) {
    const MeshData &m = sc.meshes[in.desc.mesh_id];
    const V3 lo = xform_point(in.Minv, o), ld = xform_dir(in.Minv, d);
    TravRay r = make_trav_ray(lo, ld);
    if (pruned && !AnyHit) r.tmax = pruning_limit(sc, o, d, cand.t);
    bool found = false;
    auto leaf = [&](uint32_t b, uint32_t e) {
        for (uint32_t i = b; i < e; ++i) {
            const uint32_t face = m.bvh.prim_ids[i];
            if (intersect_triangle<AnyHit>(m.tris[face], o, d, lo, ld, in.M, cand, face)) {
                found = true;
                if (pruned && !AnyHit) r.tmax = pruning_limit(sc, o, d, cand.t);
            }
        }
        return found;
    };
    traverse<AnyHit>(m.bvh, r, leaf, overflows);
    return found;
}

// TLAS::IntersectInternal (SceneRenderProxy.cpp:82-126): returns the winning TLAS slot (or -1).
template <bool AnyHit>
int32_t intersect_scene(const or_scene &sc, V3 o, V3 d, Candidate &cand, bool pruned, uint64_t &overflows) {
    TravRay r = make_trav_ray(o, d);
    int32_t hit_slot = -1;
    auto leaf = [&](uint32_t b, uint32_t e) {
        for (uint32_t i = b; i < e; ++i) {
            const Inst &in = sc.insts[sc.tlas_slot[i]];
            const bool h = in.desc.type == SPK_PRIM_SPHERE ? intersect_sphere<AnyHit>(in, o, d, cand)
                                                           : intersect_mesh<AnyHit>(sc, in, o, d, cand, pruned, overflows);
            if (h) {
                hit_slot = static_cast<int32_t>(i);
                cand.slot = hit_slot;
                if (pruned && !AnyHit) r.tmax = pruning_limit(sc, o, d, cand.t);
            }
        }
        return hit_slot >= 0;
    };
    traverse<AnyHit>(sc.tlas, r, leaf, overflows);
    return hit_slot;
}

// Möller–Trumbore local t of a triangle, or -1 when the test fails (same operations as intersect_triangle).
inline float triangle_t(const Tri &tri, V3 lo, V3 ld) {
    const V3 h = cross(ld, tri.e2);
    const float a = dot3(tri.e1, h);
    if (std::abs(a) < kEps) return -1.f;
    const V3 s = lo - tri.p0;
    const float f = 1.f / a;
    const float u = f * dot3(s, h);
    if (u < 0.f || u > 1.f) return -1.f;
    const V3 q = cross(s, tri.e1);
    const float v = f * dot3(ld, q);
    if (v < 0.f || u + v > 1.f) return -1.f;
    const float t = f * dot3(tri.e2, q);
    return t > kEps ? t : -1.f;
}

// Shadow-ray occlusion for next-event estimation (the GPU shader's IsRayOccluded with TMin/TMax,
// ray_trace.cs.slang:105-116): any triangle with Eps < t < tmax (local t; affine maps keep the ray
// parameter) or sphere root in (Eps, tmax), walking with early exit.
bool occluded(const or_scene &sc, V3 o, V3 d, float tmax, uint64_t &overflows) {
    TravRay r = make_trav_ray(o, d);
    r.tmax = tmax;
    bool hit = false;
    auto leaf = [&](uint32_t b, uint32_t e) {
        for (uint32_t i = b; i < e && !hit; ++i) {
            const Inst &in = sc.insts[sc.tlas_slot[i]];
            if (in.desc.type == SPK_PRIM_SPHERE) {
                const V3 center = mk(in.desc.transform[3], in.desc.transform[7], in.desc.transform[11]);
                const V3 co = o - center;
                const float half_b = dot3(d, co);
                const float c = sqnorm(co) - in.desc.radius * in.desc.radius;
                const float disc = half_b * half_b - 1.f * c;
                if (disc < 0) continue;
                const float sq = std::sqrt(disc);
                const float t = (-half_b + (c >= 0 ? -sq : sq)) / 1.f;
                if (t > kEps && t < tmax) hit = true;
            } else {
                const MeshData &m = sc.meshes[in.desc.mesh_id];
                const V3 lo = xform_point(in.Minv, o), ld = xform_dir(in.Minv, d);
                TravRay lr = make_trav_ray(lo, ld);
                lr.tmax = tmax;
                auto tleaf = [&](uint32_t tb, uint32_t te) {
                    for (uint32_t k = tb; k < te; ++k) {
                        const float t = triangle_t(m.tris[m.bvh.prim_ids[k]], lo, ld);
                        if (t > kEps && t < tmax) {
                            hit = true;
                            break;
                        }
                    }
                    return hit;
                };
                traverse<true>(m.bvh, lr, tleaf, overflows);
            }
        }
        return hit;
    };
    traverse<true>(sc.tlas, r, leaf, overflows);
    return hit;
}

// GetMISWeight (power heuristic, ray_trace.cs.slang:176-186).
inline float mis_weight(float current_pdf, float compensation_pdf) {
    if (current_pdf < kEps || compensation_pdf < kEps) return 1.f;
    const float c2 = current_pdf * current_pdf;
    const float o2 = compensation_pdf * compensation_pdf;
    return c2 / (o2 + c2 + kEps);
}

// Utilities::Lerp(v0, v1, v2, u, v) = v0 + (v1 - v0) * u + (v2 - v0) * v (Utilities.h:114-117).
inline float lerp3(float a, float b, float c, float u, float v) { return a + (b - a) * u + (c - a) * v; }

// GetIntersection for meshes (MeshRenderProxy.cpp:340-361, Mesh.h:86-134) and spheres
// (SphereRenderProxy.h:22-31), then Intersection::Update (Intersection.h:52-71).
// Image2D::Sample (io/Image.h:112-150): bilinear with wrap at uv * size (utilities::Decompose truncates
// toward zero, utilities::WrapMod), u lerp then v lerp, sRGB decoded after the filter (SRGBtoLinear,
// Utilities.h:416-425).
inline unsigned wrap_texel(int a, unsigned b) { return (static_cast<unsigned>(a % static_cast<int>(b)) + b) % b; }

inline float srgb_decode(float c) { return c < 0.04045f ? c / 12.92f : std::pow((c + 0.055f) / 1.055f, 2.4f); }

V3 tex_sample(const or_scene &sc, uint32_t t, const float uv[2]) {
    const or_scene::Tex &T = sc.textures[t];
    const float px = uv[0] * static_cast<float>(T.w), py = uv[1] * static_cast<float>(T.h);
    const int ui = static_cast<int>(px), vi = static_cast<int>(py);
    const float uc = px - static_cast<float>(ui), vc = py - static_cast<float>(vi);
    const unsigned x0 = wrap_texel(ui, T.w), x1 = wrap_texel(ui + 1, T.w);
    const unsigned y0 = wrap_texel(vi, T.h), y1 = wrap_texel(vi + 1, T.h);
    const V4 s00 = T.px[y0 * T.w + x0], s10 = T.px[y0 * T.w + x1], s01 = T.px[y1 * T.w + x0], s11 = T.px[y1 * T.w + x1];
    const V3 l0 = mk(s00.x + (s10.x - s00.x) * uc, s00.y + (s10.y - s00.y) * uc, s00.z + (s10.z - s00.z) * uc);
    const V3 l1 = mk(s01.x + (s11.x - s01.x) * uc, s01.y + (s11.y - s01.y) * uc, s01.z + (s11.z - s01.z) * uc);
    V3 r = mk(l0.x + (l1.x - l0.x) * vc, l0.y + (l1.y - l0.y) * vc, l0.z + (l1.z - l0.z) * vc);
    if (T.srgb) r = mk(srgb_decode(r.x), srgb_decode(r.y), srgb_decode(r.z));
    return r;
}

// which: 0 base colour, 1 metallic-roughness, 2 emissive, 3 normal; -1 when the material has none.
inline int32_t material_map(const or_scene &sc, uint32_t mat, int which) {
    if (sc.maps.empty()) return -1;
    const spk_material_maps &m = sc.maps[mat];
    return which == 0 ? m.base_color : which == 1 ? m.metallic_roughness : which == 2 ? m.emissive : m.normal;
}

// MaterialRenderProxy::GetBaseColor / GetMetallic / GetRoughness / GetEmissive (MaterialRenderProxy.h:117-160):
// texture x factor, metallic = texel.z x factor, roughness = texel.y x factor.
spk_material resolve_material(const or_scene &sc, uint32_t mat_id, const float uv[2]) {
    spk_material m = sc.materials[mat_id];
    int32_t t = material_map(sc, mat_id, 0);
    if (t >= 0) {
        const V3 c = tex_sample(sc, static_cast<uint32_t>(t), uv);
        m.base_color[0] = c.x * m.base_color[0];
        m.base_color[1] = c.y * m.base_color[1];
        m.base_color[2] = c.z * m.base_color[2];
    }
    if ((t = material_map(sc, mat_id, 1)) >= 0) {
        const V3 c = tex_sample(sc, static_cast<uint32_t>(t), uv);
        m.metallic = c.z * m.metallic;
        m.roughness = c.y * m.roughness;
    }
    if ((t = material_map(sc, mat_id, 2)) >= 0) {
        const V3 c = tex_sample(sc, static_cast<uint32_t>(t), uv);
        m.emissive[0] = c.x * m.emissive[0];
        m.emissive[1] = c.y * m.emissive[1];
        m.emissive[2] = c.z * m.emissive[2];
    }
    return m;
}

Hit make_hit(const or_scene &sc, const Candidate &cand, V3 o, V3 d) {
    Hit h;
    if (cand.slot < 0) return h;
    const uint32_t prim = sc.tlas_slot[cand.slot];
    const Inst &in = sc.insts[prim];
    h.hit = true;
    h.prim = prim;
    h.t = cand.t;
    if (in.desc.type == SPK_PRIM_SPHERE) {
        const V3 center = mk(in.desc.transform[3], in.desc.transform[7], in.desc.transform[11]);
        const V3 p = o + d * cand.t;
        h.normal = normalized(p - center);
        // GetPossibleMajorAxis (Utilities.h:222-234)
        if (std::abs(h.normal.x) < kInvSqrt3) {
            h.tangent = mk(1, 0, 0);
        } else if (std::abs(h.normal.y) < kInvSqrt3) {
            h.tangent = mk(0, 1, 0);
        } else {
            h.tangent = mk(0, 0, 1);
        }
    } else {
        const MeshData &m = sc.meshes[in.desc.mesh_id];
        const uint32_t i0 = m.idx[cand.face * 3], i1 = m.idx[cand.face * 3 + 1], i2 = m.idx[cand.face * 3 + 2];
        const float u = cand.u, v = cand.v;
        if (m.has_uv) {
            h.uv[0] = lerp3(m.uv[2 * i0], m.uv[2 * i1], m.uv[2 * i2], u, v);
            h.uv[1] = lerp3(m.uv[2 * i0 + 1], m.uv[2 * i1 + 1], m.uv[2 * i2 + 1], u, v);
        }
        const V3 n0 = m.nrm[i0], n1 = m.nrm[i1], n2 = m.nrm[i2];
        V3 sn = mk(lerp3(n0.x, n1.x, n2.x, u, v), lerp3(n0.y, n1.y, n2.y, u, v), lerp3(n0.z, n1.z, n2.z, u, v));
        V3 tg = mk(1, 0, 0);
        float tw = 1.f;
        if (m.has_tan) {
            const V4 t0 = m.tan[i0], t1 = m.tan[i1], t2 = m.tan[i2];
            tg = mk(lerp3(t0.x, t1.x, t2.x, u, v), lerp3(t0.y, t1.y, t2.y, u, v), lerp3(t0.z, t1.z, t2.z, u, v));
            tw = lerp3(t0.w, t1.w, t2.w, u, v);
        }
        const int32_t nmap = material_map(sc, in.desc.material_id, 3);
        if (nmap >= 0) {
            // MeshRenderProxy::GetIntersection (MeshRenderProxy.cpp:349-355): GetNormal = texel * 2 - 1 in the
            // tangent frame, TangentSpaceToWorldSpace (Utilities.h:403-409).
            const V3 t = tex_sample(sc, static_cast<uint32_t>(nmap), h.uv);
            const V3 tn = mk(t.x * 2.f - 1.f, t.y * 2.f - 1.f, t.z * 2.f - 1.f);
            const V3 bi = cross(sn, tg) * tw;
            sn = normalized(tg * tn.x + bi * tn.y + sn * tn.z);
        }
        // inv_transform.TransformDirectionTangentSpace(n) = M_3x3 * n (Transform.h:105-108)
        h.normal = normalized(xform_dir(in.M, sn));
        h.tangent = xform_dir(in.M, tg);
    }
    h.location = o + d * cand.t;
    return h;
}

// ------------------------------------------------------------------------------------------------
// Materials: PbrMaterialRenderProxy.h:15-51, DialetricMaterialRenderProxy.h:16-37, BxDF.h:32-140,
// Utilities.h:201-330,434-451, Sampler.h:79-165
// ------------------------------------------------------------------------------------------------
inline void local_axes(V3 normal, V3 major, V3 &u, V3 &v, V3 &w) {  // GetLocalAxisFromNormal (Utilities.h:236-244)
    u = normalized(cross(normal, major));
    v = cross(normal, u);
    w = normal;
}
inline V3 to_world(V3 dir, V3 u, V3 v, V3 w) {  // TransformBasisToWorld (Utilities.h:257-260)
    return u * dir.x + v * dir.y + w * dir.z;
}
inline V3 to_local(V3 dir, V3 u, V3 v, V3 w) {  // TransformBasisToLocal (Utilities.h:262-269)
    return mk(dot3(dir, u), dot3(dir, v), dot3(dir, w));
}
inline float schlick(float cos_i, float r0) {  // Utilities.h:291-294
    const float p = std::pow((1.f - cos_i), 5.f);
    return r0 + (1.f - r0) * p;
}
inline V3 schlick3(float cos_i, V3 r0) {  // Utilities.h:296-299
    const float p = std::pow((1.f - cos_i), 5.f);
    return mk(r0.x + (1.f - r0.x) * p, r0.y + (1.f - r0.y) * p, r0.z + (1.f - r0.z) * p);
}
inline float smith_ggx_correlated(float cos_o, float cos_i, float roughness) {  // Utilities.h:434-442
    const float a = roughness * roughness;
    const float a2 = a * a;
    const float ggx_i = cos_o * std::sqrt((-cos_i * a2 + cos_i) * cos_i + a2);
    const float ggx_o = cos_i * std::sqrt((-cos_o * a2 + cos_o) * cos_o + a2);
    return 2.f * cos_o * cos_i / (ggx_o + ggx_i);
}
inline float geometry_schlick_ggx(float cos_theta, float roughness) {  // Utilities.h:444-451
    const float a = roughness * roughness;
    const float a2 = a * a;
    const float tan2_v = (1.f - cos_theta * cos_theta) / (cos_theta * cos_theta);
    return 2.f / (1.f + std::sqrt(1.f + a2 * tan2_v));
}
inline float fr_dielectric(float cos_i, float eta_i, float eta_t) {  // Utilities.h:301-324
    const bool entering = cos_i > 0.f;
    if (!entering) {
        std::swap(eta_i, eta_t);
        cos_i = -cos_i;
    }
    const float sin_i = std::sqrt(1 - cos_i * cos_i);
    const float ref_idx = eta_i / eta_t;
    const float sin_t = ref_idx * sin_i;
    if (sin_t >= 1.f) return 1.f;
    float r0 = (1.f - ref_idx) / (1.f + ref_idx);
    r0 = r0 * r0;
    return schlick(cos_i, r0);
}
inline V3 refract(V3 w, float eta) {  // Utilities.h:211-220
    const float cos_i = w.z;
    const float sin_i2 = 1.f - cos_i * cos_i;
    const float sin_t2 = eta * eta * sin_i2;
    const float cos_t = std::sqrt(1 - sin_t2) * (cos_i > 0 ? -1.f : 1.f);
    return normalized(mk(-eta * w.x, -eta * w.y, cos_t));
}
// DistributionVn::Sample (Sampler.h:133-164).
inline V3 sample_vndf(Rng &rng, V3 w_o, float roughness) {
    const float a = roughness * roughness;
    const float u1 = rng.unit();
    const float u2 = rng.unit();
    const V3 v = normalized(mk(w_o.x * a, w_o.y * a, w_o.z));
    const V3 t1 = (v.z < 0.999f) ? normalized(cross(v, mk(0, 0, 1))) : mk(1, 0, 0);
    const V3 t2 = cross(v, t1);
    const float r = std::sqrt(u1);
    const float phi = 2.f * kPi * u2;
    const float p1 = r * std::cos(phi);
    float p2 = r * std::sin(phi);
    const float s = 0.5f * (1.f + v.z);
    p2 = (1.f - s) * std::sqrt(1.f - p1 * p1) + s * p2;
    const float sq = std::sqrt(max_std(0.f, 1.f - p1 * p1 - p2 * p2));
    const V3 n = p1 * t1 + p2 * t2 + sq * v;
    return normalized(mk(a * n.x, a * n.y, max_std(0.f, n.z)));
}

// MaterialRenderProxy::SampleSurface; returns the throughput, writes the world w_i.
V3 sample_surface(Rng &rng, const spk_material &mat, V3 ray_dir, V3 normal, V3 tangent, V3 &w_i_world,
                  bool *diffuse = nullptr, float *diffuse_z = nullptr) {
    const V3 base = load3(mat.base_color);
    const V3 w_o = -ray_dir;
    V3 fu, fv, fw;
    local_axes(normal, tangent, fu, fv, fw);
    const V3 lw_o = to_local(w_o, fu, fv, fw);
    V3 lw_i, thr;
    if (mat.type == SPK_MAT_DIELECTRIC) {
        // DieletricBxDF::Sample (BxDF.h:90-118)
        const float fresnel = fr_dielectric(lw_o.z, 1.0f, mat.eta);
        if (rng.unit() < fresnel) {
            lw_i = mk(-lw_o.x, -lw_o.y, lw_o.z);
        } else {
            const bool entering = lw_o.z > 0;
            const float ratio = entering ? 1.0f / mat.eta : mat.eta / 1.0f;
            lw_i = refract(lw_o, ratio);
        }
        thr = base;
    } else {
        // SpecularBxDF::Sample (BxDF.h:48-110), then LambertianBxDF::Sample (BxDF.h:32-45)
        const V3 w_m = sample_vndf(rng, lw_o, mat.roughness);
        const V3 cand_i = w_m * (dot3(lw_o, w_m) * 2.f) - lw_o;  // Reflect (Utilities.h:206-209)
        const float cos_o = std::abs(lw_o.z), cos_i = std::abs(cand_i.z), cos_m = std::abs(w_m.z);
        const float local_cos_i = dot3(cand_i, w_m);
        bool valid = false;
        V3 fresnel_color{};
        if (cos_o > kEps && cos_i > kEps && cos_m > kEps) {
            if (rng.unit() < mat.metallic) {
                fresnel_color = schlick3(local_cos_i, base);
                valid = true;
            } else {
                const float fresnel = schlick(local_cos_i, 0.04f);
                if (rng.unit() < fresnel) {
                    fresnel_color = mk(1, 1, 1);
                    valid = true;
                }
            }
        }
        if (valid) {
            const float occlusion = smith_ggx_correlated(cos_o, cos_i, mat.roughness);
            const float normalizer = geometry_schlick_ggx(cos_o, mat.roughness) + kEps;
            thr = mk(fresnel_color.x * occlusion / normalizer, fresnel_color.y * occlusion / normalizer,
                     fresnel_color.z * occlusion / normalizer);
            lw_i = cand_i;
        } else {
            float dx, dy;
            unit_disk(rng, dx, dy);  // CosineWeightedHemiSphere::Sample (Sampler.h:79-89)
            const float sq = dx * dx + dy * dy;
            const float z = std::sqrt(max_std(0.f, 1.0f - sq));
            lw_i = mk(dx, dy, z);
            thr = base;
            if (diffuse) *diffuse = true;
            if (diffuse_z) *diffuse_z = z;
        }
    }
    V3 gu, gv, gw;
    local_axes(normal, tangent, gu, gv, gw);
    w_i_world = normalized(to_world(lw_i, gu, gv, gw));
    return thr;
}

// ------------------------------------------------------------------------------------------------
// Sky: SkyRenderProxy::Evaluate (SkyRenderProxy.cpp:50-64), Image2DCube::Sample (Image.cpp:298-357),
// Image2D::Sample (libraries/include/io/Image.h:112-150)
// ------------------------------------------------------------------------------------------------
inline unsigned wrap_mod(int a, unsigned b) {
    return (static_cast<unsigned>(a % static_cast<int>(b)) + b) % b;
}
V3 sky_eval(const or_scene &sc, V3 d) {
    if (sc.sky.mode == SPK_SKY_CUBE) {
        const float x = d.x, y = d.y, z = d.z;
        const float ax = std::abs(x), ay = std::abs(y), az = std::abs(z);
        int face;
        float u, v;
        if (ax >= ay && ax >= az) {
            if (x > 0) {
                face = 0;
                u = -z / x;
                v = -y / x;
            } else {
                face = 1;
                u = z / -x;
                v = -y / -x;
            }
        } else if (ay >= ax && ay >= az) {
            if (y > 0) {
                face = 2;
                u = x / y;
                v = z / y;
            } else {
                face = 3;
                u = x / -y;
                v = -z / -y;
            }
        } else {
            if (z > 0) {
                face = 4;
                u = x / z;
                v = -y / z;
            } else {
                face = 5;
                u = -x / -z;
                v = -y / -z;
            }
        }
        u = (u + 1.f) * 0.5f;
        v = (v + 1.f) * 0.5f;
        const unsigned n = sc.sky.cube_size;
        const float px = u * static_cast<float>(n - 1), py = v * static_cast<float>(n - 1);
        const int ui = static_cast<int>(px), vi = static_cast<int>(py);
        const float uc = px - static_cast<float>(ui), vc = py - static_cast<float>(vi);
        const float *f = sc.cube.data() + static_cast<size_t>(face) * n * n * 4;
        auto px4 = [&](unsigned xi, unsigned yi, int c) { return f[(static_cast<size_t>(yi) * n + xi) * 4 + c]; };
        const unsigned x0 = wrap_mod(ui, n), x1 = wrap_mod(ui + 1, n), y0 = wrap_mod(vi, n), y1 = wrap_mod(vi + 1, n);
        float out[3];
        for (int c = 0; c < 3; ++c) {
            const float s00 = px4(x0, y0, c), s10 = px4(x1, y0, c), s01 = px4(x0, y1, c), s11 = px4(x1, y1, c);
            const float l0 = s00 + (s10 - s00) * uc;
            const float l1 = s01 + (s11 - s01) * uc;
            out[c] = l0 + (l1 - l0) * vc;
        }
        return mk(out[0], out[1], out[2]);
    }
    if (sc.sky.mode == SPK_SKY_GRADIENT) {
        const float t = 0.5f * d.z + 0.5f;
        return mk(1.f + (sc.sky.color[0] - 1.f) * t, 1.f + (sc.sky.color[1] - 1.f) * t,
                  1.f + (sc.sky.color[2] - 1.f) * t);
    }
    return mk(0, 0, 0);
}

// ------------------------------------------------------------------------------------------------
// IEEE binary16 conversion, round to nearest even (Eigen::half cast in Image2D::SetPixel, Image.h:174-178)
// ------------------------------------------------------------------------------------------------
uint16_t f32_to_f16(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t ax = x & 0x7FFFFFFFu;
    if (ax >= 0x7F800000u) return static_cast<uint16_t>(sign | 0x7C00u | (ax > 0x7F800000u ? 0x200u : 0u));
    if (ax >= 0x477FF000u) return static_cast<uint16_t>(sign | 0x7C00u);  // >= 65520 rounds to inf
    if (ax >= 0x38800000u) {                                                 // normal half
        const uint32_t m = ax & 0x7FFFFFu;
        uint32_t h = (((ax >> 23) - 112u) << 10) | (m >> 13);
        const uint32_t rem = m & 0x1FFFu;
        if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
        return static_cast<uint16_t>(sign | h);
    }
    const uint32_t e = ax >> 23;
    if (e == 0) return static_cast<uint16_t>(sign);
    const uint32_t m = (ax & 0x7FFFFFu) | 0x800000u;
    const uint32_t shift = 126u - e;  // >= 14
    if (shift > 24u) return static_cast<uint16_t>(sign);
    uint32_t h = m >> shift;
    const uint32_t rem = m & ((1u << shift) - 1u), halfway = 1u << (shift - 1u);
    if (rem > halfway || (rem == halfway && (h & 1u))) ++h;
    return static_cast<uint16_t>(sign | h);
}

template <class F>
void parallel_rows(uint32_t begin, uint32_t end, int num_threads, F &&fn) {
    if (end <= begin) return;
    const uint32_t n = end - begin;
    int nt = num_threads > 0 ? num_threads : static_cast<int>(std::thread::hardware_concurrency());
    nt = std::max(1, std::min<int>(nt, static_cast<int>(n)));
    if (nt == 1) {
        for (uint32_t j = begin; j < end; ++j) fn(j, 0);
        return;
    }
    std::atomic<uint32_t> next{begin};
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t) {
        pool.emplace_back([&, t]() {
            for (;;) {
                const uint32_t j = next.fetch_add(1);
                if (j >= end) break;
                fn(j, t);
            }
        });
    }
    for (auto &th : pool) th.join();
}

}  // namespace

// ------------------------------------------------------------------------------------------------
// Renderer state (CPURenderer.h:18-72 members; CameraRenderProxy sample counters)
// ------------------------------------------------------------------------------------------------
struct or_renderer {
    const or_scene *scene;
    spk_config cfg;
    spk_camera cam;
    uint32_t w, h, spp_eff;
    std::vector<V4> gcolor, ping, fb;
    std::vector<V3> gnormal;
    std::vector<uint16_t> out;
    uint32_t cumulated = 0, pending = 0, dispatched = 0;
    bool dirty = true;
    std::atomic<uint64_t> ext_rays{0}, shadow_rays{0}, paths{0};
};

namespace {

struct PixelResult {  // CPURenderer.cpp:212-217
    V3 color{0, 0, 0};
    V3 world_normal{0, 0, 0};
    float valid = 1.f;
};

// Next-event estimation at a vertex where the path took the diffuse fall-through branch of the PBR
// sampler (no counterpart in the reference cpu pipeline; the GPU shader samples only the sky,
// ray_trace.cs.slang:118-174). One point on the emissive triangles (area CDF, uniform on the triangle) and
// one cosine-weighted sky direction, each with an occlusion ray and the shader's power-heuristic weight
// against the cosine pdf of the diffuse branch. The estimator is the cpu BSDF's (base/pi * L * cos / pdf),
// so NEE converges to the plain path tracer's image.
void nee_direct(const or_scene &sc, Rng &rng, const Hit &hit, V3 base, V3 thr, V3 &color, uint64_t &shadow_rays,
                uint64_t &overflows) {
    if (!sc.lights.empty()) {
        const float u0 = rng.unit(), u1 = rng.unit(), u2 = rng.unit();
        const float target = u0 * sc.light_total;
        size_t k = static_cast<size_t>(std::upper_bound(sc.light_cdf.begin(), sc.light_cdf.end(), target) -
                                       sc.light_cdf.begin());
        if (k >= sc.lights.size()) k = sc.lights.size() - 1;
        const or_scene::Light &L = sc.lights[k];
        const float r1 = std::sqrt(u1);
        const float a = r1 * (1.f - u2), b = r1 * u2;
        const V3 x = L.p0 + L.e1 * a + L.e2 * b;
        const V3 to = x - hit.location;
        const float dist2 = sqnorm(to);
        if (dist2 > 0.f) {
            const float dist = std::sqrt(dist2);
            const V3 w = mk(to.x / dist, to.y / dist, to.z / dist);
            const float cos_s = dot3(hit.normal, w);
            const float cos_l = std::abs(dot3(L.ng, w));
            if (cos_s > 0.f && cos_l > kEps) {
                const float pdf_l = dist2 / (sc.light_total * cos_l);
                const float pdf_b = cos_s * kInvPi;
                const float wl = mis_weight(pdf_l, pdf_b);
                ++shadow_rays;
                const V3 so = hit.location + w * kTolerance;
                const float tmax = (dist - kTolerance) * (1.f - 1e-4f);
                if (!occluded(sc, so, w, tmax, overflows)) {
                    const float f = cos_s / pdf_l * wl * kInvPi;
                    color = color + mk(thr.x * base.x * L.emission.x * f, thr.y * base.y * L.emission.y * f,
                                       thr.z * base.z * L.emission.z * f);
                }
            }
        }
    }
    if (sc.sky.mode != SPK_SKY_NONE) {
        V3 fu, fv, fw;
        local_axes(hit.normal, hit.tangent, fu, fv, fw);
        float dx, dy;
        unit_disk(rng, dx, dy);
        const float z = std::sqrt(max_std(0.f, 1.0f - (dx * dx + dy * dy)));
        const V3 w = normalized(to_world(mk(dx, dy, z), fu, fv, fw));
        const float pdf = z * kInvPi;
        if (pdf > 0.f) {
            const float wl = mis_weight(pdf, pdf);
            ++shadow_rays;
            const V3 so = hit.location + w * kTolerance;
            if (!occluded(sc, so, w, 1000.f, overflows)) {
                const V3 L = sky_eval(sc, w);
                const float f = z / pdf * wl * kInvPi;
                color = color + mk(thr.x * base.x * L.x * f, thr.y * base.y * L.y * f, thr.z * base.z * L.z * f);
            }
        }
    }
}

// SamplePixel (CPURenderer.cpp:240-396) for debug_mode == Color, with SetupViewRay (:220-238).
PixelResult sample_pixel(const or_renderer &r, Rng &rng, float u, float v, bool pruned, uint64_t &rays,
                         uint64_t &shadow_rays, uint64_t &overflows) {
    const or_scene &sc = *r.scene;
    const spk_camera &cam = r.cam;
    PixelResult res;
    float ax, ay;
    unit_disk(rng, ax, ay);
    ax = ax * cam.aperture_radius;
    ay = ay * cam.aperture_radius;
    const V3 lens = ax * load3(cam.right) + ay * load3(cam.up);
    V3 o = load3(cam.position) + lens;
    const V3 focus = load3(cam.lower_left) + u * load3(cam.max_u) + v * load3(cam.max_v);
    V3 d = normalized(focus - o);
    V3 thr = mk(1, 1, 1);
    const bool nee = r.cfg.enable_nee != 0;
    bool prev_nee = false;  // the previous vertex sampled the lights (diffuse branch)
    float prev_pdf = 0.f;   // cosine pdf of the direction the previous vertex continued in
    for (uint32_t bounce = 0; bounce < r.cfg.bounce; ++bounce) {
        Candidate cand;
        ++rays;
        intersect_scene<false>(sc, o, d, cand, pruned, overflows);
        const Hit hit = make_hit(sc, cand, o, d);
        if (!hit.hit) {
            if (sc.sky.mode != SPK_SKY_NONE) {
                V3 c = cmul(sky_eval(sc, d), thr);
                if (prev_nee) c = c * mis_weight(prev_pdf, prev_pdf);
                res.color = res.color + c;
            }
            break;
        }
        const spk_material mat = resolve_material(sc, sc.insts[hit.prim].desc.material_id, hit.uv);
        if (bounce == 0) res.world_normal = hit.normal;
        const V3 emissive = load3(mat.emissive);
        if (std::sqrt(sqnorm(emissive)) > kEps) {
            V3 c = cmul(emissive, thr);
            if (prev_nee && cand.face != SPK_INVALID_ID && sc.inst_light_base[hit.prim] != SPK_INVALID_ID) {
                const or_scene::Light &L = sc.lights[sc.inst_light_base[hit.prim] + cand.face];
                const float cos_l = std::abs(dot3(L.ng, d));
                if (cos_l > kEps) c = c * mis_weight(prev_pdf, (hit.t * hit.t) / (sc.light_total * cos_l));
            }
            res.color = res.color + c;
            break;
        }
        V3 next_dir;
        bool diffuse = false;
        float dz = 0.f;
        const V3 this_thr = sample_surface(rng, mat, d, hit.normal, hit.tangent, next_dir, &diffuse, &dz);
        prev_nee = false;
        if (nee && diffuse) {
            nee_direct(sc, rng, hit, load3(mat.base_color), thr, res.color, shadow_rays, overflows);
            prev_nee = true;
            prev_pdf = dz * kInvPi;
        }
        thr = cmul(thr, this_thr);
        if (sqnorm(thr) < kEps) {
            res.valid = -1.f;
            break;
        }
        if (bounce >= 3) {
            float p = max_std(thr.x, max_std(thr.y, thr.z));  // maxCoeff
            p = (p < 0.05f) ? 0.05f : (1.0f < p) ? 1.0f : p;  // std::clamp
            if (rng.unit() > p) break;
            thr = mk(thr.x / p, thr.y / p, thr.z / p);
        }
        o = hit.location + next_dir * kTolerance;
        d = next_dir;
    }
    return res;
}

// BasePass + RenderPixel (CPURenderer.cpp:398-450).
// Rows row_begin, row_begin + row_step, ... below row_end (all rows: 0, h, 1).
void base_pass(or_renderer &r, bool pruned, int num_threads, uint32_t row_begin, uint32_t row_end, uint32_t row_step) {
    const float pw = 1.f / static_cast<float>(r.w - 1);
    const float ph = 1.f / static_cast<float>(r.h - 1);
    const uint32_t frame_seed = r.dispatched;
    const uint32_t num_rows = (row_end - row_begin + row_step - 1) / row_step;
    std::atomic<uint64_t> rays{0}, shadow{0}, ovf{0};
    parallel_rows(0, num_rows, num_threads, [&](uint32_t row, int) {
        const uint32_t j = row_begin + row * row_step;
        uint64_t my_rays = 0, my_shadow = 0, my_ovf = 0;
        Rng rng;
        for (uint32_t i = 0; i < r.w; ++i) {
            seed_pixel(rng, static_cast<int>(r.cfg.rng), r.cfg.seed, i, j, r.w, r.h, frame_seed);
            const float u = (static_cast<float>(i) + rng.unit()) * pw;
            const float v = (static_cast<float>(j) + rng.unit()) * ph;
            PixelResult res = sample_pixel(r, rng, u, v, pruned, my_rays, my_shadow, my_ovf);
            res.color = mk(clamp_sample(res.color.x), clamp_sample(res.color.y), clamp_sample(res.color.z));
            const size_t k = static_cast<size_t>(j) * r.w + i;
            r.gcolor[k] = {res.color.x, res.color.y, res.color.z, res.valid};
            r.gnormal[k] = res.world_normal;
        }
        rays += my_rays;
        shadow += my_shadow;
        ovf += my_ovf;
    });
    r.ext_rays += rays.load();
    r.shadow_rays += shadow.load();
    r.paths += static_cast<uint64_t>(num_rows) * r.w;
}

inline bool is_valid_px(const or_renderer &r, size_t k) { return r.gcolor[k].w > 0; }
inline bool is_sky_px(const or_renderer &r, size_t k) {  // CPUGBuffer::IsSky: isZero() with prec 1e-5
    const V3 n = r.gnormal[k];
    return is_valid_px(r, k) && std::abs(n.x) <= 1e-5f && std::abs(n.y) <= 1e-5f && std::abs(n.z) <= 1e-5f;
}

// SpatialDenoisePixel (CPURenderer.cpp:452-504) in its single-threaded order: rows bottom-up, pixels
// left to right, later writers overwrite earlier ones (the reference's row tasks race on shared
// neighbours; this is the result of running them one after another).
void spatial_pass(or_renderer &r) {
    static const int kDirs[8][2] = {{1, 0}, {0, 1}, {-1, 0}, {0, -1}, {-1, -1}, {1, -1}, {-1, 1}, {1, 1}};
    for (size_t k = 0; k < r.gcolor.size(); ++k) r.ping[k] = r.gcolor[k];
    for (uint32_t j = 0; j < r.h; ++j) {
        for (uint32_t i = 0; i < r.w; ++i) {
            const size_t k = static_cast<size_t>(j) * r.w + i;
            if (!is_valid_px(r, k) || is_sky_px(r, k)) continue;
            const V3 wn = r.gnormal[k];
            const V4 c = r.gcolor[k];
            for (int dk = 0; dk < 8; ++dk) {
                const int si = static_cast<int>(i) + kDirs[dk][0], sj = static_cast<int>(j) + kDirs[dk][1];
                if (si < 0 || si >= static_cast<int>(r.w) || sj < 0 || sj >= static_cast<int>(r.h)) continue;
                const size_t nk = static_cast<size_t>(sj) * r.w + static_cast<size_t>(si);
                if (r.gcolor[nk].w > 0) continue;
                const float sim = dot3(r.gnormal[nk], wn);
                if (sim < 0.99f) continue;
                r.ping[nk] = {c.x, c.y, c.z, 1.f};
                break;
            }
        }
    }
}

// DenoisePass temporal lerp (CPURenderer.cpp:528-544) and ToneMappingPass with ACESFilm (:554-576).
void denoise_and_tonemap(or_renderer &r) {
    if (r.cfg.spatial_denoise) spatial_pass(r);
    const std::vector<V4> &in = r.cfg.spatial_denoise ? r.ping : r.gcolor;
    const float f = static_cast<float>(r.cumulated) / static_cast<float>(r.cumulated + r.spp_eff);
    for (size_t k = 0; k < r.fb.size(); ++k) {
        const V4 n = in[k];
        V4 &a = r.fb[k];
        a = {n.x + (a.x - n.x) * f, n.y + (a.y - n.y) * f, n.z + (a.z - n.z) * f, n.w + (a.w - n.w) * f};
    }
    const float ea = 2.51f, eb = 0.03f, ec = 2.43f, ed = 0.59f, ee = 0.14f;
    const float exposure = r.cam.exposure;
    for (uint32_t j = 0; j < r.h; ++j) {
        for (uint32_t i = 0; i < r.w; ++i) {
            const V4 a = r.fb[static_cast<size_t>(j) * r.w + i];
            const float c3[3] = {a.x, a.y, a.z};
            uint16_t *o = &r.out[(static_cast<size_t>(r.h - 1 - j) * r.w + i) * 4];
            for (int c = 0; c < 3; ++c) {
                const float x = c3[c] * exposure;
                float y = (x * (x * ea + eb)) / (x * (x * ec + ed) + ee);
                y = (1.f < y) ? 1.f : y;  // cwiseMin(1)
                y = (y < 0.f) ? 0.f : y;  // cwiseMax(0)
                o[c] = f32_to_f16(y);
            }
            o[3] = f32_to_f16(1.f);
        }
    }
}

}  // namespace

// ------------------------------------------------------------------------------------------------
// C API
// ------------------------------------------------------------------------------------------------
// Emissive triangles for next-event estimation, in instance then face order, world space. A material
// with an emissive texture varies over the triangle and is reached by BSDF sampling only.
void build_lights(or_scene *sc) {
    const uint32_t num_instances = static_cast<uint32_t>(sc->insts.size());
    sc->lights.clear();
    sc->light_cdf.clear();
    sc->light_total = 0.f;
    sc->inst_light_base.assign(num_instances, SPK_INVALID_ID);
    for (uint32_t k = 0; k < num_instances; ++k) {
        const Inst &in = sc->insts[k];
        if (in.desc.type != SPK_PRIM_MESH) continue;
        if (material_map(*sc, in.desc.material_id, 2) >= 0) continue;
        const V3 em = load3(sc->materials[in.desc.material_id].emissive);
        if (!(std::sqrt(sqnorm(em)) > kEps)) continue;
        const MeshData &m = sc->meshes[in.desc.mesh_id];
        sc->inst_light_base[k] = static_cast<uint32_t>(sc->lights.size());
        for (uint32_t f = 0; f < m.tris.size(); ++f) {
            const V3 w0 = xform_point(in.M, m.pos[m.idx[3 * f]]);
            const V3 w1 = xform_point(in.M, m.pos[m.idx[3 * f + 1]]);
            const V3 w2 = xform_point(in.M, m.pos[m.idx[3 * f + 2]]);
            or_scene::Light L;
            L.p0 = w0;
            L.e1 = w1 - w0;
            L.e2 = w2 - w0;
            const V3 c = cross(L.e1, L.e2);
            const float len = std::sqrt(sqnorm(c));
            L.area = 0.5f * len;
            L.ng = len > 0.f ? mk(c.x / len, c.y / len, c.z / len) : mk(0, 0, 0);
            L.emission = em;
            sc->lights.push_back(L);
        }
    }
    float acc = 0.f;
    for (const auto &L : sc->lights) {
        acc = acc + L.area;
        sc->light_cdf.push_back(acc);
    }
    sc->light_total = acc;
    if (!(acc > 0.f)) {
        sc->lights.clear();
        sc->light_cdf.clear();
        sc->inst_light_base.assign(num_instances, SPK_INVALID_ID);
    }
}

extern "C" {

or_scene *or_scene_create(const spk_mesh *meshes, uint32_t num_meshes, const spk_instance *instances,
                          uint32_t num_instances, const spk_material *materials, uint32_t num_materials,
                          const spk_sky *sky) {
    auto *sc = new or_scene();
    sc->meshes.resize(num_meshes);
    for (uint32_t mi = 0; mi < num_meshes; ++mi) {
        const spk_mesh &src = meshes[mi];
        MeshData &m = sc->meshes[mi];
        m.pos.resize(src.num_vertices);
        m.nrm.resize(src.num_vertices);
        for (uint32_t k = 0; k < src.num_vertices; ++k) {
            m.pos[k] = load3(src.positions + 3 * k);
            m.nrm[k] = load3(src.normals + 3 * k);
        }
        m.has_tan = src.tangents != nullptr;
        if (m.has_tan) {
            m.tan.resize(src.num_vertices);
            for (uint32_t k = 0; k < src.num_vertices; ++k) {
                const float *t = src.tangents + 4 * k;
                m.tan[k] = {t[0], t[1], t[2], t[3]};
            }
        }
        m.has_uv = src.uvs != nullptr;
        if (m.has_uv) m.uv.assign(src.uvs, src.uvs + 2 * static_cast<size_t>(src.num_vertices));
        m.idx.assign(src.indices, src.indices + 3 * static_cast<size_t>(src.num_faces));
        // BLAS::Build (MeshRenderProxy.cpp:31-65): per-triangle box, centre and {p0, e1, e2}.
        std::vector<Box> boxes(src.num_faces);
        std::vector<V3> centers(src.num_faces);
        m.tris.resize(src.num_faces);
        Box mb = empty_box();
        for (uint32_t f = 0; f < src.num_faces; ++f) {
            const V3 v0 = m.pos[m.idx[3 * f]], v1 = m.pos[m.idx[3 * f + 1]], v2 = m.pos[m.idx[3 * f + 2]];
            Box b = empty_box();
            for (const V3 &p : {v0, v1, v2}) {
                const Box pb{{p.x, p.y, p.z}, {p.x, p.y, p.z}};
                grow(b, pb);
            }
            boxes[f] = b;
            centers[f] = mk((b.lo[0] + b.hi[0]) / 2, (b.lo[1] + b.hi[1]) / 2, (b.lo[2] + b.hi[2]) / 2);
            m.tris[f] = {v0, v1 - v0, v2 - v0};
            grow(mb, b);
        }
        m.bvh = build_bvh2(boxes, centers);
        m.bound_center = mk((mb.lo[0] + mb.hi[0]) / 2.f, (mb.lo[1] + mb.hi[1]) / 2.f, (mb.lo[2] + mb.hi[2]) / 2.f);
        m.bound_half = mk((mb.hi[0] - mb.lo[0]) / 2.f, (mb.hi[1] - mb.lo[1]) / 2.f, (mb.hi[2] - mb.lo[2]) / 2.f);
    }
    sc->insts.resize(num_instances);
    std::vector<Box> boxes(num_instances);
    std::vector<V3> centers(num_instances);
    float abs_x = 0.f;
    for (uint32_t k = 0; k < num_instances; ++k) {
        Inst &in = sc->insts[k];
        in.desc = instances[k];
        std::memcpy(in.M.m, in.desc.transform, sizeof(in.M.m));
        std::memcpy(in.Minv.m, in.desc.inv_transform, sizeof(in.Minv.m));
        Box wb = empty_box();
        if (in.desc.type == SPK_PRIM_SPHERE) {
            const float r = in.desc.radius;
            const V3 c = mk(in.desc.transform[3], in.desc.transform[7], in.desc.transform[11]);
            wb = Box{{c.x - r, c.y - r, c.z - r}, {c.x + r, c.y + r, c.z + r}};
        } else {
            // AABB::TransformTo (AABB.h:56-77) of the mesh local bound.
            const MeshData &m = sc->meshes[in.desc.mesh_id];
            static const float dirs[8][3] = {{1, 1, 1},  {-1, 1, 1},  {1, -1, 1},  {1, 1, -1},
                                             {-1, -1, 1}, {1, -1, -1}, {-1, 1, -1}, {-1, -1, -1}};
            V3 mn = mk(std::numeric_limits<float>::max(), std::numeric_limits<float>::max(),
                       std::numeric_limits<float>::max());
            V3 mx = -mn;
            for (const auto &dd : dirs) {
                const V3 lc = m.bound_center + mk(m.bound_half.x * dd[0], m.bound_half.y * dd[1], m.bound_half.z * dd[2]);
                const V3 wc = xform_point(in.M, lc);
                mn = mk(min_std(mn.x, wc.x), min_std(mn.y, wc.y), min_std(mn.z, wc.z));
                mx = mk(max_std(mx.x, wc.x), max_std(mx.y, wc.y), max_std(mx.z, wc.z));
            }
            const V3 c = mk((mn.x + mx.x) / 2.f, (mn.y + mx.y) / 2.f, (mn.z + mx.z) / 2.f);
            const V3 hs = mk(std::abs(mx.x - c.x), std::abs(mx.y - c.y), std::abs(mx.z - c.z));
            wb = Box{{c.x - hs.x, c.y - hs.y, c.z - hs.z}, {c.x + hs.x, c.y + hs.y, c.z + hs.z}};
        }
        in.world_box = wb;
        boxes[k] = wb;
        // AABB::Center
        centers[k] = mk((wb.lo[0] + wb.hi[0]) / 2.f, (wb.lo[1] + wb.hi[1]) / 2.f, (wb.lo[2] + wb.hi[2]) / 2.f);
        abs_x = std::max(abs_x, std::max(std::abs(wb.lo[0]), std::abs(wb.hi[0])));
    }
    sc->scene_abs_x = abs_x;
    // TLAS::Build (SceneRenderProxy.cpp:31-69): leaf slot i refers to primitive prim_ids[i].
    sc->tlas = build_bvh2(boxes, centers);
    sc->tlas_slot = sc->tlas.prim_ids;
    for (uint32_t i = 0; i < sc->tlas.prim_ids.size(); ++i) sc->tlas.prim_ids[i] = i;
    sc->materials.assign(materials, materials + num_materials);
    build_lights(sc);
    if (sky) {
        sc->sky = *sky;
        if (sky->mode == SPK_SKY_CUBE && sky->cube_rgba) {
            sc->cube.assign(sky->cube_rgba, sky->cube_rgba + static_cast<size_t>(6) * sky->cube_size * sky->cube_size * 4);
        }
        sc->sky.cube_rgba = nullptr;
    }
    return sc;
}

void or_scene_destroy(or_scene *scene) { delete scene; }

uint64_t or_trace(const or_scene *scene, const spk_ray *rays, uint64_t num_rays, spk_hit *hits, int32_t any_hit,
                  int32_t traversal, int32_t num_threads) {
    const bool pruned = traversal == OR_TRAVERSAL_PRUNED;
    const uint64_t chunk = 4096;
    const uint32_t nchunks = static_cast<uint32_t>((num_rays + chunk - 1) / chunk);
    std::atomic<uint64_t> ovf{0};
    parallel_rows(0, nchunks, num_threads, [&](uint32_t c, int) {
        uint64_t my_ovf = 0;
        const uint64_t b = c * chunk, e = std::min<uint64_t>(num_rays, b + chunk);
        for (uint64_t k = b; k < e; ++k) {
            const V3 o = load3(rays[k].origin), d = load3(rays[k].direction);
            Candidate cand;
            spk_hit out{0.f, 0.f, 0.f, SPK_INVALID_ID, SPK_INVALID_ID};
            if (any_hit) {
                const int32_t slot = intersect_scene<true>(*scene, o, d, cand, false, my_ovf);
                if (slot >= 0) out.prim = scene->tlas_slot[slot];
            } else {
                const int32_t slot = intersect_scene<false>(*scene, o, d, cand, pruned, my_ovf);
                if (slot >= 0) {
                    const uint32_t prim = scene->tlas_slot[slot];
                    const bool sphere = scene->insts[prim].desc.type == SPK_PRIM_SPHERE;
                    out = {cand.t, sphere ? 0.f : cand.u, sphere ? 0.f : cand.v, prim, sphere ? SPK_INVALID_ID : cand.face};
                }
            }
            hits[k] = out;
        }
        ovf += my_ovf;
    });
    return ovf.load();
}

void or_trace_brute(const or_scene *scene, const spk_ray *rays, uint64_t num_rays, spk_hit *hits,
                    int32_t num_threads) {
    const uint64_t chunk = 256;
    const uint32_t nchunks = static_cast<uint32_t>((num_rays + chunk - 1) / chunk);
    parallel_rows(0, nchunks, num_threads, [&](uint32_t c, int) {
        const uint64_t b = c * chunk, e = std::min<uint64_t>(num_rays, b + chunk);
        for (uint64_t k = b; k < e; ++k) {
            const V3 o = load3(rays[k].origin), d = load3(rays[k].direction);
            Candidate cand;
            uint32_t prim = SPK_INVALID_ID;
            for (uint32_t p = 0; p < scene->insts.size(); ++p) {
                const Inst &in = scene->insts[p];
                if (in.desc.type == SPK_PRIM_SPHERE) {
                    if (intersect_sphere<false>(in, o, d, cand)) {
                        prim = p;
                        cand.face = SPK_INVALID_ID;
                        cand.u = cand.v = 0.f;
                    }
                } else {
                    const MeshData &m = scene->meshes[in.desc.mesh_id];
                    const V3 lo = xform_point(in.Minv, o), ld = xform_dir(in.Minv, d);
                    for (uint32_t f = 0; f < m.tris.size(); ++f) {
                        if (intersect_triangle<false>(m.tris[f], o, d, lo, ld, in.M, cand, f)) prim = p;
                    }
                }
            }
            hits[k] = prim == SPK_INVALID_ID ? spk_hit{0.f, 0.f, 0.f, SPK_INVALID_ID, SPK_INVALID_ID}
                                             : spk_hit{cand.t, cand.u, cand.v, prim, cand.face};
        }
    });
}

or_renderer *or_renderer_create(const or_scene *scene, const spk_config *config, const spk_camera *camera) {
    auto *r = new or_renderer();
    r->scene = scene;
    r->cfg = *config;
    r->cam = *camera;
    r->w = config->width;
    r->h = config->height;
    const size_t n = static_cast<size_t>(r->w) * r->h;
    r->gcolor.assign(n, V4{0, 0, 0, 0});
    r->ping.assign(n, V4{0, 0, 0, 0});
    r->fb.assign(n, V4{0, 0, 0, 0});
    r->gnormal.assign(n, V3{0, 0, 0});
    r->out.assign(n * 4, 0);
    // sub_pixel_count_ = lround(sqrt(float(spp))), actual spp = its square (CPURenderer.cpp:102-104)
    const auto sub = static_cast<unsigned>(std::lround(std::sqrt(static_cast<float>(config->spp))));
    r->spp_eff = sub * sub;
    return r;
}

void or_renderer_destroy(or_renderer *r) { delete r; }

void or_render(or_renderer *r, uint32_t num_frames, int32_t traversal, int32_t num_threads, uint32_t row_begin,
               uint32_t row_end) {
    or_render_rows(r, num_frames, traversal, num_threads, row_begin, row_end, 1);
}

void or_render_rows(or_renderer *r, uint32_t num_frames, int32_t traversal, int32_t num_threads, uint32_t row_begin,
                    uint32_t row_end, uint32_t row_step) {
    if (!(row_end > row_begin)) {
        row_begin = 0;
        row_end = r->h;
    }
    row_end = std::min(row_end, r->h);
    row_step = std::max(row_step, 1u);
    for (uint32_t f = 0; f < num_frames; ++f) {
        // CameraRenderProxy::Update sample bookkeeping (CameraRenderProxy.cpp:66-75)
        if (r->dirty) {
            r->cumulated = 0;
            r->pending = 0;
        }
        r->cumulated = std::min(r->cfg.max_spp, r->cumulated + r->pending);
        r->pending = 0;
        // CPURenderer::Render (CPURenderer.cpp:119-208)
        if (r->dirty) {
            for (auto &a : r->fb) a = V4{0, 0, 0, 0};
            r->dirty = false;
            r->dispatched = r->cfg.sample_offset;
        }
        base_pass(*r, traversal == OR_TRAVERSAL_PRUNED, num_threads, row_begin, row_end, row_step);
        denoise_and_tonemap(*r);
        r->dispatched += r->spp_eff;
        r->pending += r->spp_eff;
    }
}

void or_read_framebuffer(const or_renderer *r, float *hdr_rgba, uint16_t *rgba16f) {
    if (hdr_rgba) std::memcpy(hdr_rgba, r->fb.data(), r->fb.size() * sizeof(V4));
    if (rgba16f) std::memcpy(rgba16f, r->out.data(), r->out.size() * sizeof(uint16_t));
}

void or_read_gbuffer(const or_renderer *r, float *color_rgba, float *world_normal) {
    if (color_rgba) std::memcpy(color_rgba, r->gcolor.data(), r->gcolor.size() * sizeof(V4));
    if (world_normal) std::memcpy(world_normal, r->gnormal.data(), r->gnormal.size() * sizeof(V3));
}

// Primary-hit guides (WritePrimaryHitGBuffer, ray_trace.cs.slang:282-351): one pixel-centre ray from the
// camera position (no jitter, no lens), uv = (pixel + 0.5) / (resolution - 1) with v flipped for the
// top-down pixel row; on a hit within TMax = 1000: normalize(normal), linear depth along
// normalize(cross(max_v, max_u)), base colour, and 2 for an emissive surface else 1. Misses are zero.
// Rows are written bottom-up like the frame buffer (row j is top-down pixel row h - 1 - j).
void or_guides(const or_renderer *r, float *normal_depth, float *albedo_hit) {
    const or_scene &sc = *r->scene;
    const spk_camera &cam = r->cam;
    const uint32_t w = r->w, h = r->h;
    const float pw = 1.f / static_cast<float>(w - 1), ph = 1.f / static_cast<float>(h - 1);
    const V3 front = normalized(cross(load3(cam.max_v), load3(cam.max_u)));
    for (uint32_t j = 0; j < h; ++j) {
        for (uint32_t i = 0; i < w; ++i) {
            const uint32_t py = h - 1 - j;
            const float u = (static_cast<float>(i) + 0.5f) * pw;
            const float v = 1.f - (static_cast<float>(py) + 0.5f) * ph;
            const V3 o = load3(cam.position);
            const V3 d = normalized(load3(cam.lower_left) + u * load3(cam.max_u) + v * load3(cam.max_v) - o);
            Candidate cand;
            uint64_t overflows = 0;
            intersect_scene<false>(sc, o, d, cand, true, overflows);
            const Hit hit = make_hit(sc, cand, o, d);
            float *nd = normal_depth + 4 * (static_cast<size_t>(j) * w + i);
            float *al = albedo_hit + 4 * (static_cast<size_t>(j) * w + i);
            if (!hit.hit || !(hit.t <= 1000.f)) {
                for (int c = 0; c < 4; ++c) nd[c] = al[c] = 0.f;
                continue;
            }
            const spk_material mat = resolve_material(sc, sc.insts[hit.prim].desc.material_id, hit.uv);
            const V3 n = normalized(hit.normal);
            nd[0] = n.x;
            nd[1] = n.y;
            nd[2] = n.z;
            nd[3] = dot3(hit.location - o, front);
            al[0] = mat.base_color[0];
            al[1] = mat.base_color[1];
            al[2] = mat.base_color[2];
            al[3] = std::sqrt(sqnorm(load3(mat.emissive))) > kEps ? 2.f : 1.f;
        }
    }
}

void or_scene_set_textures(or_scene *sc, const spk_texture *textures, uint32_t num_textures,
                           const spk_material_maps *maps) {
    sc->textures.clear();
    for (uint32_t k = 0; k < num_textures; ++k) {
        or_scene::Tex T{textures[k].width, textures[k].height, textures[k].srgb ? 1u : 0u, {}};
        const size_t n = static_cast<size_t>(T.w) * T.h;
        T.px.resize(n);
        for (size_t i = 0; i < n; ++i)
            T.px[i] = V4{textures[k].rgba[4 * i], textures[k].rgba[4 * i + 1], textures[k].rgba[4 * i + 2],
                         textures[k].rgba[4 * i + 3]};
        sc->textures.push_back(std::move(T));
    }
    sc->maps.clear();
    if (maps) sc->maps.assign(maps, maps + sc->materials.size());
    build_lights(sc);
}

void or_counts(const or_renderer *r, uint64_t *extension_rays, uint64_t *shadow_rays, uint64_t *paths) {
    if (extension_rays) *extension_rays = r->ext_rays.load();
    if (shadow_rays) *shadow_rays = r->shadow_rays.load();
    if (paths) *paths = r->paths.load();
}

void or_sample_counts(const or_renderer *r, uint32_t *cumulated, uint32_t *dispatched) {
    if (cumulated) *cumulated = r->cumulated;
    if (dispatched) *dispatched = r->dispatched;
}

void or_rng_fill(int32_t kind, uint64_t seed, uint32_t n, uint32_t *out_u32, float *out_unit) {
    Rng a, b;
    if (kind == SPK_RNG_XOSHIRO128P) {
        a.seed128(seed);
        b.seed128(seed);
    } else {
        a.seed256(seed);
        b.seed256(seed);
    }
    for (uint32_t k = 0; k < n; ++k) {
        if (out_u32) out_u32[k] = a.next_u32();
        if (out_unit) out_unit[k] = b.unit();
    }
}

uint32_t or_float_to_half(float f) { return f32_to_f16(f); }

// Eigen::half -> float: sign, 5-bit exponent, 10-bit mantissa; subnormals scaled by 2^-24.
static float f16_to_f32(uint16_t h) {
    const int e = (h >> 10) & 31, m = h & 1023;
    float v;
    if (e == 0) {
        v = std::ldexp(static_cast<float>(m), -24);
    } else if (e == 31) {
        v = m ? std::numeric_limits<float>::quiet_NaN() : std::numeric_limits<float>::infinity();
    } else {
        v = std::ldexp(static_cast<float>(1024 + m), e - 25);
    }
    return (h & 0x8000) ? -v : v;
}

// FloatToUint8 (Image.cpp:31-34). lround of a NaN is unspecified; it is taken as 0 here.
static uint8_t float_to_uint8(float v) {
    if (std::isnan(v)) return 0;
    return static_cast<uint8_t>(std::lround(std::clamp(v, 0.f, 1.f) * 255.f));
}

// SkyLightCookJob::Execute (SkyLight.cpp:83-113): face f texel (i, j) of an n x n cube holds the sky map's
// Image2D::Sample (Image.h:112-152) at CartesianToEquirectangular (Utilities.h:510-518) of
// TextureCoordinateToDirection(f, u, v) (Image.h:287-314) at the texel centre, stored through SetPixel
// into RGBAFloat16 (half RGB, alpha 1). `map` is w x h RGBA floats; `cube` receives 6 x n x n RGBA floats.
void or_sky_from_equirect(const float *map, uint32_t w, uint32_t h, int32_t srgb, uint32_t n, float *cube) {
    auto wrap = [](int a, unsigned b) { return (static_cast<unsigned>(a % static_cast<int>(b)) + b) % b; };
    auto decode = [](float c) { return c < 0.04045f ? c / 12.92f : std::pow((c + 0.055f) / 1.055f, 2.4f); };
    const float inv_pi = static_cast<float>(0.318309886183790671538);
    for (uint32_t f = 0; f < 6; ++f)
        for (uint32_t j = 0; j < n; ++j)
            for (uint32_t i = 0; i < n; ++i) {
                const float u = (static_cast<float>(i) + 0.5f) / static_cast<float>(n) * 2.f - 1.f;
                const float v = (static_cast<float>(j) + 0.5f) / static_cast<float>(n) * 2.f - 1.f;
                V3 d;
                switch (f) {
                case 0: d = V3{1.f, -v, -u}; break;
                case 1: d = V3{-1.f, -v, u}; break;
                case 2: d = V3{u, 1.f, v}; break;
                case 3: d = V3{u, -1.f, -v}; break;
                case 4: d = V3{u, -v, 1.f}; break;
                default: d = V3{-u, -v, -1.f}; break;
                }
                d = normalized(d);
                const float eu = std::atan2(d.y, d.x) * (inv_pi * 0.5f) + 0.5f;
                const float ev = std::asin(-d.z) * inv_pi + 0.5f;
                const float px = eu * static_cast<float>(w), py = ev * static_cast<float>(h);
                const int ui = static_cast<int>(px), vi = static_cast<int>(py);  // utilities::Decompose
                const float uc = px - static_cast<float>(ui), vc = py - static_cast<float>(vi);
                const float *s00 = map + 4ull * (wrap(vi, h) * w + wrap(ui, w));
                const float *s10 = map + 4ull * (wrap(vi, h) * w + wrap(ui + 1, w));
                const float *s01 = map + 4ull * (wrap(vi + 1, h) * w + wrap(ui, w));
                const float *s11 = map + 4ull * (wrap(vi + 1, h) * w + wrap(ui + 1, w));
                float *o = cube + 4ull * ((static_cast<uint64_t>(f) * n + j) * n + i);
                for (int c = 0; c < 3; ++c) {
                    const float l0 = s00[c] + (s10[c] - s00[c]) * uc, l1 = s01[c] + (s11[c] - s01[c]) * uc;
                    float r = l0 + (l1 - l0) * vc;
                    if (srgb) r = decode(r);
                    o[c] = f16_to_f32(static_cast<uint16_t>(f32_to_f16(r)));
                }
                o[3] = 1.f;
            }
}

// ConvertPixelsToRGBA8, the RGBAFloat16 case (Image.cpp:54-67): rgb.cwiseMax(0).cwiseMin(1), then
// utilities::LinearToSrgb = pow(x, 0.45f) (Utilities.h:411-414), each channel through FloatToUint8; alpha
// through FloatToUint8 alone.
void or_rgba16f_to_rgba8(const uint16_t *in, uint64_t pixels, uint8_t *out) {
    for (uint64_t i = 0; i < pixels; ++i) {
        for (int c = 0; c < 3; ++c) {
            float v = f16_to_f32(in[4 * i + c]);
            if (!std::isnan(v)) v = std::min(std::max(v, 0.f), 1.f);
            out[4 * i + c] = float_to_uint8(std::pow(v, 0.45f));
        }
        out[4 * i + 3] = float_to_uint8(f16_to_f32(in[4 * i + 3]));
    }
}

void or_sample_surface(const spk_material *m, const float ray_dir[3], const float normal[3], const float tangent[3],
                       uint32_t seed, float out[7]) {
    Rng rng;
    rng.seed128(seed);
    rng.draws = 0;
    V3 wi;
    const V3 thr = sample_surface(rng, *m, load3(ray_dir), load3(normal), load3(tangent), wi);
    out[0] = thr.x;
    out[1] = thr.y;
    out[2] = thr.z;
    out[3] = wi.x;
    out[4] = wi.y;
    out[5] = wi.z;
    out[6] = static_cast<float>(rng.draws);
}

}  // extern "C"
