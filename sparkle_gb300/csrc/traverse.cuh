// traverse.cuh -- two-level walk of the 8-wide quantised BVH (TLAS over instances, one BLAS per mesh).
//
// Semantics follow SceneRenderProxy::Intersect<AnyHit> (SceneRenderProxy.cpp:82-126) over
// MeshRenderProxy's BLAS (MeshRenderProxy.cpp:94-194) and SphereRenderProxy (SphereRenderProxy.cpp:5-38):
//  * closest hit: a triangle is accepted when Möller–Trumbore passes in local space and its world t,
//    computed the reference's way from the x component only (Ray::InverseAt, Ray.h:43-47), satisfies
//    0 < world_t < best (strict, so the first of equal t is kept);
//  * any hit (reference semantics): the first Möller–Trumbore pass (local t > Eps) or sphere with a
//    non-negative discriminant ends the walk (the reference does not test the sphere's t sign);
//  * occlusion (for next-event estimation): a hit with Eps < t < tmax ends the walk.
// Differences from the reference walk that cannot change a closest hit: the reference never lowers the
// ray's tmax (every box along the ray is visited); this walk prunes boxes that start beyond the current
// best t plus a bound on the x-only world-t rounding error, and visits children in an octant order.
// Two hits with bit-identical t go to the smaller (instance, face) rather than to the first visited, so
// the result never depends on the visit order (the reference's winner among exact ties does).
// One deliberate difference: for a direction component with |d| <= FLT_EPSILON, bvh v2's fast slab test
// uses 1/d = +-FLT_MAX and its -inv*org term overflows to +-inf once |org| > 1 on that axis, which culls
// every box of the level; here that axis is tested as an exact containment test instead.
//
// The walk is a resumable state machine (Walker::step) so persistent warps can replace finished rays
// with new ones while the others are still walking (dynamic ray fetch), and it postpones triangle groups
// when only a few lanes of the warp have triangles to test, keeping the lanes on the same kind of work.
#pragma once

#include "device_scene.cuh"

namespace spk {

enum : int { kTraceClosest = 0, kTraceAnyRef = 1, kTraceOcclusion = 2 };
enum : uint32_t { kErrStackOverflow = 1u, kErrIterationBudget = 2u, kErrQueueOverflow = 4u };

// Tunables (compile-time; the autotuner builds variants by defining them).
#ifndef SPK_POSTPONE_LANES
#define SPK_POSTPONE_LANES 8  // postpone triangle groups when fewer lanes than this want triangles
#endif
#ifndef SPK_REFILL_LANES
#define SPK_REFILL_LANES 20  // persistent warps refill idle lanes once fewer than this are walking
#endif
#ifndef SPK_BYTE_CONVERT_PRMT
#define SPK_BYTE_CONVERT_PRMT 0  // 1: quantised plane bytes to float with a byte permute + add
#endif
#ifndef SPK_POSTPONE_INNER
#define SPK_POSTPONE_INNER 0  // 1: also postpone inside the triangle loop as lanes drop out of it
#endif
#ifndef SPK_MINMAX3
#define SPK_MINMAX3 0  // 1: slab entry/exit with three-input min/max (exact, same results)
#endif
#ifndef SPK_META_SIMD
#define SPK_META_SIMD 1  // 1: the four meta bytes of a half node decoded together with 32-bit SIMD-in-register ops
#endif
#ifndef SPK_MT_RCP
#define SPK_MT_RCP 1  // 1: Moller-Trumbore's 1/det as a correctly rounded reciprocal (same bits as 1.f/det)
#endif
#ifndef SPK_SLAB_RCP
#define SPK_SLAB_RCP 0  // 1: the slab reciprocals as correctly rounded reciprocals (same bits as 1.f/x)
#endif
#ifndef SPK_WALK_MIN_BLOCKS
#define SPK_WALK_MIN_BLOCKS 7  // resident 128-thread blocks per SM of the closest-hit walks (72 registers)
#endif
#ifndef SPK_SHADOW_MIN_BLOCKS
#define SPK_SHADOW_MIN_BLOCKS 8  // the same for the occlusion walk of the shadow stage (64 registers)
#endif
#ifndef SPK_PACKET_MIN_BLOCKS
#define SPK_PACKET_MIN_BLOCKS 8  // resident 128-thread blocks per SM the packet walk is compiled for
#endif
#ifndef SPK_PACKET2_MIN_BLOCKS
#define SPK_PACKET2_MIN_BLOCKS 6  // resident 128-thread blocks per SM the two-rays-per-lane packet walk is compiled for
#endif
#ifndef SPK_FRUSTUM_SPREAD
#define SPK_FRUSTUM_SPREAD 0.25f  // largest relative spread of a packet's slab reciprocals tested as one
#endif
#ifndef SPK_PACKET_FRUSTUM
#define SPK_PACKET_FRUSTUM 1  // 1: packets of one octant test each node once for all rays (0: every lane its own ray)
#endif
#ifndef SPK_PACKET_WORLD_SMEM
#define SPK_PACKET_WORLD_SMEM 1  // 1: packet walks keep each lane's world rays in shared memory, not registers
#endif
#ifndef SPK_PACKET_SIBLINGS
#define SPK_PACKET_SIBLINGS 4  // sibling nodes a packet tests at once (one per 8-lane group), 1..4
#endif
#ifndef SPK_SMEM_STACK
#define SPK_SMEM_STACK 0  // top entries of each persistent walk's stack kept in shared memory (0: all local)
#endif
#ifndef SPK_STACK_REGTOP
#define SPK_STACK_REGTOP 0  // 1: the top entry of each persistent walk's local stack cached in registers
#endif

constexpr int kStackSize = 48;
constexpr int kWalkThreads = 128;  // threads per block of every persistent walking kernel
constexpr uint32_t kMaxIterations = 1u << 20;
constexpr int kPostponeLanes = SPK_POSTPONE_LANES;
constexpr uint32_t kPacketSiblings = SPK_PACKET_SIBLINGS;
constexpr uint32_t kPacketStack = 64;  // packet walks push up to 2 * kPacketSiblings - 1 groups per node step
static_assert(kPacketSiblings >= 1 && kPacketSiblings <= 4, "one to four 8-lane groups");

// Byte `c` of `word` as a float (exact for 0..255).
__device__ __forceinline__ float byte_to_float(uint32_t word, int c) {
#if SPK_BYTE_CONVERT_PRMT
    // 0x4B0000xx is 2^23 + xx; subtracting 2^23 is exact.
    return __uint_as_float(__byte_perm(word, 0x4B000000u, 0x7540u | static_cast<uint32_t>(c))) - 8388608.0f;
#else
    return static_cast<float>((word >> (8 * c)) & 0xFFu);
#endif
}

struct TraceResult {
    float t, u, v;
    uint32_t inst;  // caller instance index, kInvalid on a miss
    uint32_t face;  // original face index, kInvalid for spheres and misses
};

// Per-thread traffic counters of the instrumented walk (wide nodes visited, triangles tested).
struct TraceCounts {
    uint32_t nodes = 0, tris = 0;
};

struct LevelRay {
    f3 o, d, inv;
    uint32_t oct;  // bit k set when direction component k is negative
};

// Reciprocal for the slab test; a component with |d| <= FLT_EPSILON gets +-2^100 so that
// (bound - o) * inv keeps its exact sign without overflowing (an exact containment test on that axis).
__device__ __forceinline__ float slab_inverse(float x) {
#if SPK_SLAB_RCP
    return fabsf(x) <= 1.1920928955078125e-07f ? copysignf(0x1p100f, x) : __frcp_rn(x);  // the bits of 1.f / x
#else
    return fabsf(x) <= 1.1920928955078125e-07f ? copysignf(0x1p100f, x) : 1.f / x;
#endif
}

__device__ __forceinline__ void setup_level(LevelRay &r, f3 o, f3 d) {
    r.o = o;
    r.d = d;
    r.inv = mk3(slab_inverse(d.x), slab_inverse(d.y), slab_inverse(d.z));
    r.oct = (signbit(d.x) ? 1u : 0u) | (signbit(d.y) ? 2u : 0u) | (signbit(d.z) ? 4u : 0u);
}

// Upper bound on the t a box may start at and still hold a hit closer than `best` (in world-t terms).
__device__ __forceinline__ float prune_limit(float best, f3 wo, f3 wd, float scene_abs_x) {
    if (!(best < kFltMax)) return kFltMax;
    const float ax = fabsf(wd.x);
    const float slack = ax > 0.f ? (fabsf(wo.x) + scene_abs_x) * 0x1p-18f / ax : kFltMax;
    const float lim = best * (1.f + 0x1p-14f) + slack;
    return isfinite(lim) ? lim : kFltMax;
}

// Slab test of the 8 children of one wide node; returns the next node group (inner children, permuted
// slot bits 24..31 + imask in bits 0..7) and triangle group (leaf items, bits 0..23). The ray's own octant
// picks each slab's near and far planes; `order` (an octant) permutes the inner children's bits, which sets
// the visiting order (a single-ray walk passes its own octant, a packet one octant shared by its lanes).
// Three-input max / min (PTX max.f32 / min.f32 with three operands): the same value as the two-input
// forms applied in turn, NaN operands ignored.
__device__ __forceinline__ float max3f(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

__device__ __forceinline__ void visit_node(const uint4 *__restrict__ nodes, uint32_t idx, const LevelRay &r,
                                           uint32_t order, float tmax, uint2 &ngroup, uint2 &tgroup) {
    const uint4 *np = nodes + static_cast<size_t>(idx) * 5;
    const uint4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2), n3 = __ldg(np + 3), n4 = __ldg(np + 4);
    const float sx = __uint_as_float((n0.w & 0xFFu) << 23);
    const float sy = __uint_as_float(((n0.w >> 8) & 0xFFu) << 23);
    const float sz = __uint_as_float(((n0.w >> 16) & 0xFFu) << 23);
    const float ax = sx * r.inv.x, ay = sy * r.inv.y, az = sz * r.inv.z;
    const float ox = (__uint_as_float(n0.x) - r.o.x) * r.inv.x;
    const float oy = (__uint_as_float(n0.y) - r.o.y) * r.inv.y;
    const float oz = (__uint_as_float(n0.z) - r.o.z) * r.inv.z;
    uint32_t hitmask = 0;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const uint32_t meta4 = h ? n1.w : n1.z;
        const uint32_t lox = h ? n2.y : n2.x, loy = h ? n2.w : n2.z, loz = h ? n3.y : n3.x;
        const uint32_t hix = h ? n3.w : n3.z, hiy = h ? n4.y : n4.x, hiz = h ? n4.w : n4.z;
        const uint32_t nx = (r.oct & 1u) ? hix : lox, fx = (r.oct & 1u) ? lox : hix;
        const uint32_t ny = (r.oct & 2u) ? hiy : loy, fy = (r.oct & 2u) ? loy : hiy;
        const uint32_t nz = (r.oct & 4u) ? hiz : loz, fz = (r.oct & 4u) ? loz : hiz;
#if SPK_META_SIMD
        // Per byte: an inner child has bits 3 and 4 of its meta set; its slot bit is xor-ed with the ray's
        // octant. bit4 = the hit-mask bit index of each child, bits4 = the bits it sets there (0 for an
        // empty slot, whose meta byte is 0, so empty slots need no test of their own).
        const uint32_t inner4 = (meta4 & (meta4 << 1)) & 0x10101010u;
        const uint32_t bit4 = (meta4 ^ ((inner4 >> 4) * order)) & 0x1F1F1F1Fu;
        const uint32_t bits4 = (meta4 >> 5) & 0x07070707u;
#endif
#pragma unroll
        for (int c = 0; c < 4; ++c) {
#if !SPK_META_SIMD
            const uint32_t m = (meta4 >> (8 * c)) & 0xFFu;
#endif
            const float tnx = fmaf(byte_to_float(nx, c), ax, ox);
            const float tny = fmaf(byte_to_float(ny, c), ay, oy);
            const float tnz = fmaf(byte_to_float(nz, c), az, oz);
            const float tfx = fmaf(byte_to_float(fx, c), ax, ox);
            const float tfy = fmaf(byte_to_float(fy, c), ay, oy);
            const float tfz = fmaf(byte_to_float(fz, c), az, oz);
#if SPK_MINMAX3
            const float t0 = max3f(tnx, tny, fmaxf(tnz, 0.f));
            const float t1 = min3f(tfx, tfy, fminf(tfz, tmax));
#else
            const float t0 = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, 0.f));
            const float t1 = fminf(fminf(tfx, tfy), fminf(tfz, tmax));
#endif
#if SPK_META_SIMD
            if (t0 <= t1) hitmask |= __byte_perm(bits4, 0u, 0x4440u | c) << __byte_perm(bit4, 0u, 0x4440u | c);
#else
            if (m != 0u && t0 <= t1) {
                uint32_t bit = m & 0x1Fu;
                if ((m & 0x18u) == 0x18u) bit ^= order;
                hitmask |= ((m >> 5) & 7u) << bit;
            }
#endif
        }
    }
    ngroup = make_uint2(n1.x, (hitmask & 0xFF000000u) | (n0.w >> 24));
    tgroup = make_uint2(n1.y, hitmask & 0x00FFFFFFu);
}

// Möller–Trumbore (MeshRenderProxy.cpp:128-194) of triangle record `idx` in the level ray's (the instance's
// local) space: true when the ray passes with local t > Eps, with (t, u, v) and the record's face index.
__device__ __forceinline__ bool triangle_hit(const float4 *__restrict__ tris, uint32_t idx, const LevelRay &ray,
                                             float &t, float &u, float &v, uint32_t &face) {
    const float4 *tp = tris + static_cast<size_t>(idx) * 3;
    const float4 a4 = __ldg(tp), b4 = __ldg(tp + 1), c4 = __ldg(tp + 2);
    const f3 p0 = mk3(a4.x, a4.y, a4.z), e1 = mk3(a4.w, b4.x, b4.y), e2 = mk3(b4.z, b4.w, c4.x);
    const f3 h = cross(ray.d, e2);
    const float det = dot3(e1, h);
    if (fabsf(det) < kEps) return false;
    const f3 s = ray.o - p0;
#if SPK_MT_RCP
    const float f = __frcp_rn(det);
#else
    const float f = 1.f / det;
#endif
    u = f * dot3(s, h);
    if (u < 0.f || u > 1.f) return false;
    const f3 q = cross(s, e1);
    v = f * dot3(ray.d, q);
    if (v < 0.f || u + v > 1.f) return false;
    t = f * dot3(e2, q);
    face = __float_as_uint(c4.y);
    return t > kEps;
}

// World t of a local hit at `t`, the reference's way: from the x component only (Ray::InverseAt, Ray.h:43-47).
__device__ __forceinline__ float world_t(const DevInstance &I, const LevelRay &ray, float t, f3 wo, f3 wd) {
    const f3 wp = xform_point(I.m, ray.o + ray.d * t);
    return (wp.x - wo.x) / wd.x;
}

// SphereRenderProxy::IntersectInternal (SphereRenderProxy.cpp:5-38) in world space: false when the
// discriminant is negative, else true with the root the reference takes (the near one from outside).
__device__ __forceinline__ bool sphere_hit(const DevInstance &I, f3 wo, f3 wd, float &t) {
    const f3 center = mk3(I.m[3], I.m[7], I.m[11]);
    const f3 co = wo - center;
    const float half_b = dot3(wd, co);
    const float c = sqnorm(co) - I.radius * I.radius;
    const float disc = half_b * half_b - 1.f * c;
    if (disc < 0.f) return false;
    const float sq = sqrtf(disc);
    t = (-half_b + (c >= 0.f ? -sq : sq)) / 1.f;
    return true;
}

// Traversal stacks. Walker::push / pop address entry `i` (0 = bottom) of the current ray's stack.
// LocalStack: the whole stack in local memory (one-thread walks).
struct LocalStack {
    uint2 e[kStackSize];
    __device__ __forceinline__ void reset() {}
    __device__ __forceinline__ void put(int i, uint2 v) { e[i] = v; }
    __device__ __forceinline__ uint2 take(int i) { return e[i]; }
};

// SharedRingStack: the top K entries in a per-thread ring of shared memory, deeper entries in local memory.
// Invariant: entries [max(0, sp - K), sp) are in the ring, entry i in slot i mod K; pushing entry i >= K
// first moves entry i - K out to local memory, popping it brings entry i - K back into the freed slot. The
// ring is a column of the block's array (slot k of thread t at k * kWalkThreads + t): the 16 lanes of a
// half-warp touch 16 consecutive 8-byte words whatever their depths, so accesses are free of bank conflicts.
template <int K>
struct SharedRingStack {
    static_assert(K > 0 && (K & (K - 1)) == 0 && K < kStackSize, "ring size: a power of two below the stack size");
    uint2 *ring;  // this thread's slot 0
    uint2 spill[kStackSize - K];
    __device__ __forceinline__ void reset() {}
    __device__ __forceinline__ void put(int i, uint2 v) {
        uint2 *slot = ring + (i & (K - 1)) * kWalkThreads;
        if (i >= K) spill[i - K] = *slot;
        *slot = v;
    }
    __device__ __forceinline__ uint2 take(int i) {
        uint2 *slot = ring + (i & (K - 1)) * kWalkThreads;
        const uint2 v = *slot;
        if (i >= K) *slot = spill[i - K];
        return v;
    }
};

// RegTopStack: a local stack whose top entry may live in registers instead (`cached`): a push moves the
// cached entry out to local memory and caches the new one, a pop returns the cached entry when there is
// one, so a push followed by its pop touches no memory.
struct RegTopStack {
    uint2 top;
    bool cached = false;
    uint2 e[kStackSize];
    // A walk that ended early (an occlusion hit) may leave entries behind, the top one cached.
    __device__ __forceinline__ void reset() { cached = false; }
    __device__ __forceinline__ void put(int i, uint2 v) {
        if (cached) e[i - 1] = top;
        top = v;
        cached = true;
    }
    __device__ __forceinline__ uint2 take(int i) {
        if (cached) {
            cached = false;
            return top;
        }
        return e[i];
    }
};

// True when a hit at world t `t` on (inst, face) replaces `best`: a smaller t, or an exact tie on a smaller
// (instance, face).
__device__ __forceinline__ bool closer_hit(const TraceResult &best, float t, uint32_t inst, uint32_t face) {
    if (t < best.t) return true;
    return t == best.t && (inst < best.inst || (inst == best.inst && face < best.face));
}

// Resumable two-level walk of one ray. init() starts it; step() advances by one node visit plus the
// triangle tests it enables and returns true when the walk is over (result in `best`).
template <int kMode, bool kCount>
struct Walker {
    f3 wo, wd;
    LevelRay ray;
    uint2 ngroup, tgroup;
    int sp, blas_sp;
    uint32_t cur_inst;
    uint32_t iter, budget;
    bool in_blas;
    float tmax_box, tmax_occl;
    TraceResult best;

    // `root` is the TLAS root node of the ray's scene (S.tlas_root for a single-scene context).
    __device__ __forceinline__ void init(const DevScene &S, uint32_t root, f3 o, f3 d, float tmax) {
        wo = o;
        wd = d;
        setup_level(ray, o, d);
        ngroup = make_uint2(root, root == kInvalid ? 0u : (1u << 24));
        tgroup = make_uint2(0u, 0u);
        sp = 0;
        blas_sp = 0;
        cur_inst = 0;
        iter = 0;
        budget = S.walk_budget ? S.walk_budget : kMaxIterations;
        in_blas = false;
        tmax_occl = tmax;
        tmax_box = (kMode == kTraceOcclusion) ? tmax : kFltMax;
        best = TraceResult{kFltMax, 0.f, 0.f, kInvalid, kInvalid};
    }

    // Candidate acceptance. The reference keeps the first of equal t (IntersectionCandidate::IsCloserHit is
    // a strict <), which depends on the visit order; this walk's order depends on warp composition, so an
    // exact tie goes to the smaller (instance, face) instead, making every hit independent of scheduling.
    __device__ __forceinline__ bool closer(float t, uint32_t inst, uint32_t face) const {
        return closer_hit(best, t, inst, face);
    }

    template <class Stack>
    __device__ __forceinline__ void push(Stack &stack, uint2 v, uint32_t &err) {
        if (sp < kStackSize) {
            stack.put(sp++, v);
        } else {
            err |= kErrStackOverflow;
        }
    }

    template <class Stack>
    __device__ __forceinline__ bool step(const DevScene &S, Stack &stack, uint32_t &err, TraceCounts *counts) {
        if (++iter > budget) {
            err |= kErrIterationBudget;
            return true;
        }
        if (ngroup.y > 0x00FFFFFFu) {
            const uint32_t bit = __ffs(ngroup.y >> 24) - 1;
            ngroup.y &= ~(1u << (bit + 24));
            const uint32_t slot = bit ^ ray.oct;
            const uint32_t node_idx = ngroup.x + __popc(ngroup.y & 0xFFu & ((1u << slot) - 1u));
            if (ngroup.y > 0x00FFFFFFu) push(stack, ngroup, err);
            visit_node(S.nodes, node_idx, ray, ray.oct, tmax_box, ngroup, tgroup);
            if (kCount) ++counts->nodes;
            // Triangle postponing: when few lanes have triangles, keep walking nodes and test them later.
            const uint32_t want = __ballot_sync(__activemask(), tgroup.y != 0u);
            if (tgroup.y != 0u && ngroup.y > 0x00FFFFFFu && __popc(want) < kPostponeLanes) {
                push(stack, tgroup, err);
                tgroup.y = 0u;
            }
        } else {
            tgroup = ngroup;
            ngroup = make_uint2(0u, 0u);
        }
        while (tgroup.y != 0u) {
#if SPK_POSTPONE_INNER
            // Lanes drop out of this loop as their triangles run out; once too few are left, the rest park
            // their remaining triangles and rejoin the node walk (only when a node visit is pending, so
            // the parked group cannot come straight back).
            if (in_blas && ngroup.y > 0x00FFFFFFu && __popc(__activemask()) < kPostponeLanes) {
                push(stack, tgroup, err);
                tgroup.y = 0u;
                break;
            }
#endif
            const uint32_t k = __ffs(tgroup.y) - 1;
            tgroup.y &= tgroup.y - 1u;
            const uint32_t idx = tgroup.x + k;
            if (in_blas) {
                if (kCount) ++counts->tris;
                float t, u, v;
                uint32_t face;
                if (!triangle_hit(S.tris, idx, ray, t, u, v, face)) continue;
                if (kMode == kTraceAnyRef) {
                    best.inst = cur_inst;
                    return true;
                }
                if (kMode == kTraceOcclusion) {
                    if (t < tmax_occl) {
                        best.inst = cur_inst;
                        return true;
                    }
                    continue;
                }
                const float wt = world_t(S.instances[cur_inst], ray, t, wo, wd);
                if (wt > 0.f && closer(wt, cur_inst, face)) {
                    best.t = wt;
                    best.u = u;
                    best.v = v;
                    best.inst = cur_inst;
                    best.face = face;
                    tmax_box = prune_limit(best.t, wo, wd, S.scene_abs_x);
                }
            } else {
                const uint32_t inst = __ldg(S.tlas_items + idx);
                const DevInstance &I = S.instances[inst];
                if (I.type == 1u) {
                    // SphereRenderProxy::IntersectInternal (SphereRenderProxy.cpp:5-38), world space: sphere_hit's
                    // test, written out so the any-hit modes stop before the square root.
                    const f3 center = mk3(I.m[3], I.m[7], I.m[11]);
                    const f3 co = wo - center;
                    const float half_b = dot3(wd, co);
                    const float c = sqnorm(co) - I.radius * I.radius;
                    const float disc = half_b * half_b - 1.f * c;
                    if (disc < 0.f) continue;
                    if (kMode == kTraceAnyRef) {
                        best.inst = inst;
                        return true;
                    }
                    const float sq = sqrtf(disc);
                    const float t = (-half_b + (c >= 0.f ? -sq : sq)) / 1.f;
                    if (kMode == kTraceOcclusion) {
                        if (t > kEps && t < tmax_occl) {
                            best.inst = inst;
                            return true;
                        }
                        continue;
                    }
                    if (t > 0.f && closer(t, inst, kInvalid)) {
                        best.t = t;
                        best.u = 0.f;
                        best.v = 0.f;
                        best.inst = inst;
                        best.face = kInvalid;
                        tmax_box = prune_limit(best.t, wo, wd, S.scene_abs_x);
                    }
                } else if (I.blas_root != kInvalid) {
                    // Enter the BLAS: park the rest of this TLAS level on the stack.
                    if (tgroup.y != 0u) push(stack, tgroup, err);
                    if (ngroup.y > 0x00FFFFFFu) push(stack, ngroup, err);
                    blas_sp = sp;
                    in_blas = true;
                    cur_inst = inst;
                    setup_level(ray, xform_point(I.minv, wo), xform_dir(I.minv, wd));
                    ngroup = make_uint2(I.blas_root, 1u << 24);
                    tgroup.y = 0u;
                    break;
                }
            }
        }
        if (ngroup.y <= 0x00FFFFFFu) {
            if (in_blas && sp == blas_sp) {
                in_blas = false;
                setup_level(ray, wo, wd);
            }
            if (sp == 0) return true;
            ngroup = stack.take(--sp);
        }
        return false;
    }
};

// Whole walk of one ray by one thread (no lane refill).
template <int kMode, bool kCount = false>
__device__ __forceinline__ TraceResult trace_ray(const DevScene &S, f3 wo, f3 wd, float tmax_occl, uint32_t &err,
                                                 TraceCounts *counts = nullptr) {
    LocalStack stack;
    Walker<kMode, kCount> w;
    w.init(S, S.tlas_root, wo, wd, tmax_occl);
    while (!w.step(S, stack, err, counts)) {
    }
    return w.best;
}

// Persistent walk over a work list: each warp pulls batches of items from `cursor` and refills lanes whose
// ray has finished once fewer than `kRefillLanes` lanes are still walking. `fetch(i, o, d, tmax)` loads item
// i's ray (tmax starts at the call's `tmax`; an occlusion walk may lower it per ray) and returns the TLAS
// root of its scene; `finish(i, result)` stores its result. Every lane of every warp of the block must call
// this, and the block must have kWalkThreads threads (the shared stack rings are laid out for that many).
constexpr int kRefillLanes = SPK_REFILL_LANES;

template <int kMode, bool kCount, class Fetch, class Finish>
__device__ __forceinline__ void walk_persistent(const DevScene &S, unsigned long long *cursor, unsigned long long n,
                                                float tmax, uint32_t &err, TraceCounts *counts, Fetch &&fetch,
                                                Finish &&finish) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt_mask = (1u << lane) - 1u;
#if SPK_SMEM_STACK > 0
    __shared__ uint2 rings[SPK_SMEM_STACK * kWalkThreads];
    SharedRingStack<SPK_SMEM_STACK> stack;
    stack.ring = rings + threadIdx.x;
#elif SPK_STACK_REGTOP
    RegTopStack stack;
#else
    LocalStack stack;
#endif
    Walker<kMode, kCount> w;
    bool active = false, exhausted = false;
    unsigned long long item = 0;
    for (;;) {
        const uint32_t idle = __ballot_sync(0xFFFFFFFFu, !active);
        if (!exhausted && idle != 0u) {
            const uint32_t cnt = __popc(idle);
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(cursor, static_cast<unsigned long long>(cnt));
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (base + cnt >= n) exhausted = true;
            if (!active) {
                const unsigned long long q = base + __popc(idle & lt_mask);
                if (q < n) {
                    item = q;
                    f3 o, d;
                    float tm = tmax;
                    const uint32_t root = fetch(q, o, d, tm);
                    w.init(S, root, o, d, tm);
                    stack.reset();
                    active = true;
                }
            }
        }
        if (__ballot_sync(0xFFFFFFFFu, active) == 0u) {
            if (exhausted) break;
            continue;
        }
        while (active) {
            if (w.step(S, stack, err, counts)) {
                finish(item, w.best);
                active = false;
            }
            if (!exhausted && __popc(__ballot_sync(__activemask(), active)) < kRefillLanes) break;
        }
    }
}

// Order-preserving map of a float to an int (and back) for warp min / max reductions.
__device__ __forceinline__ int float_key(float x) {
    const int b = __float_as_int(x);
    return b ^ ((b >> 31) & 0x7FFFFFFF);
}
__device__ __forceinline__ float key_float(int k) { return __int_as_float(k ^ ((k >> 31) & 0x7FFFFFFF)); }
__device__ __forceinline__ float warp_min(float x) { return key_float(__reduce_min_sync(0xFFFFFFFFu, float_key(x))); }
__device__ __forceinline__ float warp_max(float x) { return key_float(__reduce_max_sync(0xFFFFFFFFu, float_key(x))); }

// Bounds of a packet's level rays: origins and slab reciprocals per axis over the warp's 32 lanes.
struct PacketFrustum {
    f3 omin, omax, imin, imax;
};

// Fills `f` from the level rays of every lane (kRays per lane) and returns true when the packet can be tested
// as one: every ray's direction lies in octant `order` and no component is small enough for slab_inverse's
// 2^100 stand-in (so every bound below stays finite). Every lane of the warp must call this.
template <int kRays>
__device__ __forceinline__ bool make_frustum(const LevelRay (&r)[kRays], uint32_t order, PacketFrustum &f) {
    bool ok = true;
    f3 omin = r[0].o, omax = r[0].o, imin = r[0].inv, imax = r[0].inv;
#pragma unroll
    for (int k = 0; k < kRays; ++k) {
        ok = ok && r[k].oct == order && fabsf(r[k].inv.x) < 0x1p24f && fabsf(r[k].inv.y) < 0x1p24f &&
             fabsf(r[k].inv.z) < 0x1p24f;
        if (k > 0) {
            omin = mk3(fminf(omin.x, r[k].o.x), fminf(omin.y, r[k].o.y), fminf(omin.z, r[k].o.z));
            omax = mk3(fmaxf(omax.x, r[k].o.x), fmaxf(omax.y, r[k].o.y), fmaxf(omax.z, r[k].o.z));
            imin = mk3(fminf(imin.x, r[k].inv.x), fminf(imin.y, r[k].inv.y), fminf(imin.z, r[k].inv.z));
            imax = mk3(fmaxf(imax.x, r[k].inv.x), fmaxf(imax.y, r[k].inv.y), fmaxf(imax.z, r[k].inv.z));
        }
    }
    if (!__all_sync(0xFFFFFFFFu, ok)) return false;
    f.omin = mk3(warp_min(omin.x), warp_min(omin.y), warp_min(omin.z));
    f.omax = mk3(warp_max(omax.x), warp_max(omax.y), warp_max(omax.z));
    f.imin = mk3(warp_min(imin.x), warp_min(imin.y), warp_min(imin.z));
    f.imax = mk3(warp_max(imax.x), warp_max(imax.y), warp_max(imax.z));
    // The bounds of (p - org) * inv widen with the spread of inv relative to its size: past a few tens of
    // percent (a component near zero in some rays) the packet test stops culling and walks far more nodes
    // than its rays need, so such a packet tests with its own rays instead.
    const float k = SPK_FRUSTUM_SPREAD;
    return f.imax.x - f.imin.x <= k * fminf(fabsf(f.imin.x), fabsf(f.imax.x)) &&
           f.imax.y - f.imin.y <= k * fminf(fabsf(f.imin.y), fabsf(f.imax.y)) &&
           f.imax.z - f.imin.z <= k * fminf(fabsf(f.imin.z), fabsf(f.imax.z));
}

// Bounds over the packet of one axis's slab terms: a = s * inv and o = (p - org) * inv, the two values
// visit_node forms per ray (t = fma(q, a, o) for a plane byte q). Each is a product or difference of the
// lanes' values, so rounding to nearest keeps them within the products and differences of the extremes.
__device__ __forceinline__ void axis_bounds(float p, float s, float omin, float omax, float imin, float imax,
                                            float &alo, float &ahi, float &olo, float &ohi) {
    alo = s * imin;
    ahi = s * imax;
    const float nlo = p - omax, nhi = p - omin;
    const float c0 = nlo * imin, c1 = nlo * imax, c2 = nhi * imin, c3 = nhi * imax;
    olo = fminf(fminf(c0, c1), fminf(c2, c3));
    ohi = fmaxf(fmaxf(c0, c1), fmaxf(c2, c3));
}

// visit_node for a whole packet at once: each 8-lane group of the warp visits node `idx` (its own: the groups
// may visit different nodes), lane k testing child slot k mod 8 against the packet's bounds, and the group
// ORs the results. fma(q, a, o) grows with a (q >= 0) and with o, so the lower bound of each near-plane t and
// the upper bound of each far-plane t take the extremes of a and o: a child passes whenever it passes for at
// least one lane's own ray with that lane's tmax (<= `tmax`), as visit_node computes it, and may pass for
// none (the packet then visits a node that none of its rays needs, which only costs time). Every lane of the
// warp must call this; the result is the same in every lane of a group.
__device__ __forceinline__ void visit_node_frustum(const uint4 *__restrict__ nodes, uint32_t idx,
                                                   const PacketFrustum &f, uint32_t order, float tmax,
                                                   uint2 &ngroup, uint2 &tgroup) {
    const uint4 *np = nodes + static_cast<size_t>(idx) * 5;
    const uint4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2), n3 = __ldg(np + 3), n4 = __ldg(np + 4);
    float axlo, axhi, oxlo, oxhi, aylo, ayhi, oylo, oyhi, azlo, azhi, ozlo, ozhi;
    axis_bounds(__uint_as_float(n0.x), __uint_as_float((n0.w & 0xFFu) << 23), f.omin.x, f.omax.x, f.imin.x,
                f.imax.x, axlo, axhi, oxlo, oxhi);
    axis_bounds(__uint_as_float(n0.y), __uint_as_float(((n0.w >> 8) & 0xFFu) << 23), f.omin.y, f.omax.y, f.imin.y,
                f.imax.y, aylo, ayhi, oylo, oyhi);
    axis_bounds(__uint_as_float(n0.z), __uint_as_float(((n0.w >> 16) & 0xFFu) << 23), f.omin.z, f.omax.z,
                f.imin.z, f.imax.z, azlo, azhi, ozlo, ozhi);
    const uint32_t slot = threadIdx.x & 7u, h = slot >> 2, c = slot & 3u;
    const uint32_t meta4 = h ? n1.w : n1.z;
    const uint32_t lox = h ? n2.y : n2.x, loy = h ? n2.w : n2.z, loz = h ? n3.y : n3.x;
    const uint32_t hix = h ? n3.w : n3.z, hiy = h ? n4.y : n4.x, hiz = h ? n4.w : n4.z;
    const uint32_t nx = (order & 1u) ? hix : lox, fx = (order & 1u) ? lox : hix;
    const uint32_t ny = (order & 2u) ? hiy : loy, fy = (order & 2u) ? loy : hiy;
    const uint32_t nz = (order & 4u) ? hiz : loz, fz = (order & 4u) ? loz : hiz;
    const uint32_t sel = 0x4440u | c;
    const float t0 = fmaxf(fmaxf(fmaf(static_cast<float>(__byte_perm(nx, 0u, sel)), axlo, oxlo),
                                 fmaf(static_cast<float>(__byte_perm(ny, 0u, sel)), aylo, oylo)),
                           fmaxf(fmaf(static_cast<float>(__byte_perm(nz, 0u, sel)), azlo, ozlo), 0.f));
    const float t1 = fminf(fminf(fmaf(static_cast<float>(__byte_perm(fx, 0u, sel)), axhi, oxhi),
                                 fmaf(static_cast<float>(__byte_perm(fy, 0u, sel)), ayhi, oyhi)),
                           fminf(fmaf(static_cast<float>(__byte_perm(fz, 0u, sel)), azhi, ozhi), tmax));
    const uint32_t m = __byte_perm(meta4, 0u, sel);
    uint32_t bits = 0u;
    if (m != 0u && t0 <= t1) {
        uint32_t bit = m & 0x1Fu;
        if ((m & 0x18u) == 0x18u) bit ^= order;
        bits = ((m >> 5) & 7u) << bit;
    }
    uint32_t any = bits | __shfl_xor_sync(0xFFFFFFFFu, bits, 1);
    any |= __shfl_xor_sync(0xFFFFFFFFu, any, 2);
    any |= __shfl_xor_sync(0xFFFFFFFFu, any, 4);
    ngroup = make_uint2(n1.x, (any & 0xFF000000u) | (n0.w >> 24));
    tgroup = make_uint2(n1.y, any & 0x00FFFFFFu);
}

// Closest-hit walk of coherent rays in packets (primary rays: the samples of one pixel, or neighbouring
// pixels). Each warp takes 32 * kRays consecutive items of the work list (lane l the items l, l + 32, ...)
// and walks them together: one node or triangle group at a time for the whole warp, in the order of the
// leader's octant, every lane testing its own rays against each triangle. When all the packet's rays share
// that octant (checked per level, TLAS and each BLAS), a node's 8 children are tested once for the whole
// packet (visit_node_frustum: one child per lane against the bounds of all its rays); otherwise every lane
// tests them with its own rays (visit_node) and takes only the children they hit. Either way a ray is tested
// against every box and triangle its own walk would reach, and pruned only beyond its own best t; it may be
// tested against more. Its result is still the smallest world t over every triangle and sphere it hits
// (exact ties to the smaller (instance, face)), which no visiting order or extra test changes: the results
// are walk_persistent's. `fetch(i, o, d, tmax)` and `finish(i, result)` as for walk_persistent (`fetch` may
// be called more than once for an item, `finish` must find the item from i alone); every lane of the warp
// must call this. `counts` (kCount) takes each node and triangle once per packet: one fetch serves its rays.
template <bool kCount, int kRays, class Fetch, class Finish>
__device__ __forceinline__ void walk_packets(const DevScene &S, unsigned long long *cursor, unsigned long long n,
                                             uint32_t &err, TraceCounts *counts, Fetch &&fetch, Finish &&finish) {
    static_assert(kRays == 1 || kRays == 2, "one or two rays per lane");
    constexpr uint32_t kAll = 0xFFFFFFFFu;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t budget = S.walk_budget ? S.walk_budget : kMaxIterations;
    uint2 groups[kPacketStack];  // the shared groups (the same in every lane)
    uint32_t own[kPacketStack];  // this lane's hit bits of each
#if SPK_PACKET_WORLD_SMEM
    // Each lane's world rays (origin, direction per ray) wait in shared memory, read only at a BLAS exit and
    // for a candidate hit's world t: entry k of thread t at [k][t], consecutive lanes in consecutive words.
    __shared__ float4 world[2 * kRays][kWalkThreads];
    auto world_o = [&](int r) { const float4 v = world[2 * r][threadIdx.x]; return mk3(v.x, v.y, v.z); };
    auto world_d = [&](int r) { const float4 v = world[2 * r + 1][threadIdx.x]; return mk3(v.x, v.y, v.z); };
#endif
    unsigned long long base = 0;
    bool todo[kRays];  // this lane's items not walked yet
#pragma unroll
    for (int r = 0; r < kRays; ++r) todo[r] = false;
    for (;;) {
        bool any_todo = false;
#pragma unroll
        for (int r = 0; r < kRays; ++r) any_todo = any_todo || todo[r];
        if (!__any_sync(kAll, any_todo)) {
            unsigned long long b = 0;
            if (lane == 0) b = atomicAdd(cursor, 32ull * kRays);
            base = __shfl_sync(kAll, b, 0);
            if (base >= n) break;
#pragma unroll
            for (int r = 0; r < kRays; ++r) todo[r] = base + lane + 32u * r < n;  // lane 0's first always
            any_todo = todo[0];
        }
        // One packet per TLAS root among the items (a batch of requests holds several scenes; almost every
        // warp has one). The packet is the rays with the leader's root (its lowest pending item's); the
        // others, and items past the end of the list, walk a copy of that ray and drop their results, which
        // keeps the packet's bounds and octant those of its real rays.
        const int leader = __ffs(__ballot_sync(kAll, any_todo)) - 1;
        f3 wo[kRays], wd[kRays];
        uint32_t root[kRays];
        bool valid[kRays];
#pragma unroll
        for (int r = 0; r < kRays; ++r) {
            wo[r] = mk3(0.f, 0.f, 0.f);
            wd[r] = mk3(1.f, 1.f, 1.f);
            root[r] = kInvalid;
            if (todo[r]) {
                float tm = kFltMax;
                root[r] = fetch(base + lane + 32u * r, wo[r], wd[r], tm);
            }
        }
        uint32_t first_root = root[0];
        f3 first_o = wo[0], first_d = wd[0];
        if (kRays > 1 && !todo[0]) {
            first_root = root[kRays - 1];
            first_o = wo[kRays - 1];
            first_d = wd[kRays - 1];
        }
        const uint32_t lroot = __shfl_sync(kAll, first_root, leader);
        const f3 o0 = mk3(__shfl_sync(kAll, first_o.x, leader), __shfl_sync(kAll, first_o.y, leader),
                          __shfl_sync(kAll, first_o.z, leader));
        const f3 d0 = mk3(__shfl_sync(kAll, first_d.x, leader), __shfl_sync(kAll, first_d.y, leader),
                          __shfl_sync(kAll, first_d.z, leader));
        LevelRay ray[kRays];
        TraceResult best[kRays];
        float tmax_box[kRays];
#pragma unroll
        for (int r = 0; r < kRays; ++r) {
            valid[r] = todo[r] && root[r] == lroot;
            todo[r] = todo[r] && !valid[r];
            if (!valid[r]) {
                wo[r] = o0;
                wd[r] = d0;
            }
            setup_level(ray[r], wo[r], wd[r]);
            best[r] = TraceResult{kFltMax, 0.f, 0.f, kInvalid, kInvalid};
            tmax_box[r] = kFltMax;
#if SPK_PACKET_WORLD_SMEM
            world[2 * r][threadIdx.x] = make_float4(wo[r].x, wo[r].y, wo[r].z, 0.f);
            world[2 * r + 1][threadIdx.x] = make_float4(wd[r].x, wd[r].y, wd[r].z, 0.f);
#endif
        }
        const uint32_t top_order = __shfl_sync(kAll, ray[0].oct, leader);  // the leader's ray: o0, d0
        uint32_t order = top_order;
        PacketFrustum frustum;
        bool packed = make_frustum(ray, order, frustum);  // the level's nodes are tested once for the packet
        uint2 ngroup = make_uint2(lroot, lroot == kInvalid ? 0u : (1u << 24)), tgroup = make_uint2(0u, 0u);
        uint32_t nown = 1u << 24, town = 0u;
        int sp = 0, blas_sp = 0;
        bool in_blas = false;
        uint32_t cur_inst = 0, iter = 0;
        auto push = [&](uint2 g, uint32_t mine) {
            if (sp < kPacketStack) {
                groups[sp] = g;
                own[sp] = mine;
                ++sp;
            } else {
                err |= kErrStackOverflow;
            }
        };
        auto lane_tmax = [&]() {
            float t = tmax_box[0];
#pragma unroll
            for (int r = 1; r < kRays; ++r) t = fmaxf(t, tmax_box[r]);
            return t;
        };
        for (;;) {
            if (++iter > budget) {
                err |= kErrIterationBudget;
                break;
            }
            if (ngroup.y > 0x00FFFFFFu && packed && SPK_PACKET_FRUSTUM) {
                // The nearest inner children of the group (up to kPacketSiblings, while the stack has room for
                // their groups), one per 8-lane group, each tested once for the packet against the largest
                // tmax of the rays of the lanes that reached any of them (tmax_box is never negative). A lane
                // takes every child that passes in the nodes it reached.
                const uint32_t imask = ngroup.y & 0xFFu, inner = ngroup.y >> 24;
                const uint32_t room = sp + 2 * kPacketSiblings <= kPacketStack ? kPacketSiblings : 1u;
                const uint32_t cnt = min(static_cast<uint32_t>(__popc(inner)), room);
                const uint32_t grp = (threadIdx.x >> 3) & 3u;
                uint32_t rest = inner, from = inner;
                for (uint32_t k = 0; k < cnt; ++k) {
                    if (k == grp) from = rest;
                    rest &= rest - 1u;
                }
                const uint32_t slot = (__ffs(from) - 1) ^ order;  // groups past `cnt` repeat the first child
                const uint32_t node_idx = ngroup.x + __popc(imask & ((1u << slot) - 1u));
                const uint32_t taken = inner & ~rest;
                const uint32_t mine_taken = (nown >> 24) & taken;
                ngroup.y = (rest << 24) | imask;
                nown &= ~(taken << 24);
                if (rest) push(ngroup, nown);
                if (kCount && lane == 0) counts->nodes += cnt;
                const float tmax =
                    __uint_as_float(__reduce_max_sync(kAll, mine_taken ? __float_as_uint(lane_tmax()) : 0u));
                uint2 ng, tg;
                visit_node_frustum(S.nodes, node_idx, frustum, order, tmax, ng, tg);
                // Hand each child's groups out, farthest first onto the stack so the nearest comes back first.
                uint32_t left = taken;
                for (int g = static_cast<int>(cnt) - 1; g >= 0; --g) {
                    const uint32_t b = 31 - __clz(left);
                    left &= ~(1u << b);
                    const bool mine = (mine_taken >> b) & 1u;
                    const uint2 n_g = make_uint2(__shfl_sync(kAll, ng.x, 8 * g), __shfl_sync(kAll, ng.y, 8 * g));
                    const uint2 t_g = make_uint2(__shfl_sync(kAll, tg.x, 8 * g), __shfl_sync(kAll, tg.y, 8 * g));
                    if (g == 0) {
                        ngroup = n_g;
                        tgroup = t_g;
                        nown = mine ? (n_g.y & 0xFF000000u) : 0u;
                        town = mine ? t_g.y : 0u;
                    } else {
                        if (n_g.y > 0x00FFFFFFu) push(n_g, mine ? (n_g.y & 0xFF000000u) : 0u);
                        if (t_g.y != 0u) push(t_g, mine ? t_g.y : 0u);
                    }
                }
            } else if (ngroup.y > 0x00FFFFFFu) {
                const uint32_t bit = __ffs(ngroup.y >> 24) - 1;
                const uint32_t keep = ~(1u << (bit + 24));
                const bool mine = (nown >> (bit + 24)) & 1u;
                ngroup.y &= keep;
                nown &= keep;
                const uint32_t slot = bit ^ order;
                const uint32_t node_idx = ngroup.x + __popc(ngroup.y & 0xFFu & ((1u << slot) - 1u));
                if (ngroup.y > 0x00FFFFFFu) push(ngroup, nown);
                if (kCount && lane == 0) ++counts->nodes;
                // Rays of several octants: every lane tests the node with its own rays; a lane that did not
                // reach it tests against t <= -1 (no hits).
                uint32_t hits = 0u;
#pragma unroll
                for (int r = 0; r < kRays; ++r) {
                    uint2 ng, tg;
                    visit_node(S.nodes, node_idx, ray[r], order, mine ? tmax_box[r] : -1.f, ng, tg);
                    hits |= (ng.y & 0xFF000000u) | tg.y;
                    ngroup.x = ng.x;
                    tgroup.x = tg.x;
                    ngroup.y = (ngroup.y & ~0xFFu) | (ng.y & 0xFFu);  // the child's imask
                }
                nown = hits & 0xFF000000u;
                town = hits & 0x00FFFFFFu;
                const uint32_t any = __reduce_or_sync(kAll, hits);
                ngroup.y = (any & 0xFF000000u) | (ngroup.y & 0xFFu);
                tgroup.y = any & 0x00FFFFFFu;
            } else {
                tgroup = ngroup;
                town = nown;
                ngroup = make_uint2(0u, 0u);
                nown = 0u;
            }
            while (tgroup.y != 0u) {
                const uint32_t k = __ffs(tgroup.y) - 1;
                tgroup.y &= tgroup.y - 1u;
                const bool mine = (town >> k) & 1u;
                const uint32_t idx = tgroup.x + k;
                if (in_blas) {
                    if (kCount && lane == 0) ++counts->tris;
                    if (!mine) continue;
#pragma unroll
                    for (int r = 0; r < kRays; ++r) {
                        float t, u, v;
                        uint32_t face;
                        if (!triangle_hit(S.tris, idx, ray[r], t, u, v, face)) continue;
#if SPK_PACKET_WORLD_SMEM
                        const f3 ro = world_o(r), rd = world_d(r);
#else
                        const f3 ro = wo[r], rd = wd[r];
#endif
                        const float wt = world_t(S.instances[cur_inst], ray[r], t, ro, rd);
                        if (wt > 0.f && closer_hit(best[r], wt, cur_inst, face)) {
                            best[r] = TraceResult{wt, u, v, cur_inst, face};
                            tmax_box[r] = prune_limit(wt, ro, rd, S.scene_abs_x);
                        }
                    }
                } else {
                    const uint32_t inst = __ldg(S.tlas_items + idx);
                    const DevInstance &I = S.instances[inst];
                    if (I.type == 1u) {
                        if (!mine) continue;
#pragma unroll
                        for (int r = 0; r < kRays; ++r) {
                            float t;
                            // (at the TLAS level the level ray is the world ray)
                            if (sphere_hit(I, ray[r].o, ray[r].d, t) && t > 0.f &&
                                closer_hit(best[r], t, inst, kInvalid)) {
                                best[r] = TraceResult{t, 0.f, 0.f, inst, kInvalid};
                                tmax_box[r] = prune_limit(t, ray[r].o, ray[r].d, S.scene_abs_x);
                            }
                        }
                    } else if (I.blas_root != kInvalid) {
                        // Enter the BLAS with every lane (those that did not reach it take no part); the
                        // rest of this TLAS level waits on the stack.
                        if (tgroup.y != 0u) push(tgroup, town);
                        if (ngroup.y > 0x00FFFFFFu) push(ngroup, nown);
                        blas_sp = sp;
                        in_blas = true;
                        cur_inst = inst;
#pragma unroll
                        for (int r = 0; r < kRays; ++r)
                            setup_level(ray[r], xform_point(I.minv, ray[r].o), xform_dir(I.minv, ray[r].d));
                        const uint32_t entering = __ballot_sync(kAll, mine);  // not empty: the group had bit k
                        order = __shfl_sync(kAll, ray[0].oct, __ffs(entering) - 1);
                        packed = make_frustum(ray, order, frustum);
                        ngroup = make_uint2(I.blas_root, 1u << 24);
                        nown = mine ? (1u << 24) : 0u;
                        tgroup.y = 0u;
                        break;
                    }
                }
            }
            if (ngroup.y <= 0x00FFFFFFu) {
                if (in_blas && sp == blas_sp) {
                    in_blas = false;
#pragma unroll
                    for (int r = 0; r < kRays; ++r) {
#if SPK_PACKET_WORLD_SMEM
                        setup_level(ray[r], world_o(r), world_d(r));
#else
                        setup_level(ray[r], wo[r], wd[r]);
#endif
                    }
                    order = top_order;
                    if (sp != 0) packed = make_frustum(ray, order, frustum);
                }
                if (sp == 0) break;
                --sp;
                ngroup = groups[sp];
                nown = own[sp];
            }
        }
#pragma unroll
        for (int r = 0; r < kRays; ++r)
            if (valid[r]) finish(base + lane + 32u * r, best[r]);
    }
}

}  // namespace spk
