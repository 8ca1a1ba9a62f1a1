// bvh_device.cu -- BLAS refit and device BLAS build (bvh_device.cuh).
#include "bvh_device.cuh"
#include "fault.h"

#include <algorithm>
#include <cfloat>
#include <cstring>

namespace spk {
namespace {

// The 80-byte wide node (bvh_builder.h): p[3] f32 @0, biased exponents @12, imask @15, child_base @16,
// item_base @20, meta[8] @24, qlo x/y/z @32/40/48, qhi x/y/z @56/64/72.
union NodeBytes {
    uint4 q[5];
    uint8_t b[80];
    float f[20];
    uint32_t u[20];
};

__device__ __forceinline__ void face_box(const BlasRefit &r, uint32_t record, float lo[3], float hi[3]) {
    const uint32_t face = __float_as_uint(r.tris[3ull * record + 2].y);
    if (face >= r.num_faces) return;
    const uint4 f = r.faces[face];
    const uint32_t idx[3] = {f.x, f.y, f.z};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (idx[c] >= r.num_vertices) continue;
        const float *p = r.positions + 3ull * idx[c];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            lo[a] = fminf(lo[a], p[a]);
            hi[a] = fmaxf(hi[a], p[a]);
        }
    }
}

__global__ void k_refit_triangles(BlasRefit r) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= r.tri_count) return;
    float4 *t = r.tris + 3ull * (r.tri_first + i);
    const float4 t2 = t[2];
    const uint32_t face = __float_as_uint(t2.y);
    if (face >= r.num_faces) return;
    const uint4 f = r.faces[face];
    if (f.x >= r.num_vertices || f.y >= r.num_vertices || f.z >= r.num_vertices) return;
    const float *p0 = r.positions + 3ull * f.x;
    const float *p1 = r.positions + 3ull * f.y;
    const float *p2 = r.positions + 3ull * f.z;
    const float e1[3] = {__fsub_rn(p1[0], p0[0]), __fsub_rn(p1[1], p0[1]), __fsub_rn(p1[2], p0[2])};
    const float e2[3] = {__fsub_rn(p2[0], p0[0]), __fsub_rn(p2[1], p0[1]), __fsub_rn(p2[2], p0[2])};
    t[0] = make_float4(p0[0], p0[1], p0[2], e1[0]);
    t[1] = make_float4(e1[1], e1[2], e2[0], e2[1]);
    t[2] = make_float4(e2[2], t2.y, t2.z, t2.w);
}

// Smallest e in [-126, 127] with 255 * 2^e >= ext (the host quantiser's exponent), -126 for ext <= 0.
__device__ int quant_exponent(double ext) {
    if (!(ext > 0.0)) return -126;
    int e = ilogb(ext) - 8;
    e = max(-126, min(127, e));
    while (e < 127 && ldexp(255.0, e) < ext) ++e;
    while (e > -126 && ldexp(255.0, e - 1) >= ext) --e;
    return e;
}

// Quantises as the host builder does (bvh_builder.cpp quantize_node): origin = the node box's low corner,
// the smallest power-of-two scale that spans the box in 255 steps, child boxes rounded outwards, flat
// children widened by a step. Slots with meta 0 are empty.
__device__ void quantize(NodeBytes &n, const float clo[8][3], const float chi[8][3], const float lo[3],
                         const float hi[3]) {
    for (int a = 0; a < 3; ++a) {
        const double origin = lo[a];
        const int e = quant_exponent(static_cast<double>(hi[a]) - origin);
        // Multiplying by 2^-e is exact, so it gives the host's (x - origin) / 2^e bit for bit.
        const double inv_scale = ldexp(1.0, -e);
        n.f[a] = lo[a];
        n.b[12 + a] = static_cast<uint8_t>(e + 127);
        for (int s = 0; s < 8; ++s) {
            if (n.b[24 + s] == 0) continue;
            double ql = floor((static_cast<double>(clo[s][a]) - origin) * inv_scale);
            double qh = ceil((static_cast<double>(chi[s][a]) - origin) * inv_scale);
            ql = fmax(0.0, fmin(255.0, ql));
            qh = fmax(0.0, fmin(255.0, qh));
            if (qh <= ql) {
                if (qh < 255.0) {
                    qh = ql + 1.0;
                } else {
                    ql = qh - 1.0;
                }
            }
            n.b[32 + 8 * a + s] = static_cast<uint8_t>(ql);
            n.b[56 + 8 * a + s] = static_cast<uint8_t>(qh);
        }
    }
}

__global__ void k_refit_nodes(BlasRefit r, uint32_t first, uint32_t last) {
    const uint32_t i = first + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= last) return;
    uint4 *np = r.nodes + 5ull * (r.root + i);
    NodeBytes n;
#pragma unroll
    for (int k = 0; k < 5; ++k) n.q[k] = np[k];
    const uint32_t imask = n.b[15];
    const uint32_t child_base = n.u[4], item_base = n.u[5];
    float clo[8][3], chi[8][3];
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int s = 0; s < 8; ++s) {
        const uint32_t meta = n.b[24 + s];
        float bl[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, bh[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        if (meta != 0) {
            if ((meta & 0x1Fu) >= 24u) {
                const uint32_t c = child_base + __popc(imask & ((1u << s) - 1u)) - r.root;
                if (c < r.node_count) {
                    const float *cb = r.boxes + 6ull * c;
                    for (int a = 0; a < 3; ++a) {
                        bl[a] = cb[a];
                        bh[a] = cb[3 + a];
                    }
                }
            } else {
                const uint32_t cnt = __popc(meta >> 5), off = meta & 0x1Fu;
                for (uint32_t j = 0; j < cnt; ++j) {
                    const uint32_t rec = item_base + off + j;
                    if (rec - r.tri_first < r.tri_count) face_box(r, rec, bl, bh);
                }
            }
            for (int a = 0; a < 3; ++a) {
                lo[a] = fminf(lo[a], bl[a]);
                hi[a] = fmaxf(hi[a], bh[a]);
            }
        }
        for (int a = 0; a < 3; ++a) {
            clo[s][a] = bl[a];
            chi[s][a] = bh[a];
        }
    }
    float *mb = r.boxes + 6ull * i;
    for (int a = 0; a < 3; ++a) {
        mb[a] = lo[a];
        mb[3 + a] = hi[a];
    }
    quantize(n, clo, chi, lo, hi);
#pragma unroll
    for (int k = 0; k < 5; ++k) np[k] = n.q[k];
}

__global__ void k_update_vertices(float4 *verts, uint32_t num_vertices, const float *normals, const float *tangents) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= num_vertices) return;
    float4 *r = verts + 3ull * v;
    float4 a = r[0], b = r[1];
    if (normals) {
        a.x = normals[3ull * v];
        a.y = normals[3ull * v + 1];
        a.z = normals[3ull * v + 2];
    }
    if (tangents) {
        a.w = tangents[4ull * v];
        b.x = tangents[4ull * v + 1];
        b.y = tangents[4ull * v + 2];
        b.z = tangents[4ull * v + 3];
    }
    r[0] = a;
    r[1] = b;
}


// ---------------------------------------------------------------------------------------------------------
// Device BLAS build.

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr int kSortThreads = 256;
constexpr int kSortRounds = 8;  // keys per thread per tile
constexpr uint32_t kTile = kSortThreads * kSortRounds;
constexpr int kScanThreads = 1024;

// Order-preserving map of floats to unsigned integers (for atomicMin / atomicMax of bounds).
__device__ __forceinline__ uint32_t float_key(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_float(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

// Per face: its box and centroid; the centroid bounds reduced into cb[0..5] (min xyz, max xyz as float keys).
__global__ void k_face_boxes(const float *pos, const uint32_t *idx, uint32_t n, float4 *flo, float4 *fhi,
                             uint32_t *cb) {
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    float c[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, d[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    if (f < n) {
        float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (int v = 0; v < 3; ++v) {
            const float *p = pos + 3ull * idx[3ull * f + v];
            for (int a = 0; a < 3; ++a) {
                lo[a] = fminf(lo[a], p[a]);
                hi[a] = fmaxf(hi[a], p[a]);
            }
        }
        flo[f] = make_float4(lo[0], lo[1], lo[2], 0.f);
        fhi[f] = make_float4(hi[0], hi[1], hi[2], 0.f);
        for (int a = 0; a < 3; ++a) c[a] = d[a] = __fmul_rn(0.5f, __fadd_rn(lo[a], hi[a]));
    }
    for (int off = 16; off > 0; off >>= 1)
        for (int a = 0; a < 3; ++a) {
            c[a] = fminf(c[a], __shfl_xor_sync(0xFFFFFFFFu, c[a], off));
            d[a] = fmaxf(d[a], __shfl_xor_sync(0xFFFFFFFFu, d[a], off));
        }
    if ((threadIdx.x & 31) == 0)
        for (int a = 0; a < 3; ++a) {
            atomicMin(cb + a, float_key(c[a]));
            atomicMax(cb + 3 + a, float_key(d[a]));
        }
}

__device__ __forceinline__ uint64_t spread21(uint32_t v) {  // bit i of v -> bit 3i
    uint64_t x = v & 0x1FFFFFu;
    x = (x | x << 32) & 0x1F00000000FFFFull;
    x = (x | x << 16) & 0x1F0000FF0000FFull;
    x = (x | x << 8) & 0x100F00F00F00F00Full;
    x = (x | x << 4) & 0x10C30C30C30C30C3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}

__global__ void k_morton(const float4 *flo, const float4 *fhi, uint32_t n, const uint32_t *cb, uint64_t *keys,
                         uint32_t *vals) {
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n) return;
    const float4 lo = flo[f], hi = fhi[f];
    const float c[3] = {__fmul_rn(0.5f, __fadd_rn(lo.x, hi.x)), __fmul_rn(0.5f, __fadd_rn(lo.y, hi.y)),
                        __fmul_rn(0.5f, __fadd_rn(lo.z, hi.z))};
    uint32_t q[3];
    for (int a = 0; a < 3; ++a) {
        const float b0 = key_float(cb[a]), b1 = key_float(cb[3 + a]);
        const float ext = b1 - b0;
        const float t = ext > 0.f ? (c[a] - b0) / ext : 0.f;
        q[a] = static_cast<uint32_t>(fminf(fmaxf(t * 2097152.f, 0.f), 2097151.f));
    }
    keys[f] = (spread21(q[0]) << 2) | (spread21(q[1]) << 1) | spread21(q[2]);
    vals[f] = f;
}

// Stable LSD radix sort, 8 bits per pass: per-tile digit counts, one exclusive scan over (digit, tile),
// then each tile scatters its keys in order (ranks from warp match masks and per-warp digit counts).
__global__ void k_radix_count(const uint64_t *keys, uint32_t n, int shift, uint32_t num_tiles, uint32_t *hist) {
    __shared__ uint32_t cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kTile;
    for (int r = 0; r < kSortRounds; ++r) {
        const uint64_t i = base + static_cast<uint64_t>(r) * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[static_cast<uint64_t>(threadIdx.x) * num_tiles + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void k_radix_scatter(const uint64_t *keys, const uint32_t *vals, uint32_t n, int shift,
                                uint32_t num_tiles, const uint32_t *offsets, uint64_t *keys_out,
                                uint32_t *vals_out) {
    __shared__ uint32_t running[256];
    __shared__ uint32_t warp_cnt[kSortThreads / 32][256];
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    running[tid] = offsets[static_cast<uint64_t>(tid) * num_tiles + blockIdx.x];
    for (int w = 0; w < kSortThreads / 32; ++w) warp_cnt[w][tid] = 0;
    __syncthreads();
    const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kTile;
    for (int r = 0; r < kSortRounds; ++r) {
        const uint64_t i = base + static_cast<uint64_t>(r) * kSortThreads + tid;
        const bool valid = i < n;
        const uint64_t key = valid ? keys[i] : 0;
        const uint32_t val = valid ? vals[i] : 0;
        const uint32_t digit = valid ? static_cast<uint32_t>((key >> shift) & 255u) : 256u + lane;  // unique if invalid
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, digit);
        const uint32_t rank_in_warp = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank_in_warp == 0) warp_cnt[warp][digit] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t before = 0;
            for (uint32_t w = 0; w < warp; ++w) before += warp_cnt[w][digit];
            const uint32_t dst = running[digit] + before + rank_in_warp;
            keys_out[dst] = key;
            vals_out[dst] = val;
        }
        __syncthreads();
        uint32_t total = 0;
        for (int w = 0; w < kSortThreads / 32; ++w) {
            total += warp_cnt[w][tid];
            warp_cnt[w][tid] = 0;
        }
        running[tid] += total;
        __syncthreads();
    }
}

// Block-level pass of the exclusive scan: block b scans data[b*kScanChunk ..) in place (coalesced, four
// values per thread) and writes its total to sums[b].
constexpr uint32_t kScanChunk = 4u * kScanThreads;

__global__ void k_scan_blocks(uint32_t *data, uint32_t n, uint32_t *sums) {
    __shared__ uint32_t warp_tot[kScanThreads / 32];
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kScanChunk + 4ull * tid;
    uint32_t v[4], run = 0;
    for (int k = 0; k < 4; ++k) {
        v[k] = base + k < n ? data[base + k] : 0u;
        run += v[k];
    }
    uint32_t incl = run;  // inclusive scan of the thread sums within the warp
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t o = __shfl_up_sync(0xFFFFFFFFu, incl, off);
        if (lane >= static_cast<uint32_t>(off)) incl += o;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = lane < kScanThreads / 32 ? warp_tot[lane] : 0u, x = t;
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t o = __shfl_up_sync(0xFFFFFFFFu, x, off);
            if (lane >= static_cast<uint32_t>(off)) x += o;
        }
        if (lane < kScanThreads / 32) warp_tot[lane] = x - t;  // exclusive warp offsets
        if (lane == kScanThreads / 32 - 1) sums[blockIdx.x] = x;
    }
    __syncthreads();
    uint32_t acc = warp_tot[warp] + incl - run;
    for (int k = 0; k < 4; ++k) {
        if (base + k < n) data[base + k] = acc;
        acc += v[k];
    }
}

__global__ void k_scan_add(uint32_t *data, uint32_t n, const uint32_t *offsets) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * kScanChunk + threadIdx.x;
    const uint32_t o = offsets[blockIdx.x];
    for (int k = 0; k < 4; ++k)
        if (i + k * kScanThreads < n) data[i + k * kScanThreads] += o;
}

// In-place exclusive scan of data[0..n) by one block; *total receives the sum.
__global__ void k_scan(uint32_t *data, uint32_t n, uint32_t *total) {
    __shared__ uint32_t part[kScanThreads];
    const uint32_t tid = threadIdx.x;
    const uint32_t chunk = (n + kScanThreads - 1) / kScanThreads;
    const uint64_t b = static_cast<uint64_t>(tid) * chunk;
    const uint64_t e = min(static_cast<uint64_t>(n), b + chunk);
    uint32_t sum = 0;
    for (uint64_t i = b; i < e; ++i) sum += data[i];
    part[tid] = sum;
    __syncthreads();
    for (uint32_t off = 1; off < kScanThreads; off <<= 1) {
        const uint32_t v = tid >= off ? part[tid - off] : 0u;
        __syncthreads();
        part[tid] += v;
        __syncthreads();
    }
    uint32_t run = part[tid] - sum;
    for (uint64_t i = b; i < e; ++i) {
        const uint32_t v = data[i];
        data[i] = run;
        run += v;
    }
    if (tid == kScanThreads - 1 && total) *total = part[tid];
}

// Karras 2012 binary radix tree over the sorted codes (ties broken by position). Internal node i in
// [0, n-1), leaf m is node n-1+m; node 0 is the root. Writes children, parent links and each internal
// node's leaf range.
__device__ __forceinline__ int common_prefix(const uint64_t *k, int64_t n, int64_t i, int64_t j) {
    if (j < 0 || j >= n) return -1;
    const uint64_t a = k[i], b = k[j];
    return a != b ? __clzll(a ^ b) : 64 + __clzll(static_cast<uint64_t>(i ^ j));
}

__global__ void k_karras(const uint64_t *keys, uint32_t n, uint32_t *left, uint32_t *right, uint32_t *parent,
                         uint32_t *first, uint32_t *count) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    const int64_t N = n;
    if (i >= N - 1) return;
    const int d = common_prefix(keys, N, i, i + 1) - common_prefix(keys, N, i, i - 1) >= 0 ? 1 : -1;
    const int dmin = common_prefix(keys, N, i, i - d);
    int64_t lmax = 2;
    while (common_prefix(keys, N, i, i + lmax * d) > dmin) lmax *= 2;
    int64_t l = 0;
    for (int64_t t = lmax / 2; t >= 1; t /= 2)
        if (common_prefix(keys, N, i, i + (l + t) * d) > dmin) l += t;
    const int64_t j = i + l * d;
    const int dnode = common_prefix(keys, N, i, j);
    int64_t s = 0;
    for (int64_t t = (l + 1) / 2;; t = (t + 1) / 2) {
        if (common_prefix(keys, N, i, i + (s + t) * d) > dnode) s += t;
        if (t == 1) break;
    }
    const int64_t gamma = i + s * d + min(d, 0);
    const int64_t lo = min(i, j), hi = max(i, j);
    const uint32_t lc = static_cast<uint32_t>(lo == gamma ? (N - 1) + gamma : gamma);
    const uint32_t rc = static_cast<uint32_t>(hi == gamma + 1 ? (N - 1) + gamma + 1 : gamma + 1);
    left[i] = lc;
    right[i] = rc;
    parent[lc] = static_cast<uint32_t>(i);
    parent[rc] = static_cast<uint32_t>(i);
    first[i] = static_cast<uint32_t>(lo);
    count[i] = static_cast<uint32_t>(hi - lo + 1);
}

// Bottom-up SAH cost of a binary node (traversal cost 1 : triangle cost 1, as the host build): a subtree of
// at most max_leaf triangles may stay one leaf when that is not dearer than keeping it split. The cost goes
// to the low corner's w, the "one leaf" decision (1 / 0) to the high corner's w; the collapse reads it.
__device__ __forceinline__ void node_cost(float4 &lo, float4 &hi, float cost_a, float cost_b, uint32_t count,
                                          uint32_t max_leaf) {
    const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    const float area = dx * dy + dy * dz + dz * dx;
    const float inner = area + cost_a + cost_b;
    const float leaf = count <= max_leaf ? area * static_cast<float>(count) : FLT_MAX;
    lo.w = fminf(inner, leaf);
    hi.w = leaf <= inner ? 1.f : 0.f;
}

__device__ __forceinline__ void leaf_cost(float4 &lo, float4 &hi) {
    const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    lo.w = dx * dy + dy * dz + dz * dx;
    hi.w = 1.f;
}

// Leaf boxes, then up the tree: the second child to arrive at a node writes its box and goes on.
__global__ void k_bottom_up(const uint32_t *sorted_faces, const float4 *flo, const float4 *fhi, uint32_t n,
                            const uint32_t *left, const uint32_t *right, const uint32_t *parent, const uint32_t *count,
                            uint32_t max_leaf, uint32_t *arrivals, float4 *nlo, float4 *nhi) {
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    uint32_t node = n - 1 + m;
    float4 lo = flo[sorted_faces[m]], hi = fhi[sorted_faces[m]];
    leaf_cost(lo, hi);
    nlo[node] = lo;
    nhi[node] = hi;
    for (uint32_t steps = 0; steps < n; ++steps) {
        const uint32_t p = parent[node];
        if (p == kNone) break;
        __threadfence();
        if (atomicAdd(&arrivals[p], 1u) == 0) break;
        const uint32_t other = left[p] == node ? right[p] : left[p];
        const float4 ol = __ldcg(nlo + other), oh = __ldcg(nhi + other);
        const float ca = lo.w, cb = ol.w;
        lo = make_float4(fminf(lo.x, ol.x), fminf(lo.y, ol.y), fminf(lo.z, ol.z), 0.f);
        hi = make_float4(fmaxf(hi.x, oh.x), fmaxf(hi.y, oh.y), fmaxf(hi.z, oh.z), 0.f);
        node_cost(lo, hi, ca, cb, count[p], max_leaf);
        nlo[p] = lo;
        nhi[p] = hi;
        node = p;
    }
}

// PLOC (Meister and Bittner, "Parallel Locally-Ordered Clustering for Bounding Volume Hierarchy
// Construction", 2018): starting from the leaves in Morton order, every cluster finds the neighbour within
// kPlocRadius positions whose merged box has the smallest area; mutual nearest neighbours merge into a new
// node (ids handed out downwards from n - 2, so the last merge is the root, node 0), and the survivors are
// compacted in order. Ties go to the lower position, merge ids come from a scan: deterministic.
constexpr int kPlocRadius = 16;
constexpr int kPlocThreads = 256;

__global__ void k_leaf_init(const uint32_t *sorted_faces, const float4 *flo, const float4 *fhi, uint32_t n,
                            float4 *nlo, float4 *nhi, uint32_t *clusters) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t node = n - 1 + i;
    float4 lo = flo[sorted_faces[i]], hi = fhi[sorted_faces[i]];
    leaf_cost(lo, hi);
    nlo[node] = lo;
    nhi[node] = hi;
    clusters[i] = node;
}

__device__ __forceinline__ float merged_half_area(float4 al, float4 ah, float4 bl, float4 bh) {
    const float dx = fmaxf(ah.x, bh.x) - fminf(al.x, bl.x);
    const float dy = fmaxf(ah.y, bh.y) - fminf(al.y, bl.y);
    const float dz = fmaxf(ah.z, bh.z) - fminf(al.z, bl.z);
    return dx * dy + dy * dz + dz * dx;
}

__global__ void k_ploc_nn(const uint32_t *clusters, uint32_t m, const float4 *nlo, const float4 *nhi, uint32_t *nn) {
    __shared__ float4 slo[kPlocThreads + 2 * kPlocRadius], shi[kPlocThreads + 2 * kPlocRadius];
    const int64_t base = static_cast<int64_t>(blockIdx.x) * kPlocThreads - kPlocRadius;
    for (int k = threadIdx.x; k < kPlocThreads + 2 * kPlocRadius; k += blockDim.x) {
        const int64_t i = base + k;
        if (i >= 0 && i < m) {
            const uint32_t c = clusters[i];
            slo[k] = nlo[c];
            shi[k] = nhi[c];
        }
    }
    __syncthreads();
    const int64_t i = static_cast<int64_t>(blockIdx.x) * kPlocThreads + threadIdx.x;
    if (i >= m) return;
    const int li = static_cast<int>(threadIdx.x) + kPlocRadius;
    float best = FLT_MAX;
    int64_t bj = i;
    for (int d = -kPlocRadius; d <= kPlocRadius; ++d) {
        const int64_t j = i + d;
        if (d == 0 || j < 0 || j >= m) continue;
        const float a = merged_half_area(slo[li], shi[li], slo[li + d], shi[li + d]);
        if (a < best) {  // ascending j: the first of equal areas is kept
            best = a;
            bj = j;
        }
    }
    nn[i] = static_cast<uint32_t>(bj);
}

// keep[i]: cluster i survives this round (merged into a new node or unchanged); merge[i]: it is the lower
// position of a mutual pair and makes the new node.
__global__ void k_ploc_flags(const uint32_t *nn, uint32_t m, uint32_t *keep, uint32_t *merge) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const uint32_t j = nn[i];
    const bool mutual = j != i && j < m && nn[j] == i;
    merge[i] = mutual && i < j ? 1u : 0u;
    keep[i] = mutual && i > j ? 0u : 1u;
}

__global__ void k_ploc_write(const uint32_t *clusters, uint32_t m, const uint32_t *nn, const uint32_t *merge_off,
                             const uint32_t *pos, uint32_t id_base, uint32_t n, uint32_t max_leaf, float4 *nlo, float4 *nhi,
                             uint32_t *left, uint32_t *right, uint32_t *count, uint32_t *out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const uint32_t j = nn[i];
    const bool mutual = j != i && j < m && nn[j] == i;
    if (mutual && i > j) return;  // merged into the node made at position j
    uint32_t c = clusters[i];
    if (mutual) {
        const uint32_t id = id_base - merge_off[i];
        const uint32_t a = c, b = clusters[j];
        if (id < n - 1) {
            left[id] = a;
            right[id] = b;
            const uint32_t cnt = (a >= n - 1 ? 1u : count[a]) + (b >= n - 1 ? 1u : count[b]);
            count[id] = cnt;
            const float4 al = nlo[a], ah = nhi[a], bl = nlo[b], bh = nhi[b];
            float4 lo = make_float4(fminf(al.x, bl.x), fminf(al.y, bl.y), fminf(al.z, bl.z), 0.f);
            float4 hi = make_float4(fmaxf(ah.x, bh.x), fmaxf(ah.y, bh.y), fmaxf(ah.z, bh.z), 0.f);
            node_cost(lo, hi, al.w, bl.w, cnt, max_leaf);
            nlo[id] = lo;
            nhi[id] = hi;
        }
        c = id;
    }
    out[pos[i]] = c;
}

struct BinaryTree {
    const uint32_t *left, *right, *first, *count;
    const float4 *nlo, *nhi;
    uint32_t n;  // leaves
    __device__ uint32_t leaves(uint32_t x) const { return x >= n - 1 ? 1u : count[x]; }
    // One wide-BVH leaf: a triangle, or a subtree the bottom-up SAH costs chose to keep whole.
    __device__ bool is_leaf(uint32_t x) const { return x >= n - 1 || nhi[x].w != 0.f; }
    __device__ float half_area(uint32_t x) const {
        const float4 a = nlo[x], b = nhi[x];
        const float dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
        return dx * dy + dy * dz + dz * dx;
    }
};

// One breadth-first level of the collapse, pass 1: open each job's binary subtree into at most
// `max_children` kids (always the inner kid of largest area; kids of <= max_leaf leaves stay closed) and
// count the inner kids and leaf items.
__global__ void k_collapse_open(BinaryTree t, const uint32_t *jobs, uint32_t num_jobs, int max_children, int max_leaf,
                                uint32_t *kids, uint32_t *inner_count, uint32_t *item_count) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= num_jobs) return;
    const uint32_t b = jobs[j];
    uint32_t k[8];
    int nk = 0;
    if (b >= 2 * t.n - 1) {  // not a node: emit an empty job (the host then reports the item count mismatch)
        for (int q = 0; q < 8; ++q) kids[8ull * j + q] = kNone;
        inner_count[j] = item_count[j] = 0;
        return;
    }
    if (t.is_leaf(b)) {
        k[nk++] = b;
    } else {
        k[nk++] = t.left[b];
        k[nk++] = t.right[b];
        while (nk < max_children) {
            int best = -1;
            float best_area = -1.f;
            for (int q = 0; q < nk; ++q) {
                if (!t.is_leaf(k[q])) {
                    const float a = t.half_area(k[q]);
                    if (a > best_area) {
                        best_area = a;
                        best = q;
                    }
                }
            }
            if (best < 0) break;
            const uint32_t x = k[best];
            k[best] = t.left[x];
            k[nk++] = t.right[x];
        }
    }
    uint32_t inner = 0, items = 0;
    for (int q = 0; q < 8; ++q) {
        kids[8ull * j + q] = q < nk ? k[q] : kNone;
        if (q < nk) {
            if (!t.is_leaf(k[q]) && k[q] != b) {
                ++inner;
            } else {
                items += t.leaves(k[q]);
            }
        }
    }
    inner_count[j] = inner;
    item_count[j] = items;
}

// Pass 2: octant slot order, quantised boxes, children and items. Job j is node level_base + j; its inner
// kids become next-level jobs inner_off[j].. (nodes next_base + inner_off[j] ..) in slot order; its leaf
// items go to items[item_base + item_off[j] ..] in slot order.
__global__ void k_collapse_emit(BinaryTree t, uint32_t num_jobs, int max_leaf, const uint32_t *jobs, const uint32_t *kids,
                                const uint32_t *inner_off, const uint32_t *item_off, uint32_t level_base,
                                uint32_t next_base, uint32_t item_base, const uint32_t *sorted_faces, uint4 *nodes,
                                uint32_t *items, uint32_t *next_jobs) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= num_jobs) return;
    const uint32_t b = jobs[j];
    uint32_t k[8];
    int nk = 0;
    for (int q = 0; q < 8; ++q) {
        k[q] = kids[8ull * j + q];
        if (k[q] != kNone) nk = q + 1;
    }
    float clo[8][3], chi[8][3], blo[8][3], bhi[8][3];
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int q = 0; q < nk; ++q) {
        const float4 a = t.nlo[k[q]], c = t.nhi[k[q]];
        blo[q][0] = a.x, blo[q][1] = a.y, blo[q][2] = a.z;
        bhi[q][0] = c.x, bhi[q][1] = c.y, bhi[q][2] = c.z;
        for (int x = 0; x < 3; ++x) {
            lo[x] = fminf(lo[x], blo[q][x]);
            hi[x] = fmaxf(hi[x], bhi[q][x]);
        }
    }
    // Slot s is the near-most kid for rays whose direction sign bits equal s: pairs (kid, slot) taken in
    // ascending order of the kid centre's projection on the slot's diagonal, each kid and slot once.
    float pc[3];
    for (int x = 0; x < 3; ++x) pc[x] = __fmul_rn(0.5f, __fadd_rn(lo[x], hi[x]));
    float dk[8][3];
    for (int q = 0; q < nk; ++q)
        for (int x = 0; x < 3; ++x) dk[q][x] = __fsub_rn(__fmul_rn(0.5f, __fadd_rn(blo[q][x], bhi[q][x])), pc[x]);
    int slot_of[8], kid_in_slot[8];
    for (int q = 0; q < 8; ++q) slot_of[q] = kid_in_slot[q] = -1;
    for (int round = 0; round < nk; ++round) {
        float best = FLT_MAX;
        int bq = -1, bs = -1;
        for (int q = 0; q < nk; ++q) {
            if (slot_of[q] >= 0) continue;
            for (int s = 0; s < 8; ++s) {
                if (kid_in_slot[s] >= 0) continue;
                const float v = __fadd_rn(__fadd_rn(s & 1 ? -dk[q][0] : dk[q][0], s & 2 ? -dk[q][1] : dk[q][1]),
                                          s & 4 ? -dk[q][2] : dk[q][2]);
                if (bq < 0 || v < best) {  // first minimum in (kid, slot) order
                    best = v;
                    bq = q;
                    bs = s;
                }
            }
        }
        slot_of[bq] = bs;
        kid_in_slot[bs] = bq;
    }
    NodeBytes n;
    for (int w = 0; w < 20; ++w) n.u[w] = 0;
    const uint32_t child_base = next_base + inner_off[j];
    const uint32_t ibase = item_base + item_off[j];
    n.u[4] = child_base;
    n.u[5] = ibase;
    uint32_t inner = 0, offset = 0, imask = 0;
    for (int s = 0; s < 8; ++s) {
        const int q = kid_in_slot[s];
        if (q < 0) continue;
        for (int x = 0; x < 3; ++x) {
            clo[s][x] = blo[q][x];
            chi[s][x] = bhi[q][x];
        }
        const uint32_t kid = k[q];
        const uint32_t cnt = t.leaves(kid);
        if (!t.is_leaf(kid) && kid != b) {
            imask |= 1u << s;
            n.b[24 + s] = static_cast<uint8_t>(0x20u | (24u + s));
            if (inner_off[j] + inner < t.n) next_jobs[inner_off[j] + inner] = kid;
            ++inner;
        } else {
            n.b[24 + s] = static_cast<uint8_t>((((1u << cnt) - 1u) << 5) | offset);
            // The leaves of the kid's subtree (<= 3), left first: a Morton-ordered range for the radix tree,
            // any leaves for the clustered one.
            uint32_t st[4], sp = 0, o = 0;
            st[sp++] = kid;
            while (sp > 0 && o < cnt) {
                const uint32_t x = st[--sp];
                if (x >= t.n - 1) {
                    const uint32_t m = x - (t.n - 1);
                    if (ibase + offset + o < t.n && m < t.n) items[ibase + offset + o] = sorted_faces[m];
                    ++o;
                } else if (sp + 2 <= 4) {
                    st[sp++] = t.right[x];
                    st[sp++] = t.left[x];
                }
            }
            offset += cnt;
        }
    }
    n.b[15] = static_cast<uint8_t>(imask);
    quantize(n, clo, chi, lo, hi);
    uint4 *dst = nodes + 5ull * (level_base + j);
    for (int w = 0; w < 5; ++w) dst[w] = n.q[w];
}
}  // namespace

cudaError_t launch_refit_triangles(const BlasRefit &r, cudaStream_t stream) {
    if (r.tri_count == 0) return cudaSuccess;
    k_refit_triangles<<<(r.tri_count + 255) / 256, 256, 0, stream>>>(r);
    return cudaGetLastError();
}

cudaError_t launch_refit_nodes(const BlasRefit &r, uint32_t first, uint32_t last, cudaStream_t stream) {
    if (last <= first || last > r.node_count) return last <= first ? cudaSuccess : cudaErrorInvalidValue;
    k_refit_nodes<<<(last - first + 127) / 128, 128, 0, stream>>>(r, first, last);
    return cudaGetLastError();
}

cudaError_t launch_update_vertices(float4 *verts, uint32_t vert_base, uint32_t num_vertices, const float *normals,
                                   const float *tangents, cudaStream_t stream) {
    if (num_vertices == 0 || (!normals && !tangents)) return cudaSuccess;
    k_update_vertices<<<(num_vertices + 255) / 256, 256, 0, stream>>>(verts + 3ull * vert_base, num_vertices, normals,
                                                                         tangents);
    return cudaGetLastError();
}

}  // namespace spk

namespace spk {
namespace {

// Device scratch freed on every exit path.
struct Scratch {
    std::vector<void *> ptrs;
    template <class T>
    cudaError_t get(T *&p, size_t count) {
        p = nullptr;
        void *q = nullptr;
        const cudaError_t e =
            fault_allocation() ? cudaErrorMemoryAllocation : cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
        if (e != cudaSuccess) return e;
        ptrs.push_back(q);
        p = static_cast<T *>(q);
        return cudaSuccess;
    }
    ~Scratch() {
        for (void *q : ptrs) cudaFree(q);
    }
};

#define SPK_TRY(x)                              \
    do {                                        \
        const cudaError_t e_ = (x);             \
        if (e_ != cudaSuccess) return e_;       \
    } while (0)

inline uint32_t blocks(uint64_t n, uint32_t threads) { return static_cast<uint32_t>((n + threads - 1) / threads); }

// Exclusive scan of data[0..n) in place; *total (device) receives the sum. One block for short arrays,
// else block scans, one scan of the block totals (scratch: blocks(n, kScanChunk) + 1 words) and an add.
void scan(uint32_t *data, uint32_t n, uint32_t *total, uint32_t *scratch, cudaStream_t stream) {
    if (n <= kScanChunk) {
        k_scan<<<1, kScanThreads, 0, stream>>>(data, n, total);
        return;
    }
    const uint32_t nb = blocks(n, kScanChunk);
    k_scan_blocks<<<nb, kScanThreads, 0, stream>>>(data, n, scratch);
    k_scan<<<1, kScanThreads, 0, stream>>>(scratch, nb, total);
    k_scan_add<<<nb, kScanThreads, 0, stream>>>(data, n, scratch);
}

}  // namespace

cudaError_t build_wide_device(const float *positions, uint32_t num_vertices, const uint32_t *indices,
                              uint32_t num_faces, int max_children, int max_leaf, bool clustered, cudaStream_t stream,
                              WideBvh &out, std::vector<uint32_t> &levels) {
    out = WideBvh{};
    levels.clear();
    if (num_faces == 0) return cudaSuccess;
    max_children = std::max(2, std::min(8, max_children));
    max_leaf = std::max(1, std::min(3, max_leaf));
    const uint32_t n = num_faces;
    const uint32_t tiles = blocks(n, kTile);
    Scratch sc;
    float *d_pos;
    uint32_t *d_idx, *cb, *hist, *vals[2], *left, *right, *parent, *first, *count, *arrivals, *jobs[2], *kids,
        *inner_cnt, *item_cnt, *totals, *items;
    uint64_t *keys[2];
    float4 *flo, *fhi, *nlo, *nhi;
    uint4 *nodes;
    SPK_TRY(sc.get(d_pos, 3ull * num_vertices));
    SPK_TRY(sc.get(d_idx, 3ull * n));
    SPK_TRY(sc.get(cb, 6));
    SPK_TRY(sc.get(flo, n));
    SPK_TRY(sc.get(fhi, n));
    SPK_TRY(sc.get(keys[0], n));
    SPK_TRY(sc.get(keys[1], n));
    SPK_TRY(sc.get(vals[0], n));
    SPK_TRY(sc.get(vals[1], n));
    SPK_TRY(sc.get(hist, 256ull * tiles));
    SPK_TRY(sc.get(left, n));
    SPK_TRY(sc.get(right, n));
    SPK_TRY(sc.get(first, n));
    SPK_TRY(sc.get(count, n));
    SPK_TRY(sc.get(parent, 2ull * n));
    SPK_TRY(sc.get(arrivals, n));
    SPK_TRY(sc.get(nlo, 2ull * n));
    SPK_TRY(sc.get(nhi, 2ull * n));
    SPK_TRY(sc.get(jobs[0], n));
    SPK_TRY(sc.get(jobs[1], n));
    SPK_TRY(sc.get(kids, 8ull * n));
    SPK_TRY(sc.get(inner_cnt, n));
    SPK_TRY(sc.get(item_cnt, n));
    uint32_t *scan_tmp;
    SPK_TRY(sc.get(totals, 2));
    SPK_TRY(sc.get(scan_tmp, blocks(256ull * tiles > n ? 256ull * tiles : n, kScanChunk) + 1));
    SPK_TRY(sc.get(items, n));
    SPK_TRY(sc.get(nodes, 5ull * n));

    SPK_TRY(cudaMemcpyAsync(d_pos, positions, 3ull * num_vertices * sizeof(float), cudaMemcpyHostToDevice, stream));
    SPK_TRY(cudaMemcpyAsync(d_idx, indices, 3ull * n * sizeof(uint32_t), cudaMemcpyHostToDevice, stream));
    const uint32_t cb_init[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u};
    SPK_TRY(cudaMemcpyAsync(cb, cb_init, sizeof(cb_init), cudaMemcpyHostToDevice, stream));
    k_face_boxes<<<blocks(n, 256), 256, 0, stream>>>(d_pos, d_idx, n, flo, fhi, cb);
    k_morton<<<blocks(n, 256), 256, 0, stream>>>(flo, fhi, n, cb, keys[0], vals[0]);
    int cur = 0;
    for (int shift = 0; shift < 64; shift += 8) {
        k_radix_count<<<tiles, kSortThreads, 0, stream>>>(keys[cur], n, shift, tiles, hist);
        scan(hist, 256u * tiles, nullptr, scan_tmp, stream);
        k_radix_scatter<<<tiles, kSortThreads, 0, stream>>>(keys[cur], vals[cur], n, shift, tiles, hist, keys[cur ^ 1],
                                                            vals[cur ^ 1]);
        cur ^= 1;
    }
    SPK_TRY(cudaGetLastError());
    const uint64_t *skeys = keys[cur];
    const uint32_t *sfaces = vals[cur];
    if (clustered) {
        // PLOC rounds until one cluster is left; clusters ping-pong between jobs[0] and jobs[1], the nearest
        // neighbours live in kids, the keep / merge flags (scanned in place) in item_cnt / inner_cnt.
        k_leaf_init<<<blocks(n, 256), 256, 0, stream>>>(sfaces, flo, fhi, n, nlo, nhi, jobs[0]);
        uint32_t m = n, merged = 0;
        int cc = 0;
        for (uint32_t round = 0; m > 1; ++round) {
            if (round > n) return cudaErrorUnknown;  // cannot happen: every round merges at least one pair
            k_ploc_nn<<<blocks(m, kPlocThreads), kPlocThreads, 0, stream>>>(jobs[cc], m, nlo, nhi, kids);
            k_ploc_flags<<<blocks(m, 256), 256, 0, stream>>>(kids, m, item_cnt, inner_cnt);
            scan(inner_cnt, m, totals, scan_tmp, stream);
            scan(item_cnt, m, totals + 1, scan_tmp, stream);
            k_ploc_write<<<blocks(m, 256), 256, 0, stream>>>(jobs[cc], m, kids, inner_cnt, item_cnt, n - 2 - merged, n,
                                                             static_cast<uint32_t>(max_leaf), nlo, nhi, left, right,
                                                             count, jobs[cc ^ 1]);
            SPK_TRY(cudaGetLastError());
            uint32_t tot[2];
            SPK_TRY(cudaMemcpyAsync(tot, totals, sizeof(tot), cudaMemcpyDeviceToHost, stream));
            SPK_TRY(cudaStreamSynchronize(stream));
            if (tot[0] == 0 || tot[1] != m - tot[0]) return cudaErrorUnknown;
            merged += tot[0];
            m = tot[1];
            cc ^= 1;
        }
    } else {
        SPK_TRY(cudaMemsetAsync(parent, 0xFF, 2ull * n * sizeof(uint32_t), stream));
        SPK_TRY(cudaMemsetAsync(arrivals, 0, n * sizeof(uint32_t), stream));
        if (n > 1) k_karras<<<blocks(n - 1, 256), 256, 0, stream>>>(skeys, n, left, right, parent, first, count);
        k_bottom_up<<<blocks(n, 256), 256, 0, stream>>>(sfaces, flo, fhi, n, left, right, parent, count,
                                                        static_cast<uint32_t>(max_leaf), arrivals, nlo, nhi);
    }
    SPK_TRY(cudaGetLastError());

    BinaryTree t{left, right, first, count, nlo, nhi, n};
    const uint32_t root = 0;  // internal node 0, or leaf 0 (= node 0) when n == 1
    SPK_TRY(cudaMemcpyAsync(jobs[0], &root, sizeof(root), cudaMemcpyHostToDevice, stream));
    uint32_t num_jobs = 1, level_base = 0, item_base = 0;
    int jc = 0;
    levels.push_back(0);
    while (num_jobs > 0) {
        if (static_cast<uint64_t>(level_base) + num_jobs > n) return cudaErrorUnknown;  // cannot happen: <= n nodes
        k_collapse_open<<<blocks(num_jobs, 128), 128, 0, stream>>>(t, jobs[jc], num_jobs, max_children, max_leaf, kids,
                                                                   inner_cnt, item_cnt);
        scan(inner_cnt, num_jobs, totals, scan_tmp, stream);
        scan(item_cnt, num_jobs, totals + 1, scan_tmp, stream);
        const uint32_t next_base = level_base + num_jobs;
        k_collapse_emit<<<blocks(num_jobs, 128), 128, 0, stream>>>(t, num_jobs, max_leaf, jobs[jc], kids, inner_cnt,
                                                                   item_cnt, level_base, next_base, item_base, sfaces,
                                                                   nodes, items, jobs[jc ^ 1]);
        SPK_TRY(cudaGetLastError());
        uint32_t tot[2];
        SPK_TRY(cudaMemcpyAsync(tot, totals, sizeof(tot), cudaMemcpyDeviceToHost, stream));
        SPK_TRY(cudaStreamSynchronize(stream));
        level_base = next_base;
        item_base += tot[1];
        num_jobs = tot[0];
        jc ^= 1;
        levels.push_back(level_base);
    }
    if (item_base != n) return cudaErrorUnknown;
    out.nodes.resize(level_base);
    out.items.resize(n);
    static_assert(sizeof(WideNode) == 5 * sizeof(uint4), "node size");
    SPK_TRY(cudaMemcpyAsync(out.nodes.data(), nodes, level_base * sizeof(WideNode), cudaMemcpyDeviceToHost, stream));
    SPK_TRY(cudaMemcpyAsync(out.items.data(), items, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
    return cudaStreamSynchronize(stream);
}

}  // namespace spk
