// bvh_device.cu -- BLAS refit kernels (bvh_device.cuh).
#include "bvh_device.cuh"

#include <cfloat>

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
    // Quantise as the host builder does: origin = the node box's low corner, the smallest power-of-two
    // scale that spans the box in 255 steps, child boxes rounded outwards, flat children widened by a step.
    for (int a = 0; a < 3; ++a) {
        const double origin = lo[a];
        const int e = quant_exponent(static_cast<double>(hi[a]) - origin);
        const double scale = ldexp(1.0, e);
        n.f[a] = lo[a];
        n.b[12 + a] = static_cast<uint8_t>(e + 127);
        for (int s = 0; s < 8; ++s) {
            if (n.b[24 + s] == 0) continue;
            double ql = floor((static_cast<double>(clo[s][a]) - origin) / scale);
            double qh = ceil((static_cast<double>(chi[s][a]) - origin) / scale);
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
