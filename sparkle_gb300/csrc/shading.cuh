// shading.cuh -- per-pixel RNG, camera rays, hit attributes, BSDF sampling and sky on the device.
//
// Restates, in the reference's operation order: Sampler.h:16-165 (RNG, UnitDisk, VNDF, cosine
// hemisphere), BxDF.h:32-140 + PbrMaterialRenderProxy.h:15-51 + DialetricMaterialRenderProxy.h:16-37
// (SampleSurface), Utilities.h:201-330,434-451 (frames, Fresnel, Smith), MeshRenderProxy.cpp:340-361 and
// SphereRenderProxy.h:22-31 (hit attributes), SkyRenderProxy.cpp:50-64 and Image.cpp:298-357 (sky),
// CPURenderer.cpp:220-238 (SetupViewRay). Transcendentals are CUDA's sqrtf/sinf/cosf/powf (full
// precision; sqrtf and division are correctly rounded like the host's).
#pragma once

#include "traverse.cuh"

namespace spk {

// ------------------------------------------------------------------------------------------------
// RNG: Xoshiro128+ seeded through SplitMix64 (reference policy) or xoshiro256** (second policy).
// ------------------------------------------------------------------------------------------------
struct Rng {
    uint32_t s[8];  // xoshiro128+: s[0..3]; xoshiro256**: four 64-bit words as (lo, hi) pairs
};

__device__ __forceinline__ uint64_t splitmix64_next(uint64_t &st) {
    st += 0x9E3779B97F4A7C15ull;
    uint64_t z = st;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

template <int kKind>
__device__ __forceinline__ void rng_seed_pixel(Rng &r, uint32_t seed, uint32_t i, uint32_t j, uint32_t w, uint32_t h,
                                               uint32_t frame_seed) {
    if (kKind == 0) {
        // ReseedCurrentThread(j * W + i + frame_seed * W * H) in 32-bit arithmetic (CPURenderer.cpp:442-443)
        uint64_t sm = static_cast<uint64_t>(j * w + i + frame_seed * w * h);
#pragma unroll
        for (int k = 0; k < 4; ++k) r.s[k] = static_cast<uint32_t>(splitmix64_next(sm));
    } else {
        const uint64_t idx = static_cast<uint64_t>(frame_seed) * w * h + static_cast<uint64_t>(j) * w + i;
        uint64_t sm = (static_cast<uint64_t>(seed) << 40) ^ idx;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint64_t v = splitmix64_next(sm);
            r.s[2 * k] = static_cast<uint32_t>(v);
            r.s[2 * k + 1] = static_cast<uint32_t>(v >> 32);
        }
    }
}

template <int kKind>
__device__ __forceinline__ uint32_t rng_next(Rng &r) {
    if (kKind == 0) {
        const uint32_t result = r.s[0] + r.s[3];
        const uint32_t t = r.s[1] << 9;
        r.s[2] ^= r.s[0];
        r.s[3] ^= r.s[1];
        r.s[1] ^= r.s[2];
        r.s[0] ^= r.s[3];
        r.s[2] ^= t;
        r.s[3] = __funnelshift_l(r.s[3], r.s[3], 11);
        return result;
    }
    uint64_t s0 = (static_cast<uint64_t>(r.s[1]) << 32) | r.s[0];
    uint64_t s1 = (static_cast<uint64_t>(r.s[3]) << 32) | r.s[2];
    uint64_t s2 = (static_cast<uint64_t>(r.s[5]) << 32) | r.s[4];
    uint64_t s3 = (static_cast<uint64_t>(r.s[7]) << 32) | r.s[6];
    const uint64_t x = s1 * 5;
    const uint64_t result = ((x << 7) | (x >> 57)) * 9;
    const uint64_t t = s1 << 17;
    s2 ^= s0;
    s3 ^= s1;
    s1 ^= s2;
    s0 ^= s3;
    s2 ^= t;
    s3 = (s3 << 45) | (s3 >> 19);
    r.s[0] = static_cast<uint32_t>(s0);
    r.s[1] = static_cast<uint32_t>(s0 >> 32);
    r.s[2] = static_cast<uint32_t>(s1);
    r.s[3] = static_cast<uint32_t>(s1 >> 32);
    r.s[4] = static_cast<uint32_t>(s2);
    r.s[5] = static_cast<uint32_t>(s2 >> 32);
    r.s[6] = static_cast<uint32_t>(s3);
    r.s[7] = static_cast<uint32_t>(s3 >> 32);
    return static_cast<uint32_t>(result >> 32);
}

// RandomUnit: float(u32) / float(UINT32_MAX) with float(UINT32_MAX) == 2^32 (Sampler.h:32-41).
template <int kKind>
__device__ __forceinline__ float rng_unit(Rng &r) {
    return __uint2float_rn(rng_next<kKind>(r)) / 4294967296.0f;
}

template <int kKind>
__device__ __forceinline__ void unit_disk(Rng &r, float &x, float &y) {
    const float rand = rng_unit<kKind>(r);
    const float theta = rng_unit<kKind>(r) * 2.0f * kPi;
    const float rr = sqrtf(rand);
    x = rr * cosf(theta);
    y = rr * sinf(theta);
}

// ------------------------------------------------------------------------------------------------
// Surface interaction
// ------------------------------------------------------------------------------------------------
struct Surface {
    f3 location, normal, tangent;
    float uv[2];
    uint32_t material;
};

// Image2D::Sample (io/Image.h:112-150): bilinear with wrap at uv * size, the integer part truncated toward
// zero (utilities::Decompose), u lerp then v lerp, sRGB decoded after the filter.
__device__ __forceinline__ unsigned wrap_texel(int a, unsigned b) {
    return (static_cast<unsigned>(a % static_cast<int>(b)) + b) % b;  // utilities::WrapMod
}

__device__ __forceinline__ float srgb_decode(float c) {  // utilities::SRGBtoLinear per channel
    return c < 0.04045f ? c / 12.92f : powf((c + 0.055f) / 1.055f, 2.4f);
}

// One out-of-line copy: a material samples up to four textures (each with three sRGB powf), and inlining
// every call site would grow the shading kernels' code for scenes that have no textures at all.
#ifndef SPK_TEX_NOINLINE
#define SPK_TEX_NOINLINE 1
#endif
#if SPK_TEX_NOINLINE
static __device__ __noinline__ f3 tex_sample(const DevScene &S, uint32_t t, const float uv[2]) {
#else
__device__ __forceinline__ f3 tex_sample(const DevScene &S, uint32_t t, const float uv[2]) {
#endif
    const DevTexture T = S.textures[t];
    const float px = uv[0] * static_cast<float>(T.width), py = uv[1] * static_cast<float>(T.height);
    const int ui = static_cast<int>(px), vi = static_cast<int>(py);
    const float uc = px - static_cast<float>(ui), vc = py - static_cast<float>(vi);
    const unsigned x0 = wrap_texel(ui, T.width), x1 = wrap_texel(ui + 1, T.width);
    const unsigned y0 = wrap_texel(vi, T.height), y1 = wrap_texel(vi + 1, T.height);
    const float4 *px4 = S.texels + T.offset;
    const float4 s00 = __ldg(px4 + y0 * T.width + x0), s10 = __ldg(px4 + y0 * T.width + x1);
    const float4 s01 = __ldg(px4 + y1 * T.width + x0), s11 = __ldg(px4 + y1 * T.width + x1);
    const f3 l0 = mk3(s00.x + (s10.x - s00.x) * uc, s00.y + (s10.y - s00.y) * uc, s00.z + (s10.z - s00.z) * uc);
    const f3 l1 = mk3(s01.x + (s11.x - s01.x) * uc, s01.y + (s11.y - s01.y) * uc, s01.z + (s11.z - s01.z) * uc);
    f3 r = mk3(l0.x + (l1.x - l0.x) * vc, l0.y + (l1.y - l0.y) * vc, l0.z + (l1.z - l0.z) * vc);
    if (T.srgb) r = mk3(srgb_decode(r.x), srgb_decode(r.y), srgb_decode(r.z));
    return r;
}

// Per-hit material values: texture x factor (MaterialRenderProxy::GetBaseColor / GetMetallic / GetRoughness /
// GetEmissive, MaterialRenderProxy.h:117-160); a textured emission is tested per hit with SamplePixel's
// `norm() > Eps` (CPURenderer.cpp:286-287).
__device__ __forceinline__ DevMaterial resolve_material(const DevScene &S, const DevMaterial &m, const float uv[2]) {
    DevMaterial r = m;
    if (m.tex_base != kInvalid) {
        const f3 t = tex_sample(S, m.tex_base, uv);
        r.base[0] = t.x * m.base[0];
        r.base[1] = t.y * m.base[1];
        r.base[2] = t.z * m.base[2];
    }
    if (m.tex_mr != kInvalid) {
        const f3 t = tex_sample(S, m.tex_mr, uv);
        r.metallic = t.z * m.metallic;
        r.roughness = t.y * m.roughness;
    }
    if (m.tex_emissive != kInvalid) {
        const f3 t = tex_sample(S, m.tex_emissive, uv);
        r.emissive[0] = t.x * m.emissive[0];
        r.emissive[1] = t.y * m.emissive[1];
        r.emissive[2] = t.z * m.emissive[2];
        r.is_emissive = sqrtf(sqnorm(mk3(r.emissive[0], r.emissive[1], r.emissive[2]))) > kEps ? 1u : 0u;
    }
    return r;
}

// GetIntersection + Intersection::Update for the winning candidate.
__device__ __forceinline__ Surface make_surface(const DevScene &S, const TraceResult &hit, f3 o, f3 d) {
    Surface s;
    const DevInstance &I = S.instances[hit.inst];
    s.material = I.material;
    s.uv[0] = 0.f;
    s.uv[1] = 0.f;
    if (I.type == 1u) {
        const f3 center = mk3(I.m[3], I.m[7], I.m[11]);
        const f3 p = o + d * hit.t;
        s.normal = normalized(p - center);
        if (fabsf(s.normal.x) < kInvSqrt3) {
            s.tangent = mk3(1.f, 0.f, 0.f);
        } else if (fabsf(s.normal.y) < kInvSqrt3) {
            s.tangent = mk3(0.f, 1.f, 0.f);
        } else {
            s.tangent = mk3(0.f, 0.f, 1.f);
        }
    } else {
        const uint4 fi = __ldg(S.faces + I.face_base + hit.face);
        const float4 *v0 = S.verts + static_cast<size_t>(I.vert_base + fi.x) * 3;
        const float4 *v1 = S.verts + static_cast<size_t>(I.vert_base + fi.y) * 3;
        const float4 *v2 = S.verts + static_cast<size_t>(I.vert_base + fi.z) * 3;
        const float4 a0 = __ldg(v0), b0 = __ldg(v0 + 1), c0 = __ldg(v0 + 2);
        const float4 a1 = __ldg(v1), b1 = __ldg(v1 + 1), c1 = __ldg(v1 + 2);
        const float4 a2 = __ldg(v2), b2 = __ldg(v2 + 1), c2 = __ldg(v2 + 2);
        const float u = hit.u, v = hit.v;
        s.uv[0] = lerp3(b0.w, b1.w, b2.w, u, v);
        s.uv[1] = lerp3(c0.x, c1.x, c2.x, u, v);
        f3 sn = mk3(lerp3(a0.x, a1.x, a2.x, u, v), lerp3(a0.y, a1.y, a2.y, u, v), lerp3(a0.z, a1.z, a2.z, u, v));
        const f3 tg = mk3(lerp3(a0.w, a1.w, a2.w, u, v), lerp3(b0.x, b1.x, b2.x, u, v), lerp3(b0.y, b1.y, b2.y, u, v));
        const uint32_t nmap = I.normal_map;
        if (nmap != kInvalid) {
            // Normal map in the vertex tangent frame (MeshRenderProxy.cpp:349-355, TangentSpaceToWorldSpace,
            // Utilities.h:403-409): tangent-space normal = texel * 2 - 1.
            const float tw = lerp3(b0.z, b1.z, b2.z, u, v);
            const f3 t = tex_sample(S, nmap, s.uv);
            const f3 tn = mk3(t.x * 2.f - 1.f, t.y * 2.f - 1.f, t.z * 2.f - 1.f);
            const f3 bi = cross(sn, tg) * tw;
            sn = normalized(tg * tn.x + bi * tn.y + sn * tn.z);
        }
        s.normal = normalized(xform_dir(I.m, sn));
        s.tangent = xform_dir(I.m, tg);
    }
    s.location = o + d * hit.t;
    return s;
}

__device__ __forceinline__ void local_axes(f3 n, f3 major, f3 &u, f3 &v) {
    u = normalized(cross(n, major));
    v = cross(n, u);
}

__device__ __forceinline__ float schlick(float cos_i, float r0) {
    const float p = powf((1.f - cos_i), 5.f);
    return r0 + (1.f - r0) * p;
}

__device__ __forceinline__ float smith_ggx_correlated(float cos_o, float cos_i, float roughness) {
    const float a = roughness * roughness;
    const float a2 = a * a;
    const float ggx_i = cos_o * sqrtf((-cos_i * a2 + cos_i) * cos_i + a2);
    const float ggx_o = cos_i * sqrtf((-cos_o * a2 + cos_o) * cos_o + a2);
    return 2.f * cos_o * cos_i / (ggx_o + ggx_i);
}

__device__ __forceinline__ float geometry_schlick_ggx(float cos_theta, float roughness) {
    const float a = roughness * roughness;
    const float a2 = a * a;
    const float tan2_v = (1.f - cos_theta * cos_theta) / (cos_theta * cos_theta);
    return 2.f / (1.f + sqrtf(1.f + a2 * tan2_v));
}

__device__ __forceinline__ float fr_dielectric(float cos_i, float eta_i, float eta_t) {
    if (!(cos_i > 0.f)) {
        const float tmp = eta_i;
        eta_i = eta_t;
        eta_t = tmp;
        cos_i = -cos_i;
    }
    const float sin_i = sqrtf(1 - cos_i * cos_i);
    const float ref_idx = eta_i / eta_t;
    const float sin_t = ref_idx * sin_i;
    if (sin_t >= 1.f) return 1.f;
    float r0 = (1.f - ref_idx) / (1.f + ref_idx);
    r0 = r0 * r0;
    return schlick(cos_i, r0);
}

template <int kKind>
__device__ __forceinline__ f3 sample_vndf(Rng &rng, f3 w_o, float roughness) {
    const float a = roughness * roughness;
    const float u1 = rng_unit<kKind>(rng);
    const float u2 = rng_unit<kKind>(rng);
    const f3 v = normalized(mk3(w_o.x * a, w_o.y * a, w_o.z));
    const f3 t1 = (v.z < 0.999f) ? normalized(cross(v, mk3(0.f, 0.f, 1.f))) : mk3(1.f, 0.f, 0.f);
    const f3 t2 = cross(v, t1);
    const float r = sqrtf(u1);
    const float phi = 2.f * kPi * u2;
    const float p1 = r * cosf(phi);
    float p2 = r * sinf(phi);
    const float s = 0.5f * (1.f + v.z);
    p2 = (1.f - s) * sqrtf(1.f - p1 * p1) + s * p2;
    const float sq = sqrtf(max_std(0.f, 1.f - p1 * p1 - p2 * p2));
    const f3 n = p1 * t1 + p2 * t2 + sq * v;
    return normalized(mk3(a * n.x, a * n.y, max_std(0.f, n.z)));
}

// MaterialRenderProxy::SampleSurface; returns the throughput and writes the world-space w_i.
template <int kKind>
__device__ __forceinline__ f3 sample_surface(Rng &rng, const DevMaterial &mat, f3 ray_dir, f3 normal, f3 tangent,
                                             f3 &w_i, float *diffuse_z = nullptr) {
    const f3 base = mk3(mat.base[0], mat.base[1], mat.base[2]);
    const f3 w_o = -ray_dir;
    f3 fu, fv;
    local_axes(normal, tangent, fu, fv);
    const f3 lw_o = mk3(dot3(w_o, fu), dot3(w_o, fv), dot3(w_o, normal));
    f3 lw_i, thr;
    if (mat.type == 1u) {
        const float fresnel = fr_dielectric(lw_o.z, 1.0f, mat.eta);
        if (rng_unit<kKind>(rng) < fresnel) {
            lw_i = mk3(-lw_o.x, -lw_o.y, lw_o.z);
        } else {
            const float ratio = (lw_o.z > 0.f) ? 1.0f / mat.eta : mat.eta / 1.0f;
            const float cos_i = lw_o.z;
            const float sin_i2 = 1.f - cos_i * cos_i;
            const float sin_t2 = ratio * ratio * sin_i2;
            const float cos_t = sqrtf(1 - sin_t2) * (cos_i > 0.f ? -1.f : 1.f);
            lw_i = normalized(mk3(-ratio * lw_o.x, -ratio * lw_o.y, cos_t));
        }
        thr = base;
    } else {
        const f3 w_m = sample_vndf<kKind>(rng, lw_o, mat.roughness);
        const f3 cand_i = w_m * (dot3(lw_o, w_m) * 2.f) - lw_o;
        const float cos_o = fabsf(lw_o.z), cos_i = fabsf(cand_i.z), cos_m = fabsf(w_m.z);
        const float local_cos_i = dot3(cand_i, w_m);
        bool valid = false;
        f3 fc = mk3(0.f, 0.f, 0.f);
        if (cos_o > kEps && cos_i > kEps && cos_m > kEps) {
            if (rng_unit<kKind>(rng) < mat.metallic) {
                const float p = powf((1.f - local_cos_i), 5.f);
                fc = mk3(base.x + (1.f - base.x) * p, base.y + (1.f - base.y) * p, base.z + (1.f - base.z) * p);
                valid = true;
            } else {
                const float fresnel = schlick(local_cos_i, 0.04f);
                if (rng_unit<kKind>(rng) < fresnel) {
                    fc = mk3(1.f, 1.f, 1.f);
                    valid = true;
                }
            }
        }
        if (valid) {
            const float occlusion = smith_ggx_correlated(cos_o, cos_i, mat.roughness);
            const float normalizer = geometry_schlick_ggx(cos_o, mat.roughness) + kEps;
            thr = mk3(fc.x * occlusion / normalizer, fc.y * occlusion / normalizer, fc.z * occlusion / normalizer);
            lw_i = cand_i;
        } else {
            float dx, dy;
            unit_disk<kKind>(rng, dx, dy);
            const float sq = dx * dx + dy * dy;
            lw_i = mk3(dx, dy, sqrtf(max_std(0.f, 1.0f - sq)));
            thr = base;
            if (diffuse_z) *diffuse_z = lw_i.z;  // the diffuse fall-through branch was taken
        }
    }
    f3 gu, gv;
    local_axes(normal, tangent, gu, gv);
    w_i = normalized(gu * lw_i.x + gv * lw_i.y + normal * lw_i.z);
    return thr;
}

// GetMISWeight (power heuristic, ray_trace.cs.slang:176-186).
__device__ __forceinline__ float mis_weight(float current_pdf, float compensation_pdf) {
    if (current_pdf < kEps || compensation_pdf < kEps) return 1.f;
    const float c2 = current_pdf * current_pdf;
    const float o2 = compensation_pdf * compensation_pdf;
    return c2 / (o2 + c2 + kEps);
}

constexpr float kInvPi = 0.318309886183790671538f;  // std::numbers::inv_pi_v<float> (Types.h:52)

// ------------------------------------------------------------------------------------------------
// Sky
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t wrap_mod(int a, uint32_t b) {
    return (static_cast<uint32_t>(a % static_cast<int>(b)) + b) % b;
}

__device__ __forceinline__ f3 sky_eval(const DevScene &S, f3 d) {
    if (S.sky_mode == 2u) {
        const float x = d.x, y = d.y, z = d.z;
        const float ax = fabsf(x), ay = fabsf(y), az = fabsf(z);
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
        const uint32_t n = S.sky_size;
        const float px = u * static_cast<float>(n - 1), py = v * static_cast<float>(n - 1);
        const int ui = static_cast<int>(px), vi = static_cast<int>(py);
        const float uc = px - static_cast<float>(ui), vc = py - static_cast<float>(vi);
        const float4 *f = S.sky_cube + static_cast<size_t>(face) * n * n;
        const uint32_t x0 = wrap_mod(ui, n), x1 = wrap_mod(ui + 1, n), y0 = wrap_mod(vi, n), y1 = wrap_mod(vi + 1, n);
        const float4 s00 = __ldg(f + y0 * n + x0), s10 = __ldg(f + y0 * n + x1);
        const float4 s01 = __ldg(f + y1 * n + x0), s11 = __ldg(f + y1 * n + x1);
        const float lx0 = s00.x + (s10.x - s00.x) * uc, lx1 = s01.x + (s11.x - s01.x) * uc;
        const float ly0 = s00.y + (s10.y - s00.y) * uc, ly1 = s01.y + (s11.y - s01.y) * uc;
        const float lz0 = s00.z + (s10.z - s00.z) * uc, lz1 = s01.z + (s11.z - s01.z) * uc;
        return mk3(lx0 + (lx1 - lx0) * vc, ly0 + (ly1 - ly0) * vc, lz0 + (lz1 - lz0) * vc);
    }
    if (S.sky_mode == 1u) {
        const float t = 0.5f * d.z + 0.5f;
        return mk3(1.f + (S.sky_color[0] - 1.f) * t, 1.f + (S.sky_color[1] - 1.f) * t,
                   1.f + (S.sky_color[2] - 1.f) * t);
    }
    return mk3(0.f, 0.f, 0.f);
}

// ------------------------------------------------------------------------------------------------
// Next-event estimation (no counterpart in the reference cpu pipeline; its GPU shader samples only the
// sky, ray_trace.cs.slang:118-174). Called at a vertex where the PBR sampler took the diffuse
// fall-through branch: one point on the emissive triangles (area CDF, uniform on the triangle) and one
// cosine-weighted sky direction, each with an occlusion ray and the shader's power-heuristic weight
// against the diffuse branch's cosine pdf. The estimator is the cpu BSDF's (base/pi * L * cos / pdf), so
// NEE converges to the plain path tracer's image. Contributions are added to `color` in that order.
//
// nee_prepare draws the random numbers and computes both occlusion rays and the radiance each adds when
// it is unoccluded; nee_direct walks the two rays inline and adds. The wavefront's shadow stage walks the
// prepared rays in their own persistent kernel and adds the same contributions in the same order, so
// both give the same bits.
// ------------------------------------------------------------------------------------------------
struct NeeRay {
    f3 o, d;
    float tmax;
    f3 contrib;  // added to the path's colour when the ray is unoccluded
    bool valid;  // false: no ray (no light / sky, or a back-facing sample)
};

template <int kKind>
__device__ __forceinline__ void nee_prepare(const DevScene &S, Rng &rng, const Surface &surf, f3 base, f3 thr,
                                            NeeRay &light, NeeRay &sky) {
    light.valid = false;
    sky.valid = false;
    if (S.num_lights > 0) {
        const float u0 = rng_unit<kKind>(rng), u1 = rng_unit<kKind>(rng), u2 = rng_unit<kKind>(rng);
        const float target = u0 * S.light_total;
        uint32_t lo = 0, hi = S.num_lights;  // first cdf entry > target
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (__ldg(S.light_cdf + mid) > target) {
                hi = mid;
            } else {
                lo = mid + 1;
            }
        }
        const DevLight &L = S.lights[lo < S.num_lights ? lo : S.num_lights - 1];
        const float r1 = sqrtf(u1);
        const float a = r1 * (1.f - u2), b = r1 * u2;
        const f3 x = mk3(L.p0[0], L.p0[1], L.p0[2]) + mk3(L.e1[0], L.e1[1], L.e1[2]) * a +
                     mk3(L.e2[0], L.e2[1], L.e2[2]) * b;
        const f3 to = x - surf.location;
        const float dist2 = sqnorm(to);
        if (dist2 > 0.f) {
            const float dist = sqrtf(dist2);
            const f3 w = mk3(to.x / dist, to.y / dist, to.z / dist);
            const float cos_s = dot3(surf.normal, w);
            const float cos_l = fabsf(dot3(mk3(L.ng[0], L.ng[1], L.ng[2]), w));
            if (cos_s > 0.f && cos_l > kEps) {
                const float pdf_l = dist2 / (S.light_total * cos_l);
                const float pdf_b = cos_s * kInvPi;
                const float wl = mis_weight(pdf_l, pdf_b);
                light.o = surf.location + w * kTolerance;
                light.d = w;
                light.tmax = (dist - kTolerance) * (1.f - 1e-4f);
                const float f = cos_s / pdf_l * wl * kInvPi;
                light.contrib = mk3(thr.x * base.x * L.emission[0] * f, thr.y * base.y * L.emission[1] * f,
                                    thr.z * base.z * L.emission[2] * f);
                light.valid = true;
            }
        }
    }
    if (S.sky_mode != 0u) {
        f3 fu, fv;
        local_axes(surf.normal, surf.tangent, fu, fv);
        float dx, dy;
        unit_disk<kKind>(rng, dx, dy);
        const float z = sqrtf(max_std(0.f, 1.0f - (dx * dx + dy * dy)));
        const f3 w = normalized(fu * dx + fv * dy + surf.normal * z);
        const float pdf = z * kInvPi;
        if (pdf > 0.f) {
            const float wl = mis_weight(pdf, pdf);
            sky.o = surf.location + w * kTolerance;
            sky.d = w;
            sky.tmax = 1000.f;
            const f3 Ls = sky_eval(S, w);
            const float f = z / pdf * wl * kInvPi;
            sky.contrib = mk3(thr.x * base.x * Ls.x * f, thr.y * base.y * Ls.y * f, thr.z * base.z * Ls.z * f);
            sky.valid = true;
        }
    }
}

template <int kKind, bool kCount>
__device__ __forceinline__ void nee_direct(const DevScene &S, Rng &rng, const Surface &surf, f3 base, f3 thr,
                                           f3 &color, uint32_t &shadow_rays, uint32_t &err, TraceCounts *tc) {
    NeeRay rays[2];
    nee_prepare<kKind>(S, rng, surf, base, thr, rays[0], rays[1]);
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        if (!rays[k].valid) continue;
        ++shadow_rays;
        if (trace_ray<kTraceOcclusion, kCount>(S, rays[k].o, rays[k].d, rays[k].tmax, err, tc).inst == kInvalid)
            color = color + rays[k].contrib;
    }
}

// MIS weight of the emission a BSDF-sampled ray collects when the previous vertex also sampled the lights
// (prev_pdf = cosine pdf of the direction it continued in; 0 when it did not sample the lights).
__device__ __forceinline__ float bsdf_hit_weight(const DevScene &S, float prev_pdf, const TraceResult &hit, f3 d) {
    if (!(prev_pdf > 0.f) || hit.face == kInvalid) return 1.f;
    const uint32_t base = S.instances[hit.inst].light_base;
    if (base == kInvalid) return 1.f;
    const DevLight &L = S.lights[base + hit.face];
    const float cos_l = fabsf(dot3(mk3(L.ng[0], L.ng[1], L.ng[2]), d));
    if (!(cos_l > kEps)) return 1.f;
    return mis_weight(prev_pdf, (hit.t * hit.t) / (S.light_total * cos_l));
}

// ------------------------------------------------------------------------------------------------
// Camera (SetupViewRay, CPURenderer.cpp:220-238)
// ------------------------------------------------------------------------------------------------
struct DevCamera {
    float position[3], right[3], up[3], front[3], lower_left[3], max_u[3], max_v[3];
    float aperture_radius, exposure, far_plane;
};

template <int kKind>
__device__ __forceinline__ void camera_ray(const DevCamera &cam, Rng &rng, float u, float v, f3 &o, f3 &d) {
    float ax, ay;
    unit_disk<kKind>(rng, ax, ay);
    ax = ax * cam.aperture_radius;
    ay = ay * cam.aperture_radius;
    const f3 right = mk3(cam.right[0], cam.right[1], cam.right[2]);
    const f3 up = mk3(cam.up[0], cam.up[1], cam.up[2]);
    const f3 lens = ax * right + ay * up;
    o = mk3(cam.position[0], cam.position[1], cam.position[2]) + lens;
    const f3 focus = mk3(cam.lower_left[0], cam.lower_left[1], cam.lower_left[2]) +
                     u * mk3(cam.max_u[0], cam.max_u[1], cam.max_u[2]) + v * mk3(cam.max_v[0], cam.max_v[1], cam.max_v[2]);
    d = normalized(focus - o);
}

}  // namespace spk
