// spk_math.cuh -- single-precision vector math in the evaluation order of the reference's Eigen code.
//
// The reference computes with Eigen 3 fixed-size vectors (libraries/include/core/math/Types.h:10-40).
// Eigen evaluates a 3-term reduction (dot, squaredNorm, one row of a 3x3 product) as x0 + (x1 + x2) and
// normalized() as v / sqrt(squaredNorm) when squaredNorm > 0; every helper here keeps that order. The
// translation units that include this header are compiled with -fmad=false, so no multiply-add is
// contracted unless written as fmaf() explicitly (the slab tests do that on purpose).
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define SPK_HD __host__ __device__ __forceinline__
#else
#define SPK_HD inline
#endif

namespace spk {

constexpr float kEps = 1e-6f;        // Types.h:54 Eps
constexpr float kTolerance = 1e-4f;  // Types.h:55 Tolerance
constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvSqrt3 = 0.577350269189625764509f;
constexpr float kOutputLimit = 6.f;  // CameraRenderProxy.h:16 OutputLimit
constexpr float kFltMax = 3.402823466e+38f;
constexpr uint32_t kInvalid = 0xFFFFFFFFu;

struct f3 {
    float x, y, z;
};

SPK_HD f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
SPK_HD f3 operator+(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
SPK_HD f3 operator-(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
SPK_HD f3 operator-(f3 a) { return f3{-a.x, -a.y, -a.z}; }
SPK_HD f3 operator*(f3 a, float s) { return f3{a.x * s, a.y * s, a.z * s}; }
SPK_HD f3 operator*(float s, f3 a) { return f3{s * a.x, s * a.y, s * a.z}; }
SPK_HD f3 cmul(f3 a, f3 b) { return f3{a.x * b.x, a.y * b.y, a.z * b.z}; }
SPK_HD float sum3(float a, float b, float c) { return a + (b + c); }
SPK_HD float dot3(f3 a, f3 b) { return sum3(a.x * b.x, a.y * b.y, a.z * b.z); }
SPK_HD float sqnorm(f3 a) { return dot3(a, a); }
SPK_HD f3 cross(f3 a, f3 b) { return f3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
SPK_HD f3 normalized(f3 a) {
    const float z = sqnorm(a);
    if (z > 0.f) {
        const float s = sqrtf(z);
        return f3{a.x / s, a.y / s, a.z / s};
    }
    return a;
}
// std::min / std::max operand order (NaN in the left operand is returned by min only if b < a fails).
SPK_HD float min_std(float a, float b) { return (b < a) ? b : a; }
SPK_HD float max_std(float a, float b) { return (a < b) ? b : a; }
// RenderPixel's per-sample clamp min(c, OutputLimit) (CPURenderer.cpp:408), except that a non-finite
// component becomes 0. The reference lets a NaN through the clamp into the running mean, where it stays
// for good; NaN samples come from its Refract (Utilities.h:213-220, no total-internal-reflection guard)
// when RandomUnit() returns exactly 1.0 or when FrDielectric's `sin_t >= 1` test and Refract's sin^2
// round differently at the critical angle. Every finite sample is unchanged.
SPK_HD float clamp_sample(float c) { return (c - c == 0.f) ? min_std(c, kOutputLimit) : 0.f; }

// Affine 3x4, row-major: TransformPoint = t + L*p, TransformDirection = L*d (Transform.h:95-103).
SPK_HD f3 xform_point(const float *m, f3 p) {
    return f3{m[3] + sum3(m[0] * p.x, m[1] * p.y, m[2] * p.z), m[7] + sum3(m[4] * p.x, m[5] * p.y, m[6] * p.z),
              m[11] + sum3(m[8] * p.x, m[9] * p.y, m[10] * p.z)};
}
SPK_HD f3 xform_dir(const float *m, f3 d) {
    return f3{sum3(m[0] * d.x, m[1] * d.y, m[2] * d.z), sum3(m[4] * d.x, m[5] * d.y, m[6] * d.z),
              sum3(m[8] * d.x, m[9] * d.y, m[10] * d.z)};
}

// Utilities::Lerp(v0, v1, v2, u, v) (Utilities.h:114-117).
SPK_HD float lerp3(float a, float b, float c, float u, float v) { return a + (b - a) * u + (c - a) * v; }

}  // namespace spk
