// flip.cu -- image evaluators on the device: LDR-FLIP and relMSE (include/spk.h, spk_flip / spk_relmse).
//
// The reference scores rendering tests by the mean FLIP error between a screenshot and a ground-truth PNG
// (tests/rendering/render_test_support.py:43-59, through NVIDIA's flip_evaluator package with LDR sRGB
// inputs and default parameters). This is the published LDR-FLIP (Andersson et al., HPG 2020) on the
// device: colour pipeline (sRGB -> YCxCz, contrast-sensitivity filters per opponent channel, back to linear
// RGB clamped to [0, 1], CIELAB with the Hunt adjustment, HyAB distance, power 0.7 and the piecewise map
// with pc = 0.4, pt = 0.95) and feature pipeline (first and second Gaussian-derivative filters of the
// luminance, sd = 0.5 * 0.082 degrees), combined as dEc^(1 - dF). Borders replicate the edge pixel. Filter
// weights are built on the host in double precision; all per-pixel arithmetic is fp32.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/spk.h"

namespace {

constexpr double kPi = 3.14159265358979323846;
// sRGB D65 primaries (RGB -> XYZ) and the inverse; white = XYZ of linear RGB (1, 1, 1).
constexpr double kRgb2Xyz[9] = {0.4124564, 0.3575761, 0.1804375, 0.2126729, 0.7151522,
                                0.0721750, 0.0193339, 0.1191920, 0.9503041};

struct FlipConsts {
    float rgb2xyz[9], xyz2rgb[9], white[3];
    float cmax;  // HyAB(Hunt(green), Hunt(blue))^0.7
    int sr, fr;  // spatial and feature kernel radii
};

__device__ __forceinline__ float srgb_decode(float c) {
    return c <= 0.04045f ? c / 12.92f : powf((c + 0.055f) / 1.055f, 2.4f);
}

__device__ __forceinline__ void mul3(const float *m, const float v[3], float o[3]) {
    for (int r = 0; r < 3; ++r) o[r] = m[3 * r] * v[0] + m[3 * r + 1] * v[1] + m[3 * r + 2] * v[2];
}

// Per pixel of both images: YCxCz planes (3 per image) and the luminance Y / Yn (1 per image).
__global__ void k_flip_prepare(const float *ref, const float *test, uint32_t n, FlipConsts c, float *ycc, float *lum) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int im = 0; im < 2; ++im) {
        const float *src = (im ? test : ref) + 3ull * i;
        const float lin[3] = {srgb_decode(src[0]), srgb_decode(src[1]), srgb_decode(src[2])};
        float xyz[3];
        mul3(c.rgb2xyz, lin, xyz);
        for (int a = 0; a < 3; ++a) xyz[a] /= c.white[a];
        float *o = ycc + 3ull * n * im;
        o[i] = 116.f * xyz[1] - 16.f;
        o[n + i] = 500.f * (xyz[0] - xyz[1]);
        o[2ull * n + i] = 200.f * (xyz[1] - xyz[2]);
        lum[n * im + i] = xyz[1];
    }
}

__device__ __forceinline__ float lab_f(float t) {
    const float d = 6.f / 29.f;
    return t > d * d * d ? cbrtf(t) : t / (3.f * d * d) + 4.f / 29.f;
}

// Filtered YCxCz -> Hunt-adjusted CIELAB.
__device__ void ycc_to_hunt_lab(const float ycc[3], const FlipConsts &c, float lab[3]) {
    const float y = (ycc[0] + 16.f) / 116.f;
    float xyz[3] = {(ycc[1] / 500.f + y) * c.white[0], y * c.white[1], (y - ycc[2] / 200.f) * c.white[2]};
    float rgb[3];
    mul3(c.xyz2rgb, xyz, rgb);
    for (int a = 0; a < 3; ++a) rgb[a] = fminf(fmaxf(rgb[a], 0.f), 1.f);
    mul3(c.rgb2xyz, rgb, xyz);
    const float fx = lab_f(xyz[0] / c.white[0]), fy = lab_f(xyz[1] / c.white[1]), fz = lab_f(xyz[2] / c.white[2]);
    const float L = 116.f * fy - 16.f;
    lab[0] = L;
    lab[1] = 0.01f * L * (500.f * (fx - fy));
    lab[2] = 0.01f * L * (200.f * (fy - fz));
}

// Colour error per pixel: both images' three channels through their spatial filters (kernels: A, RG, BY,
// each (2 sr + 1)^2 weights), HyAB of the Hunt-adjusted Lab values, the 0.7 power and the piecewise map.
__global__ void k_flip_colour(const float *ycc, uint32_t w, uint32_t h, const float *kernels, FlipConsts c,
                              float *dec) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = w * h;
    if (i >= n) return;
    const int x = static_cast<int>(i % w), y = static_cast<int>(i / w);
    const int r = c.sr, kw = 2 * r + 1;
    float lab[2][3];
    for (int im = 0; im < 2; ++im) {
        float f[3] = {0.f, 0.f, 0.f};
        for (int ch = 0; ch < 3; ++ch) {
            const float *plane = ycc + (3ull * im + ch) * n;
            const float *k = kernels + static_cast<size_t>(ch) * kw * kw;
            float s = 0.f;
            for (int dy = -r; dy <= r; ++dy) {
                const int yy = min(max(y + dy, 0), static_cast<int>(h) - 1);
                const float *row = plane + static_cast<size_t>(yy) * w;
                const float *krow = k + (dy + r) * kw + r;
                for (int dx = -r; dx <= r; ++dx) {
                    const int xx = min(max(x + dx, 0), static_cast<int>(w) - 1);
                    s += __ldg(krow + dx) * __ldg(row + xx);
                }
            }
            f[ch] = s;
        }
        ycc_to_hunt_lab(f, c, lab[im]);
    }
    const float dl = lab[0][0] - lab[1][0], da = lab[0][1] - lab[1][1], db = lab[0][2] - lab[1][2];
    const float de = powf(fabsf(dl) + sqrtf(da * da + db * db), 0.7f);
    const float pc = 0.4f, pt = 0.95f;
    dec[i] = de < pc * c.cmax ? pt / (pc * c.cmax) * de : pt + (de - pc * c.cmax) / (c.cmax - pc * c.cmax) * (1.f - pt);
}

// Feature difference and the final error; kernels: edge_x then point_x ((2 fr + 1)^2 each), the y kernels
// are their transposes. Adds the map's sum into *sum.
__global__ void k_flip_feature(const float *lum, uint32_t w, uint32_t h, const float *kernels, FlipConsts c,
                               const float *dec, float *map, double *sum) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = w * h;
    float v = 0.f;
    if (i < n) {
        const int x = static_cast<int>(i % w), y = static_cast<int>(i / w);
        const int r = c.fr, kw = 2 * r + 1;
        float mag[2][2];
        for (int im = 0; im < 2; ++im) {
            const float *plane = lum + static_cast<size_t>(im) * n;
            float ex = 0.f, ey = 0.f, px = 0.f, py = 0.f;
            for (int dy = -r; dy <= r; ++dy) {
                const int yy = min(max(y + dy, 0), static_cast<int>(h) - 1);
                for (int dx = -r; dx <= r; ++dx) {
                    const int xx = min(max(x + dx, 0), static_cast<int>(w) - 1);
                    const float p = __ldg(plane + static_cast<size_t>(yy) * w + xx);
                    const int kxy = (dy + r) * kw + (dx + r), kyx = (dx + r) * kw + (dy + r);
                    ex += __ldg(kernels + kxy) * p;
                    ey += __ldg(kernels + kyx) * p;
                    px += __ldg(kernels + kw * kw + kxy) * p;
                    py += __ldg(kernels + kw * kw + kyx) * p;
                }
            }
            mag[im][0] = sqrtf(ex * ex + ey * ey);
            mag[im][1] = sqrtf(px * px + py * py);
        }
        const float df = sqrtf(fmaxf(fabsf(mag[0][0] - mag[1][0]), fabsf(mag[0][1] - mag[1][1])) * 0.70710678f);
        v = powf(dec[i], 1.f - df);
        if (map) map[i] = v;
    }
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, off);
    __shared__ float part[8];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < static_cast<int>(blockDim.x >> 5); ++k) s += part[k];
        atomicAdd(sum, s);
    }
}

__global__ void k_relmse(const float *x, const float *ref, uint64_t n, float eps, double *sum) {
    double s = 0.0;
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const float d = x[i] - ref[i];
        s += static_cast<double>(d * d / (ref[i] * ref[i] + eps));
    }
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(sum, s);
}

// ---- host -----------------------------------------------------------------------------------------------

void inverse3(const double *m, double *o) {
    const double a = m[0], b = m[1], c = m[2], d = m[3], e = m[4], f = m[5], g = m[6], h = m[7], k = m[8];
    const double det = a * (e * k - f * h) - b * (d * k - f * g) + c * (d * h - e * g);
    o[0] = (e * k - f * h) / det;
    o[1] = (c * h - b * k) / det;
    o[2] = (b * f - c * e) / det;
    o[3] = (f * g - d * k) / det;
    o[4] = (a * k - c * g) / det;
    o[5] = (c * d - a * f) / det;
    o[6] = (d * h - e * g) / det;
    o[7] = (b * g - a * h) / det;
    o[8] = (a * e - b * d) / det;
}

void hunt_lab(const double rgb[3], const double white[3], double lab[3]) {
    double t[3];
    for (int r = 0; r < 3; ++r)
        t[r] = (kRgb2Xyz[3 * r] * rgb[0] + kRgb2Xyz[3 * r + 1] * rgb[1] + kRgb2Xyz[3 * r + 2] * rgb[2]) / white[r];
    const double d = 6.0 / 29.0;
    double f[3];
    for (int r = 0; r < 3; ++r) f[r] = t[r] > d * d * d ? std::cbrt(t[r]) : t[r] / (3 * d * d) + 4.0 / 29.0;
    const double L = 116.0 * f[1] - 16.0;
    lab[0] = L;
    lab[1] = 0.01 * L * 500.0 * (f[0] - f[1]);
    lab[2] = 0.01 * L * 200.0 * (f[1] - f[2]);
}

struct Weights {
    FlipConsts c{};
    std::vector<float> spatial, feature;
};

Weights make_weights(double ppd) {
    Weights wt;
    double white[3], inv[9];
    for (int r = 0; r < 3; ++r) white[r] = kRgb2Xyz[3 * r] + kRgb2Xyz[3 * r + 1] + kRgb2Xyz[3 * r + 2];
    inverse3(kRgb2Xyz, inv);
    for (int k = 0; k < 9; ++k) {
        wt.c.rgb2xyz[k] = static_cast<float>(kRgb2Xyz[k]);
        wt.c.xyz2rgb[k] = static_cast<float>(inv[k]);
    }
    for (int r = 0; r < 3; ++r) wt.c.white[r] = static_cast<float>(white[r]);
    const double green[3] = {0, 1, 0}, blue[3] = {0, 0, 1};
    double lg[3], lb[3];
    hunt_lab(green, white, lg);
    hunt_lab(blue, white, lb);
    wt.c.cmax = static_cast<float>(
        std::pow(std::fabs(lg[0] - lb[0]) + std::hypot(lg[1] - lb[1], lg[2] - lb[2]), 0.7));
    // contrast-sensitivity filters (a1, b1, a2, b2) of the A, RG and BY channels
    const double csf[3][4] = {{1.0, 0.0047, 0.0, 1e-5}, {1.0, 0.0053, 0.0, 1e-5}, {34.1, 0.04, 13.5, 0.025}};
    const int sr = static_cast<int>(std::ceil(3.0 * std::sqrt(0.04 / (2.0 * kPi * kPi)) * ppd));
    const int sw = 2 * sr + 1;
    wt.c.sr = sr;
    for (const auto &p : csf) {
        std::vector<double> g(static_cast<size_t>(sw) * sw);
        double s = 0.0;
        for (int y = -sr; y <= sr; ++y)
            for (int x = -sr; x <= sr; ++x) {
                const double r2 = (static_cast<double>(x) * x + static_cast<double>(y) * y) / (ppd * ppd);
                const double v = p[0] * std::sqrt(kPi / p[1]) * std::exp(-kPi * kPi * r2 / p[1]) +
                                 p[2] * std::sqrt(kPi / p[3]) * std::exp(-kPi * kPi * r2 / p[3]);
                g[(y + sr) * sw + (x + sr)] = v;
                s += v;
            }
        for (double v : g) wt.spatial.push_back(static_cast<float>(v / s));
    }
    const double sd = 0.5 * 0.082 * ppd;
    const int fr = static_cast<int>(std::ceil(3.0 * sd));
    const int fw = 2 * fr + 1;
    wt.c.fr = fr;
    for (int kind = 0; kind < 2; ++kind) {
        std::vector<double> g(static_cast<size_t>(fw) * fw);
        double neg = 0.0, pos = 0.0;
        for (int y = -fr; y <= fr; ++y)
            for (int x = -fr; x <= fr; ++x) {
                const double e = std::exp(-(static_cast<double>(x) * x + static_cast<double>(y) * y) / (2.0 * sd * sd));
                const double v = kind == 0 ? -x * e : (static_cast<double>(x) * x / (sd * sd) - 1.0) * e;
                g[(y + fr) * fw + (x + fr)] = v;
                (v < 0 ? neg : pos) += std::fabs(v);
            }
        for (double v : g) wt.feature.push_back(static_cast<float>(v < 0 ? v / neg : v / pos));
    }
    return wt;
}

struct DevScratch {
    std::vector<void *> ptrs;
    template <class T>
    cudaError_t get(T *&p, size_t count) {
        void *q = nullptr;
        const cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
        p = static_cast<T *>(q);
        if (e == cudaSuccess) ptrs.push_back(q);
        return e;
    }
    ~DevScratch() {
        for (void *q : ptrs) cudaFree(q);
    }
};

spk_status cuda_status(cudaError_t e) {
    return e == cudaSuccess ? SPK_OK : (e == cudaErrorMemoryAllocation ? SPK_ERR_OUT_OF_MEMORY : SPK_ERR_CUDA);
}

#define SPK_FLIP_TRY(x)                                  \
    do {                                                 \
        const cudaError_t e_ = (x);                      \
        if (e_ != cudaSuccess) return cuda_status(e_);   \
    } while (0)

}  // namespace

extern "C" {

spk_status spk_flip(int32_t device, const float *reference_rgb, const float *test_rgb, uint32_t width, uint32_t height,
                    float pixels_per_degree, float *error_map, double *mean_error) {
    if (!reference_rgb || !test_rgb || width == 0 || height == 0 || !mean_error || !(pixels_per_degree > 0.f) ||
        pixels_per_degree > 1000.f || static_cast<uint64_t>(width) * height > (1ull << 31))
        return SPK_ERR_INVALID_ARGUMENT;
    SPK_FLIP_TRY(cudaSetDevice(device));
    const uint32_t n = width * height;
    const Weights wt = make_weights(pixels_per_degree);
    DevScratch s;
    float *ref, *test, *ycc, *lum, *dec, *map, *ks, *kf;
    double *sum;
    cudaStream_t st = nullptr;
    SPK_FLIP_TRY(s.get(ref, 3ull * n));
    SPK_FLIP_TRY(s.get(test, 3ull * n));
    SPK_FLIP_TRY(s.get(ycc, 6ull * n));
    SPK_FLIP_TRY(s.get(lum, 2ull * n));
    SPK_FLIP_TRY(s.get(dec, n));
    SPK_FLIP_TRY(s.get(map, n));
    SPK_FLIP_TRY(s.get(ks, wt.spatial.size()));
    SPK_FLIP_TRY(s.get(kf, wt.feature.size()));
    SPK_FLIP_TRY(s.get(sum, 1));
    SPK_FLIP_TRY(cudaMemcpyAsync(ref, reference_rgb, 3ull * n * sizeof(float), cudaMemcpyDefault, st));
    SPK_FLIP_TRY(cudaMemcpyAsync(test, test_rgb, 3ull * n * sizeof(float), cudaMemcpyDefault, st));
    SPK_FLIP_TRY(cudaMemcpyAsync(ks, wt.spatial.data(), wt.spatial.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    SPK_FLIP_TRY(cudaMemcpyAsync(kf, wt.feature.data(), wt.feature.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    SPK_FLIP_TRY(cudaMemsetAsync(sum, 0, sizeof(double), st));
    const unsigned blocks = (n + 255) / 256;
    k_flip_prepare<<<blocks, 256, 0, st>>>(ref, test, n, wt.c, ycc, lum);
    k_flip_colour<<<blocks, 256, 0, st>>>(ycc, width, height, ks, wt.c, dec);
    k_flip_feature<<<blocks, 256, 0, st>>>(lum, width, height, kf, wt.c, dec, map, sum);
    SPK_FLIP_TRY(cudaGetLastError());
    double total = 0.0;
    SPK_FLIP_TRY(cudaMemcpyAsync(&total, sum, sizeof(double), cudaMemcpyDeviceToHost, st));
    if (error_map) SPK_FLIP_TRY(cudaMemcpyAsync(error_map, map, n * sizeof(float), cudaMemcpyDefault, st));
    SPK_FLIP_TRY(cudaStreamSynchronize(st));
    *mean_error = total / n;
    return SPK_OK;
}

spk_status spk_relmse(int32_t device, const float *x, const float *reference, uint64_t count, float eps, double *out) {
    if (!x || !reference || !out || count == 0 || !(eps > 0.f)) return SPK_ERR_INVALID_ARGUMENT;
    SPK_FLIP_TRY(cudaSetDevice(device));
    DevScratch s;
    float *dx, *dr;
    double *sum;
    cudaStream_t st = nullptr;
    SPK_FLIP_TRY(s.get(dx, count));
    SPK_FLIP_TRY(s.get(dr, count));
    SPK_FLIP_TRY(s.get(sum, 1));
    SPK_FLIP_TRY(cudaMemcpyAsync(dx, x, count * sizeof(float), cudaMemcpyDefault, st));
    SPK_FLIP_TRY(cudaMemcpyAsync(dr, reference, count * sizeof(float), cudaMemcpyDefault, st));
    SPK_FLIP_TRY(cudaMemsetAsync(sum, 0, sizeof(double), st));
    const uint64_t blocks = std::min<uint64_t>((count + 255) / 256, 152ull * 8);
    k_relmse<<<static_cast<unsigned>(blocks), 256, 0, st>>>(dx, dr, count, eps, sum);
    SPK_FLIP_TRY(cudaGetLastError());
    double total = 0.0;
    SPK_FLIP_TRY(cudaMemcpyAsync(&total, sum, sizeof(double), cudaMemcpyDeviceToHost, st));
    SPK_FLIP_TRY(cudaStreamSynchronize(st));
    *out = total / static_cast<double>(count);
    return SPK_OK;
}

}  // extern "C"
