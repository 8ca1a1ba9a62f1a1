// unet.cu -- the learned denoiser (include/spk_denoise.h): U-Net graph, training step, inference and
// the per-tile fallback, on the tcgen05 convolutions of conv_tc.cu plus memory-bound glue kernels.
//
// Tensors are NHWC BF16 in device memory. Level l has P_l = n * (h >> l) * (w >> l) pixels. The skip
// concatenation of level l < 4 is one buffer cat[l] of (W[l+1] + W[l]) channels per pixel: the decoder's
// upsampled input fills channels [0, W[l+1]) and the encoder's second conv writes its output straight into
// channels [W[l+1], W[l+1] + W[l]), so concatenation costs nothing.
#include <cuda_bf16.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "conv_tc.cuh"
#include "fault.h"
#include "spk_denoise.h"
#include "../../include/spk.h"

using bf16 = __nv_bfloat16;

namespace spk {
namespace {

constexpr uint32_t kLevels = 5;
constexpr uint32_t kW[kLevels] = {32, 64, 96, 128, 128};
constexpr uint32_t kInPad = 32;   // 10 features padded to 32 channels
constexpr uint32_t kOutPad = 32;  // 3 outputs padded to 32 channels
constexpr uint32_t kNumLayers = 19;
constexpr float kOutClamp = 16.f;  // log1p-space output clamp before expm1

// Layer order: enc0a enc0b enc1a enc1b ... enc4a enc4b, dec3a dec3b dec2a dec2b dec1a dec1b dec0a dec0b, out.
constexpr uint32_t enc_a(uint32_t l) { return 2 * l; }
constexpr uint32_t enc_b(uint32_t l) { return 2 * l + 1; }
constexpr uint32_t dec_a(uint32_t l) { return 10 + 2 * (3 - l); }
constexpr uint32_t dec_b(uint32_t l) { return 11 + 2 * (3 - l); }
constexpr uint32_t kOutLayer = 18;
constexpr uint32_t cat_channels(uint32_t l) { return kW[l + 1] + kW[l]; }

struct Layer {
    uint32_t cin, cout;
    bool relu;
    size_t w_off, b_off;  // offsets into the FP32 parameter vector
    size_t wb_off;        // offset into the BF16 weight buffers (elements)
};

std::vector<Layer> make_layers() {
    std::vector<Layer> L(kNumLayers);
    for (uint32_t l = 0; l < kLevels; ++l) {
        L[enc_a(l)] = {l == 0 ? kInPad : kW[l - 1], kW[l], true, 0, 0, 0};
        L[enc_b(l)] = {kW[l], kW[l], true, 0, 0, 0};
    }
    for (uint32_t l = 0; l < 4; ++l) {
        L[dec_a(l)] = {cat_channels(l), kW[l], true, 0, 0, 0};
        L[dec_b(l)] = {kW[l], kW[l], true, 0, 0, 0};
    }
    L[kOutLayer] = {kW[0], kOutPad, false, 0, 0, 0};
    size_t off = 0, wb = 0;
    for (Layer &x : L) {
        x.w_off = off;
        off += static_cast<size_t>(x.cout) * 9 * x.cin;
        x.b_off = off;
        off += x.cout;
        x.wb_off = wb;
        wb += static_cast<size_t>(x.cout) * 9 * x.cin;
    }
    return L;
}

size_t param_count(const std::vector<Layer> &L) { return L.back().b_off + L.back().cout; }
size_t weight_count(const std::vector<Layer> &L) {
    return L.back().wb_off + static_cast<size_t>(L.back().cout) * 9 * L.back().cin;
}

template <class T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t count) {
        if (count <= n) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        const cudaError_t e = fault_allocation() ? cudaErrorMemoryAllocation
                                                 : cudaMalloc(reinterpret_cast<void **>(&p), std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) n = count;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

// ------------------------------------------------------------------------------------------------
// Glue kernels
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ float bf(const bf16 v) { return __bfloat162float(v); }

// features fp32 [n][h][w][10] -> X0 bf16 [n][hp][wp][32], edge replication into the padding. One thread
// per (pixel, 8-channel group), so a warp writes 512 contiguous bytes.
__global__ void k_input(const float *feat, bf16 *x0, uint32_t n, uint32_t h, uint32_t w, uint32_t hp, uint32_t wp) {
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;  // (pixel, channel group)
    const size_t total = static_cast<size_t>(n) * hp * wp * (kInPad / 8u);
    if (i >= total) return;
    const uint32_t grp = static_cast<uint32_t>(i % (kInPad / 8u));
    const size_t q = i / (kInPad / 8u);
    const uint32_t x = static_cast<uint32_t>(q % wp), y = static_cast<uint32_t>((q / wp) % hp);
    const uint32_t img = static_cast<uint32_t>(q / (static_cast<size_t>(wp) * hp));
    const uint32_t sx = min(x, w - 1), sy = min(y, h - 1);
    const float *f = feat + ((static_cast<size_t>(img) * h + sy) * w + sx) * SPK_DN_FEATURES;
    uint32_t pk[4];
#pragma unroll
    for (uint32_t k = 0; k < 4; ++k) {
        const uint32_t c = grp * 8u + 2u * k;
        const float a = c < SPK_DN_FEATURES ? f[c] : 0.f, b = c + 1 < SPK_DN_FEATURES ? f[c + 1] : 0.f;
        const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
        pk[k] = *reinterpret_cast<const uint32_t *>(&v);
    }
    *reinterpret_cast<uint4 *>(x0 + q * kInPad + grp * 8u) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
}

// Nearest 2x upsampling: src [n][h][w][c] (dense) -> dst view [n][2h][2w] (ld_d, first c channels).
__global__ void k_upsample(const bf16 *src, bf16 *dst, uint32_t ld_d, uint32_t n, uint32_t h, uint32_t w, uint32_t c) {
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;  // (fine pixel, 8-channel group)
    const uint32_t cg = c / 8;
    const size_t total = static_cast<size_t>(n) * 4 * h * w * cg;
    if (i >= total) return;
    const uint32_t g = static_cast<uint32_t>(i % cg);
    const size_t p = i / cg;
    const uint32_t W2 = 2 * w, H2 = 2 * h;
    const uint32_t x = static_cast<uint32_t>(p % W2), y = static_cast<uint32_t>((p / W2) % H2);
    const uint32_t img = static_cast<uint32_t>(p / (static_cast<size_t>(W2) * H2));
    const size_t q = (static_cast<size_t>(img) * h + y / 2) * w + x / 2;
    *reinterpret_cast<uint4 *>(dst + p * ld_d + g * 8) = *reinterpret_cast<const uint4 *>(src + q * c + g * 8);
}

__device__ __forceinline__ float relu_mask(const bf16 *ref, size_t idx) { return bf(ref[idx]) > 0.f ? 1.f : 0.f; }

// Upsampling backward + ReLU mask: dst[q][ch] = (sum of the 4 children of q in src view) * (ref[q] > 0).
__global__ void k_upsample_bwd(const bf16 *src, uint32_t ld_s, const bf16 *ref, uint32_t ld_r, bf16 *dst, uint32_t n,
                               uint32_t h, uint32_t w, uint32_t c) {
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const size_t total = static_cast<size_t>(n) * h * w * c;
    if (i >= total) return;
    const uint32_t ch = static_cast<uint32_t>(i % c);
    const size_t q = i / c;
    const uint32_t x = static_cast<uint32_t>(q % w), y = static_cast<uint32_t>((q / w) % h);
    const uint32_t img = static_cast<uint32_t>(q / (static_cast<size_t>(w) * h));
    float s = 0.f;
    for (uint32_t dy = 0; dy < 2; ++dy)
        for (uint32_t dx = 0; dx < 2; ++dx) {
            const size_t p = (static_cast<size_t>(img) * 2 * h + 2 * y + dy) * (2 * w) + 2 * x + dx;
            s += bf(src[p * ld_s + ch]);
        }
    dst[q * c + ch] = __float2bfloat16_rn(s * relu_mask(ref, q * ld_r + ch));
}

// Pooling backward + skip gradient + ReLU mask at the fine level:
// dst[p][ch] = (gpool[parent(p)][ch] / 4 + skip[p][ch]) * (ref[p][ch] > 0).
__global__ void k_pool_bwd(const bf16 *gpool, const bf16 *skip, uint32_t ld_skip, const bf16 *ref, uint32_t ld_r,
                           bf16 *dst, uint32_t n, uint32_t h, uint32_t w, uint32_t c) {
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;  // fine (pixel, channel)
    const size_t total = static_cast<size_t>(n) * h * w * c;
    if (i >= total) return;
    const uint32_t ch = static_cast<uint32_t>(i % c);
    const size_t p = i / c;
    const uint32_t x = static_cast<uint32_t>(p % w), y = static_cast<uint32_t>((p / w) % h);
    const uint32_t img = static_cast<uint32_t>(p / (static_cast<size_t>(w) * h));
    const size_t q = (static_cast<size_t>(img) * (h / 2) + y / 2) * (w / 2) + x / 2;
    const float g = 0.25f * bf(gpool[q * c + ch]) + bf(skip[p * ld_skip + ch]);
    dst[p * c + ch] = __float2bfloat16_rn(g * relu_mask(ref, p * ld_r + ch));
}

// relMSE loss and its gradient with respect to the network output o (log1p space):
// d = expm1(o), L = mean((d - t)^2 / (t^2 + 0.01)), dL/do = 2 (d - t) / (t^2 + 0.01) * exp(o) / (3P).
__global__ void k_loss(const bf16 *out, const float *target, bf16 *gout, uint32_t n, uint32_t h, uint32_t w,
                       double *loss_sum) {
    const size_t p = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const size_t total = static_cast<size_t>(n) * h * w;
    float l = 0.f;
    if (p < total) {
        const float scale = 1.f / (3.f * static_cast<float>(total));
        bf16 *g = gout + p * kOutPad;
        for (uint32_t c = 0; c < 3; ++c) {
            float o = bf(out[p * kOutPad + c]);
            const bool clamped = o > kOutClamp;
            o = fminf(o, kOutClamp);
            const float e = expf(o);
            const float d = e - 1.f;
            const float t = target[p * 3 + c];
            const float den = t * t + 0.01f;
            const float diff = d - t;
            l += diff * diff / den;
            g[c] = __float2bfloat16_rn(clamped ? 0.f : 2.f * diff / den * e * scale);
        }
        for (uint32_t c = 3; c < kOutPad; ++c) g[c] = __float2bfloat16_rn(0.f);
    }
    // block reduction
    __shared__ float red[32];
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xFFFFFFFFu, l, o);
    if ((threadIdx.x & 31u) == 0) red[threadIdx.x >> 5] = l;
    __syncthreads();
    if (threadIdx.x < 32) {
        float v = threadIdx.x < blockDim.x / 32 ? red[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
        if (threadIdx.x == 0) atomicAdd(loss_sum, static_cast<double>(v));
    }
}

// db[c] += sum_p g[p][c] (dense [P][c]); 256 threads: 8 pixel rows x 32 channel lanes per pass.
__global__ void k_bias_grad(const bf16 *g, size_t npix, uint32_t c, float *db) {
    const uint32_t lane = threadIdx.x & 31u, row = threadIdx.x >> 5;
    for (uint32_t c0 = 0; c0 < c; c0 += 32) {
        float s = 0.f;
        for (size_t p = static_cast<size_t>(blockIdx.x) * 8 + row; p < npix; p += static_cast<size_t>(gridDim.x) * 8)
            s += bf(g[p * c + c0 + lane]);
        __shared__ float red[8][32];
        red[row][lane] = s;
        __syncthreads();
        if (row == 0) {
            float t = 0.f;
            for (int r = 0; r < 8; ++r) t += red[r][lane];
            atomicAdd(db + c0 + lane, t);
        }
        __syncthreads();
    }
}

__global__ void k_adam(float *w, const float *g, float *m, float *v, size_t n, float lr, float b1, float b2, float eps,
                       float bc1, float bc2) {
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

// Every layer's weights in one launch: layer k covers the weight elements [first[k], first[k + 1]) of
// the concatenated BF16 buffers.
struct WeightTable {
    uint32_t count;
    uint32_t cin[kNumLayers], cout[kNumLayers];
    unsigned long long w_off[kNumLayers], wb_off[kNumLayers], first[kNumLayers + 1];
};

// BF16 copy w_b[co][tap][ci] of each FP32 weight and the dgrad copy wt[ci][8 - tap][co] of the same
// value (the layout conv3x3_transpose_weights writes), one thread per weight element of all layers.
__global__ void k_refresh_weights(const __grid_constant__ WeightTable T, const float *params, bf16 *wb, bf16 *wt) {
    const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= T.first[T.count]) return;
    uint32_t k = 0;
    while (k + 1 < T.count && T.first[k + 1] <= i) ++k;
    const unsigned long long j = i - T.first[k];  // (co * 9 + tap) * cin + ci within the layer
    const uint32_t cin = T.cin[k], cout = T.cout[k];
    const uint32_t ci = static_cast<uint32_t>(j % cin), tap = static_cast<uint32_t>((j / cin) % 9u);
    const uint32_t co = static_cast<uint32_t>(j / (9ull * cin));
    const bf16 v = __float2bfloat16_rn(params[T.w_off[k] + j]);
    wb[T.wb_off[k] + j] = v;
    wt[T.wb_off[k] + (static_cast<unsigned long long>(ci) * 9u + (8u - tap)) * cout + co] = v;
}


// OUT [n][hp][wp][32] -> rgb float4 [n][h][w] (expm1 of the log1p prediction).
__global__ void k_decode(const bf16 *out, float4 *dst, uint32_t n, uint32_t h, uint32_t w, uint32_t hp, uint32_t wp) {
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const size_t total = static_cast<size_t>(n) * h * w;
    if (i >= total) return;
    const uint32_t x = static_cast<uint32_t>(i % w), y = static_cast<uint32_t>((i / w) % h);
    const uint32_t img = static_cast<uint32_t>(i / (static_cast<size_t>(w) * h));
    const bf16 *o = out + ((static_cast<size_t>(img) * hp + y) * wp + x) * kOutPad;
    float r[3];
    for (int c = 0; c < 3; ++c) r[c] = fmaxf(expm1f(fminf(bf(o[c]), kOutClamp)), 0.f);
    dst[i] = make_float4(r[0], r[1], r[2], 1.f);
}

__device__ __forceinline__ void write_features(float4 c, float4 n, float4 a, float *f) {
    f[0] = log1pf(fmaxf(c.x, 0.f));
    f[1] = log1pf(fmaxf(c.y, 0.f));
    f[2] = log1pf(fmaxf(c.z, 0.f));
    f[3] = a.x;
    f[4] = a.y;
    f[5] = a.z;
    f[6] = n.x;
    f[7] = n.y;
    f[8] = n.z;
    f[9] = 0.25f * log1pf(fmaxf(n.w, 0.f));
}

__global__ void k_pack_features(const float4 *hdr, const float4 *nd, const float4 *alb, float *feat, size_t total) {
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= total) return;
    write_features(hdr[i], nd[i], alb[i], feat + i * SPK_DN_FEATURES);
}

__global__ void k_pack_halves(const float4 *full, const float4 *half_a, const float4 *nd, const float4 *alb,
                              float *feat_a, float *feat_b, size_t total) {
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const float4 f = full[i], a = half_a[i];
    const float4 b = make_float4(2.f * f.x - a.x, 2.f * f.y - a.y, 2.f * f.z - a.z, 1.f);
    write_features(a, nd[i], alb[i], feat_a + i * SPK_DN_FEATURES);
    write_features(b, nd[i], alb[i], feat_b + i * SPK_DN_FEATURES);
}

// One block per tile: relative variance of the two denoised halves; tiles above the threshold take the
// plain image.
__global__ void k_fallback(const float4 *den, const float4 *da, const float4 *db, const float4 *plain, float4 *out,
                           uint32_t h, uint32_t w, uint32_t tile, float threshold, unsigned int *count) {
    const uint32_t tiles_x = (w + tile - 1) / tile;
    const uint32_t tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
    const uint32_t x0 = tx * tile, y0 = ty * tile;
    const uint32_t tw = min(tile, w - x0), th = min(tile, h - y0);
    float var = 0.f, mean = 0.f;
    for (uint32_t k = threadIdx.x; k < tw * th; k += blockDim.x) {
        const size_t p = static_cast<size_t>(y0 + k / tw) * w + x0 + k % tw;
        const float4 a = da[p], b = db[p], d = den[p];
        const float ex = 0.5f * (a.x - b.x), ey = 0.5f * (a.y - b.y), ez = 0.5f * (a.z - b.z);
        var += ex * ex + ey * ey + ez * ez;
        mean += d.x + d.y + d.z;
    }
    __shared__ float rv[32], rm[32];
    for (int o = 16; o > 0; o >>= 1) {
        var += __shfl_xor_sync(0xFFFFFFFFu, var, o);
        mean += __shfl_xor_sync(0xFFFFFFFFu, mean, o);
    }
    if ((threadIdx.x & 31u) == 0) {
        rv[threadIdx.x >> 5] = var;
        rm[threadIdx.x >> 5] = mean;
    }
    __syncthreads();
    __shared__ int use_plain;
    if (threadIdx.x == 0) {
        float V = 0.f, M = 0.f;
        for (uint32_t k = 0; k < blockDim.x / 32; ++k) {
            V += rv[k];
            M += rm[k];
        }
        const float cnt = 3.f * static_cast<float>(tw * th);
        V /= cnt;
        M /= cnt;
        use_plain = V / (M * M + 1e-4f) > threshold;
        if (use_plain) atomicAdd(count, 1u);
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < tw * th; k += blockDim.x) {
        const size_t p = static_cast<size_t>(y0 + k / tw) * w + x0 + k % tw;
        out[p] = use_plain ? plain[p] : den[p];
    }
}

unsigned blocks_for(size_t n, unsigned t) { return static_cast<unsigned>((n + t - 1) / t); }

// Splitmix64-driven Box-Muller normal draws (the same on every host).
struct NormalGen {
    uint64_t s;
    bool has = false;
    double spare = 0.0;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (static_cast<double>(next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
    double normal() {
        if (has) {
            has = false;
            return spare;
        }
        const double u1 = uniform(), u2 = uniform();
        const double r = std::sqrt(-2.0 * std::log(u1)), th = 6.283185307179586 * u2;
        spare = r * std::sin(th);
        has = true;
        return r * std::cos(th);
    }
};

}  // namespace
}  // namespace spk

using namespace spk;

// An NVTX range around one denoiser entry point (shown by Nsight tools; free when none is attached).
struct DnRange {
    explicit DnRange(const char *name) { nvtxRangePushA(name); }
    ~DnRange() { nvtxRangePop(); }
};

struct spk_denoiser {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::string error;
    std::vector<Layer> layers;
    size_t nparams = 0, nweights = 0;
    DBuf<float> params, grads, adam_m, adam_v;
    DBuf<bf16> wb, wt;  // BF16 weights [cout][9][cin] and dgrad weights [cin][9][cout]
    uint64_t adam_t = 0;
    DBuf<uint32_t> err;
    DBuf<float> frame;  // spk_render_denoised scratch
    DBuf<double> loss;
    // activations (forward) and gradients (backward), sized for the largest batch seen
    DBuf<bf16> x0, out, gout;
    DBuf<bf16> ea[kLevels], eb4, cat[4], pool[4], da[4], db[4];
    DBuf<bf16> g_ea[kLevels], g_eb[kLevels], g_cat[4], g_pool[4], g_da[4], g_db[4];
    DBuf<bf16> conv_wt_scratch;
    bool weights_dirty = true;
};

namespace {

spk_status dn_fail(spk_denoiser *dn, spk_status st, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    dn->error = buf;
    return st;
}

spk_status dn_cuda(spk_denoiser *dn, cudaError_t e, const char *what) {
    return dn_fail(dn, e == cudaErrorMemoryAllocation ? SPK_ERR_OUT_OF_MEMORY : SPK_ERR_CUDA, "%s: %s", what,
                   cudaGetErrorString(e));
}

#define DN_TRY(expr, what)                               \
    do {                                                 \
        const cudaError_t _e = (expr);                   \
        if (_e != cudaSuccess) return dn_cuda(dn, _e, what); \
    } while (0)

// BF16 weight copies (and the transposed dgrad copies) from the FP32 master parameters, one launch.
cudaError_t refresh_weights(spk_denoiser *dn) {
    WeightTable T{};
    T.count = static_cast<uint32_t>(dn->layers.size());
    if (T.count > kNumLayers) return cudaErrorInvalidValue;
    unsigned long long total = 0;
    for (uint32_t k = 0; k < T.count; ++k) {
        const Layer &L = dn->layers[k];
        T.cin[k] = L.cin;
        T.cout[k] = L.cout;
        T.w_off[k] = L.w_off;
        T.wb_off[k] = L.wb_off;
        T.first[k] = total;
        total += static_cast<unsigned long long>(L.cout) * 9u * L.cin;
    }
    T.first[T.count] = total;
    k_refresh_weights<<<blocks_for(total, 256), 256, 0, dn->stream>>>(T, dn->params.p, dn->wb.p, dn->wt.p);
    dn->weights_dirty = false;
    return cudaGetLastError();
}

spk_status dn_init(spk_denoiser *dn, uint64_t seed) {
    std::vector<float> host(dn->nparams, 0.f);
    NormalGen g{seed ^ 0x5DEECE66Dull};
    for (const Layer &L : dn->layers) {
        const double std_dev = std::sqrt(2.0 / (9.0 * L.cin));
        const size_t n = static_cast<size_t>(L.cout) * 9 * L.cin;
        for (size_t i = 0; i < n; ++i) host[L.w_off + i] = static_cast<float>(g.normal() * std_dev);
    }
    DN_TRY(cudaMemcpyAsync(dn->params.p, host.data(), dn->nparams * sizeof(float), cudaMemcpyHostToDevice, dn->stream),
           "parameter upload");
    DN_TRY(cudaMemsetAsync(dn->adam_m.p, 0, dn->nparams * sizeof(float), dn->stream), "adam reset");
    DN_TRY(cudaMemsetAsync(dn->adam_v.p, 0, dn->nparams * sizeof(float), dn->stream), "adam reset");
    dn->adam_t = 0;
    DN_TRY(refresh_weights(dn), "weight conversion");
    DN_TRY(cudaStreamSynchronize(dn->stream), "synchronize");
    return SPK_OK;
}

// Allocates the activations (and, for training, the gradients) of a batch of level-0 size n x hp x wp.
cudaError_t ensure_buffers(spk_denoiser *dn, uint32_t n, uint32_t hp, uint32_t wp, bool training) {
    auto P = [&](uint32_t l) { return static_cast<size_t>(n) * (hp >> l) * (wp >> l); };
    cudaError_t e;
    if ((e = dn->x0.ensure(P(0) * kInPad)) != cudaSuccess || (e = dn->out.ensure(P(0) * kOutPad)) != cudaSuccess ||
        (e = dn->eb4.ensure(P(4) * kW[4])) != cudaSuccess)
        return e;
    for (uint32_t l = 0; l < kLevels; ++l)
        if ((e = dn->ea[l].ensure(P(l) * kW[l])) != cudaSuccess) return e;
    for (uint32_t l = 0; l < 4; ++l) {
        if ((e = dn->cat[l].ensure(P(l) * cat_channels(l))) != cudaSuccess ||
            (e = dn->pool[l].ensure(P(l + 1) * kW[l])) != cudaSuccess ||
            (e = dn->da[l].ensure(P(l) * kW[l])) != cudaSuccess || (e = dn->db[l].ensure(P(l) * kW[l])) != cudaSuccess)
            return e;
    }
    if (!training) return cudaSuccess;
    if ((e = dn->gout.ensure(P(0) * kOutPad)) != cudaSuccess) return e;
    for (uint32_t l = 0; l < kLevels; ++l)
        if ((e = dn->g_ea[l].ensure(P(l) * kW[l])) != cudaSuccess ||
            (e = dn->g_eb[l].ensure(P(l) * kW[l])) != cudaSuccess)
            return e;
    for (uint32_t l = 0; l < 4; ++l)
        if ((e = dn->g_cat[l].ensure(P(l) * cat_channels(l))) != cudaSuccess ||
            (e = dn->g_pool[l].ensure(P(l + 1) * kW[l])) != cudaSuccess ||
            (e = dn->g_da[l].ensure(P(l) * kW[l])) != cudaSuccess ||
            (e = dn->g_db[l].ensure(P(l) * kW[l])) != cudaSuccess)
            return e;
    return cudaSuccess;
}

NhwcView view(bf16 *p, uint32_t channels, uint32_t ld) { return NhwcView{p, channels, ld}; }
NhwcView dense(bf16 *p, uint32_t channels) { return NhwcView{p, channels, channels}; }

// Encoder output of level l: inside cat[l] for l < 4, eb4 at the bottom.
NhwcView enc_out(spk_denoiser *dn, uint32_t l) {
    if (l == 4) return dense(dn->eb4.p, kW[4]);
    return view(dn->cat[l].p + kW[l + 1], kW[l], cat_channels(l));
}

// Forward of layer li; with `pool`, the epilogue also writes the 2x2 average pooling of the output there.
cudaError_t conv_fwd(spk_denoiser *dn, uint32_t li, const NhwcView &x, const NhwcView &y, const ConvGeom &g,
                     bf16 *pool = nullptr) {
    const Layer &L = dn->layers[li];
    ConvEpilogue epi;
    epi.bias = dn->params.p + L.b_off;
    epi.relu = L.relu;
    epi.pool = pool;
    return conv3x3_forward(x, dn->wb.p + L.wb_off, L.cout, y, g, epi, dn->err.p, dn->stream);
}

// Input gradient of layer li: dx = conv(dy, wt), optionally times (mask > 0).
cudaError_t conv_dgrad(spk_denoiser *dn, uint32_t li, const NhwcView &dy, const NhwcView &dx, const ConvGeom &g,
                       const NhwcView *mask) {
    const Layer &L = dn->layers[li];
    ConvEpilogue epi;
    if (mask) epi.mask = *mask;
    return conv3x3_forward(dy, dn->wt.p + L.wb_off, L.cin, dx, g, epi, dn->err.p, dn->stream);
}

cudaError_t layer_grads(spk_denoiser *dn, uint32_t li, const NhwcView &x, const NhwcView &dy, const ConvGeom &g) {
    const Layer &L = dn->layers[li];
    cudaError_t e = conv3x3_wgrad(x, dy, dn->grads.p + L.w_off, g, dn->err.p, dn->stream);
    if (e != cudaSuccess) return e;
    const size_t npix = static_cast<size_t>(g.n) * g.h * g.w;
    k_bias_grad<<<std::min<unsigned>(blocks_for(npix, 8), 1024), 256, 0, dn->stream>>>(
        static_cast<const bf16 *>(dy.ptr), npix, dy.channels, dn->grads.p + L.b_off);
    return cudaGetLastError();
}

cudaError_t forward(spk_denoiser *dn, const float *feat, uint32_t n, uint32_t h, uint32_t w, uint32_t hp,
                    uint32_t wp) {
    cudaError_t e;
    const size_t p0 = static_cast<size_t>(n) * hp * wp;
    k_input<<<blocks_for(p0 * (kInPad / 8u), 256), 256, 0, dn->stream>>>(feat, dn->x0.p, n, h, w, hp, wp);
    auto G = [&](uint32_t l) { return ConvGeom{n, hp >> l, wp >> l}; };
    NhwcView in = dense(dn->x0.p, kInPad);
    for (uint32_t l = 0; l < kLevels; ++l) {
        if ((e = conv_fwd(dn, enc_a(l), in, dense(dn->ea[l].p, kW[l]), G(l))) != cudaSuccess) return e;
        const NhwcView eo = enc_out(dn, l);
        // the encoder's second conv also writes the 2x2 average pooling of its output (the next level's input)
        if ((e = conv_fwd(dn, enc_b(l), dense(dn->ea[l].p, kW[l]), eo, G(l), l < 4 ? dn->pool[l].p : nullptr)) !=
            cudaSuccess)
            return e;
        if (l < 4) in = dense(dn->pool[l].p, kW[l]);
    }
    NhwcView up = dense(dn->eb4.p, kW[4]);
    for (int l = 3; l >= 0; --l) {
        const ConvGeom c = G(l + 1);
        const size_t work = static_cast<size_t>(n) * 4 * c.h * c.w * (up.channels / 8);
        k_upsample<<<blocks_for(work, 256), 256, 0, dn->stream>>>(static_cast<const bf16 *>(up.ptr), dn->cat[l].p,
                                                                   cat_channels(l), n, c.h, c.w, up.channels);
        if ((e = conv_fwd(dn, dec_a(l), dense(dn->cat[l].p, cat_channels(l)), dense(dn->da[l].p, kW[l]), G(l))) !=
                cudaSuccess ||
            (e = conv_fwd(dn, dec_b(l), dense(dn->da[l].p, kW[l]), dense(dn->db[l].p, kW[l]), G(l))) != cudaSuccess)
            return e;
        up = dense(dn->db[l].p, kW[l]);
    }
    if ((e = conv_fwd(dn, kOutLayer, dense(dn->db[0].p, kW[0]), dense(dn->out.p, kOutPad), G(0))) != cudaSuccess)
        return e;
    return cudaGetLastError();
}

cudaError_t backward(spk_denoiser *dn, uint32_t n, uint32_t hp, uint32_t wp) {
    cudaError_t e;
    auto G = [&](uint32_t l) { return ConvGeom{n, hp >> l, wp >> l}; };
    // output layer
    const NhwcView db0 = dense(dn->db[0].p, kW[0]);
    if ((e = layer_grads(dn, kOutLayer, db0, dense(dn->gout.p, kOutPad), G(0))) != cudaSuccess) return e;
    if ((e = conv_dgrad(dn, kOutLayer, dense(dn->gout.p, kOutPad), dense(dn->g_db[0].p, kW[0]), G(0), &db0)) !=
        cudaSuccess)
        return e;
    // decoder, level 0 upwards
    for (uint32_t l = 0; l < 4; ++l) {
        const NhwcView da = dense(dn->da[l].p, kW[l]);
        const NhwcView gdb = dense(dn->g_db[l].p, kW[l]), gda = dense(dn->g_da[l].p, kW[l]);
        const NhwcView cat = dense(dn->cat[l].p, cat_channels(l)), gcat = dense(dn->g_cat[l].p, cat_channels(l));
        if ((e = layer_grads(dn, dec_b(l), da, gdb, G(l))) != cudaSuccess ||
            (e = conv_dgrad(dn, dec_b(l), gdb, gda, G(l), &da)) != cudaSuccess ||
            (e = layer_grads(dn, dec_a(l), cat, gda, G(l))) != cudaSuccess ||
            (e = conv_dgrad(dn, dec_a(l), gda, gcat, G(l), nullptr)) != cudaSuccess)
            return e;
        // gradient of the upsampled input -> the level below's decoder output (or the bottleneck)
        const ConvGeom c = G(l + 1);
        const uint32_t cu = kW[l + 1];
        const bf16 *ref = l < 3 ? dn->db[l + 1].p : dn->eb4.p;
        bf16 *dst = l < 3 ? dn->g_db[l + 1].p : dn->g_eb[4].p;
        const size_t work = static_cast<size_t>(n) * c.h * c.w * cu;
        k_upsample_bwd<<<blocks_for(work, 256), 256, 0, dn->stream>>>(dn->g_cat[l].p, cat_channels(l), ref, cu, dst, n,
                                                                       c.h, c.w, cu);
    }
    // encoder, bottom up
    for (int l = 4; l >= 0; --l) {
        const NhwcView ea = dense(dn->ea[l].p, kW[l]);
        const NhwcView geb = dense(dn->g_eb[l].p, kW[l]), gea = dense(dn->g_ea[l].p, kW[l]);
        if ((e = layer_grads(dn, enc_b(l), ea, geb, G(l))) != cudaSuccess ||
            (e = conv_dgrad(dn, enc_b(l), geb, gea, G(l), &ea)) != cudaSuccess)
            return e;
        const NhwcView in = l == 0 ? dense(dn->x0.p, kInPad) : dense(dn->pool[l - 1].p, kW[l - 1]);
        if ((e = layer_grads(dn, enc_a(l), in, gea, G(l))) != cudaSuccess) return e;
        if (l == 0) break;
        const NhwcView gpool = dense(dn->g_pool[l - 1].p, kW[l - 1]);
        if ((e = conv_dgrad(dn, enc_a(l), gea, gpool, G(l), nullptr)) != cudaSuccess) return e;
        // gradient at the level above's encoder output: pooling backward + skip gradient, ReLU mask
        const ConvGeom f = G(l - 1);
        const uint32_t cf = kW[l - 1];
        const NhwcView eo = enc_out(dn, l - 1);
        const size_t work = static_cast<size_t>(n) * f.h * f.w * cf;
        k_pool_bwd<<<blocks_for(work, 256), 256, 0, dn->stream>>>(dn->g_pool[l - 1].p, dn->g_cat[l - 1].p + kW[l],
                                                                   cat_channels(l - 1), static_cast<const bf16 *>(eo.ptr),
                                                                   eo.ld, dn->g_eb[l - 1].p, n, f.h, f.w, cf);
    }
    return cudaGetLastError();
}

spk_status check_errors(spk_denoiser *dn) {
    uint32_t err = 0;
    DN_TRY(cudaMemcpyAsync(&err, dn->err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, dn->stream), "error read");
    DN_TRY(cudaStreamSynchronize(dn->stream), "synchronize");
    if (err) {
        cudaMemsetAsync(dn->err.p, 0, sizeof(uint32_t), dn->stream);
        return dn_fail(dn, SPK_ERR_DEVICE_LIMIT, "tensor-core kernel error bits 0x%x", err);
    }
    return SPK_OK;
}

spk_status loss_and_grads(spk_denoiser *dn, const float *feat, const float *target, uint32_t n, uint32_t h,
                          uint32_t w, float *loss) {
    if (!feat || !target || n == 0 || h == 0 || w == 0 || h % SPK_DN_ALIGN || w % SPK_DN_ALIGN)
        return dn_fail(dn, SPK_ERR_INVALID_ARGUMENT, "batch sides must be non-zero multiples of %u", SPK_DN_ALIGN);
    DN_TRY(ensure_buffers(dn, n, h, w, true), "activation buffers");
    if (dn->weights_dirty) DN_TRY(refresh_weights(dn), "weight conversion");
    DN_TRY(cudaMemsetAsync(dn->grads.p, 0, dn->nparams * sizeof(float), dn->stream), "gradient reset");
    DN_TRY(cudaMemsetAsync(dn->loss.p, 0, sizeof(double), dn->stream), "loss reset");
    DN_TRY(cudaEventRecord(dn->ev0, dn->stream), "event");
    DN_TRY(forward(dn, feat, n, h, w, h, w), "forward");
    const size_t p0 = static_cast<size_t>(n) * h * w;
    k_loss<<<blocks_for(p0, 256), 256, 0, dn->stream>>>(dn->out.p, target, dn->gout.p, n, h, w, dn->loss.p);
    DN_TRY(backward(dn, n, h, w), "backward");
    double l = 0.0;
    DN_TRY(cudaMemcpyAsync(&l, dn->loss.p, sizeof(double), cudaMemcpyDeviceToHost, dn->stream), "loss read");
    const spk_status st = check_errors(dn);
    if (st != SPK_OK) return st;
    if (loss) *loss = static_cast<float>(l / (3.0 * static_cast<double>(p0)));
    return SPK_OK;
}

}  // namespace

extern "C" {

spk_status spk_dn_create(int32_t device, uint64_t seed, spk_denoiser **out) {
    if (!out) return SPK_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return SPK_ERR_CUDA;
    if (device < 0 || device >= count) return SPK_ERR_INVALID_ARGUMENT;
    auto *dn = new (std::nothrow) spk_denoiser();
    if (!dn) return SPK_ERR_OUT_OF_MEMORY;
    dn->device = device;
    dn->layers = make_layers();
    dn->nparams = param_count(dn->layers);
    dn->nweights = weight_count(dn->layers);
    cudaError_t e;
    if ((e = cudaSetDevice(device)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&dn->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreate(&dn->ev0)) != cudaSuccess || (e = cudaEventCreate(&dn->ev1)) != cudaSuccess ||
        (e = dn->params.ensure(dn->nparams)) != cudaSuccess || (e = dn->grads.ensure(dn->nparams)) != cudaSuccess ||
        (e = dn->adam_m.ensure(dn->nparams)) != cudaSuccess || (e = dn->adam_v.ensure(dn->nparams)) != cudaSuccess ||
        (e = dn->wb.ensure(dn->nweights)) != cudaSuccess || (e = dn->wt.ensure(dn->nweights)) != cudaSuccess ||
        (e = dn->err.ensure(1)) != cudaSuccess || (e = dn->loss.ensure(1)) != cudaSuccess ||
        (e = cudaMemset(dn->err.p, 0, sizeof(uint32_t))) != cudaSuccess) {
        spk_dn_destroy(dn);
        return e == cudaErrorMemoryAllocation ? SPK_ERR_OUT_OF_MEMORY : SPK_ERR_CUDA;
    }
    if (dn_init(dn, seed) != SPK_OK) {
        spk_dn_destroy(dn);
        return SPK_ERR_CUDA;
    }
    *out = dn;
    return SPK_OK;
}

spk_status spk_dn_destroy(spk_denoiser *dn) {
    if (!dn) return SPK_OK;
    cudaSetDevice(dn->device);
    if (dn->stream) cudaStreamSynchronize(dn->stream);
    DBuf<float> *fb[] = {&dn->params, &dn->grads, &dn->adam_m, &dn->adam_v, &dn->frame};
    for (auto *b : fb) b->release();
    DBuf<bf16> *bb[] = {&dn->wb, &dn->wt, &dn->x0, &dn->out, &dn->gout, &dn->eb4, &dn->conv_wt_scratch};
    for (auto *b : bb) b->release();
    for (uint32_t l = 0; l < kLevels; ++l) {
        dn->ea[l].release();
        dn->g_ea[l].release();
        dn->g_eb[l].release();
    }
    for (uint32_t l = 0; l < 4; ++l) {
        DBuf<bf16> *lb[] = {&dn->cat[l], &dn->pool[l], &dn->da[l], &dn->db[l],
                            &dn->g_cat[l], &dn->g_pool[l], &dn->g_da[l], &dn->g_db[l]};
        for (auto *b : lb) b->release();
    }
    dn->err.release();
    dn->loss.release();
    if (dn->ev0) cudaEventDestroy(dn->ev0);
    if (dn->ev1) cudaEventDestroy(dn->ev1);
    if (dn->stream) cudaStreamDestroy(dn->stream);
    delete dn;
    return SPK_OK;
}

const char *spk_dn_last_error(const spk_denoiser *dn) { return dn ? dn->error.c_str() : "null denoiser"; }

spk_status spk_dn_init(spk_denoiser *dn, uint64_t seed) {
    if (!dn) return SPK_ERR_INVALID_ARGUMENT;
    cudaSetDevice(dn->device);
    return dn_init(dn, seed);
}

spk_status spk_dn_num_params(const spk_denoiser *dn, uint64_t *count) {
    if (!dn || !count) return SPK_ERR_INVALID_ARGUMENT;
    *count = dn->nparams;
    return SPK_OK;
}

spk_status spk_dn_get_params(spk_denoiser *dn, float *host, uint64_t count) {
    if (!dn || !host) return SPK_ERR_INVALID_ARGUMENT;
    if (count != dn->nparams) return dn_fail(dn, SPK_ERR_INVALID_ARGUMENT, "expected %zu parameters", dn->nparams);
    cudaSetDevice(dn->device);
    DN_TRY(cudaMemcpyAsync(host, dn->params.p, count * sizeof(float), cudaMemcpyDeviceToHost, dn->stream), "read");
    DN_TRY(cudaStreamSynchronize(dn->stream), "synchronize");
    return SPK_OK;
}

spk_status spk_dn_set_params(spk_denoiser *dn, const float *host, uint64_t count) {
    if (!dn || !host) return SPK_ERR_INVALID_ARGUMENT;
    if (count != dn->nparams) return dn_fail(dn, SPK_ERR_INVALID_ARGUMENT, "expected %zu parameters", dn->nparams);
    cudaSetDevice(dn->device);
    DN_TRY(cudaMemcpyAsync(dn->params.p, host, count * sizeof(float), cudaMemcpyHostToDevice, dn->stream), "write");
    DN_TRY(refresh_weights(dn), "weight conversion");
    DN_TRY(cudaStreamSynchronize(dn->stream), "synchronize");
    return SPK_OK;
}

namespace {
struct DnStateHeader {
    char magic[8];
    uint32_t version, reserved;
    uint64_t nparams, adam_t;
};
constexpr char kDnStateMagic[8] = {'S', 'P', 'K', 'D', 'N', 'S', 'T', '1'};
}  // namespace

spk_status spk_dn_state_size(const spk_denoiser *dn, uint64_t *bytes) {
    if (!dn || !bytes) return SPK_ERR_INVALID_ARGUMENT;
    *bytes = sizeof(DnStateHeader) + 3ull * dn->nparams * sizeof(float);
    return SPK_OK;
}

spk_status spk_dn_save_state(spk_denoiser *dn, void *host, uint64_t size) {
    if (!dn || !host) return SPK_ERR_INVALID_ARGUMENT;
    const uint64_t nb = dn->nparams * sizeof(float);
    if (size < sizeof(DnStateHeader) + 3 * nb) return dn_fail(dn, SPK_ERR_INVALID_ARGUMENT, "state buffer too small");
    cudaSetDevice(dn->device);
    DnStateHeader h{};
    std::memcpy(h.magic, kDnStateMagic, 8);
    h.version = 1;
    h.nparams = dn->nparams;
    h.adam_t = dn->adam_t;
    auto *out = static_cast<uint8_t *>(host);
    std::memcpy(out, &h, sizeof(h));
    out += sizeof(h);
    DN_TRY(cudaMemcpyAsync(out, dn->params.p, nb, cudaMemcpyDeviceToHost, dn->stream), "state read");
    DN_TRY(cudaMemcpyAsync(out + nb, dn->adam_m.p, nb, cudaMemcpyDeviceToHost, dn->stream), "state read");
    DN_TRY(cudaMemcpyAsync(out + 2 * nb, dn->adam_v.p, nb, cudaMemcpyDeviceToHost, dn->stream), "state read");
    DN_TRY(cudaStreamSynchronize(dn->stream), "synchronize");
    return SPK_OK;
}

spk_status spk_dn_load_state(spk_denoiser *dn, const void *host, uint64_t size) {
    if (!dn || !host) return SPK_ERR_INVALID_ARGUMENT;
    DnStateHeader h{};
    if (size < sizeof(h)) return dn_fail(dn, SPK_ERR_INVALID_ARGUMENT, "state truncated");
    std::memcpy(&h, host, sizeof(h));
    if (std::memcmp(h.magic, kDnStateMagic, 8) != 0 || h.version != 1)
        return dn_fail(dn, SPK_ERR_INVALID_ARGUMENT, "not a denoiser training state of this version");
    if (h.nparams != dn->nparams) return dn_fail(dn, SPK_ERR_INVALID_ARGUMENT, "state holds another network size");
    const uint64_t nb = dn->nparams * sizeof(float);
    if (size < sizeof(h) + 3 * nb) return dn_fail(dn, SPK_ERR_INVALID_ARGUMENT, "state truncated");
    cudaSetDevice(dn->device);
    const auto *in = static_cast<const uint8_t *>(host) + sizeof(h);
    DN_TRY(cudaMemcpyAsync(dn->params.p, in, nb, cudaMemcpyHostToDevice, dn->stream), "state write");
    DN_TRY(cudaMemcpyAsync(dn->adam_m.p, in + nb, nb, cudaMemcpyHostToDevice, dn->stream), "state write");
    DN_TRY(cudaMemcpyAsync(dn->adam_v.p, in + 2 * nb, nb, cudaMemcpyHostToDevice, dn->stream), "state write");
    DN_TRY(refresh_weights(dn), "weight conversion");
    DN_TRY(cudaStreamSynchronize(dn->stream), "synchronize");
    dn->adam_t = h.adam_t;
    return SPK_OK;
}

spk_status spk_render_denoised(spk_ctx *ctx, spk_denoiser *dn, uint32_t spp, uint32_t tile, float threshold,
                               float *denoised_rgba, uint32_t *fallback_tiles) try {
    if (!ctx || !dn || !denoised_rgba || spp == 0 || tile == 0) return SPK_ERR_INVALID_ARGUMENT;
    const DnRange range("spk_render_denoised");
    spk_config cfg{};
    spk_status st = spk_get_config(ctx, &cfg);
    if (st != SPK_OK) return st;
    const uint32_t w = cfg.width, h = cfg.height;
    const size_t px = static_cast<size_t>(w) * h;
    cudaSetDevice(dn->device);
    // scratch: half A, three feature sets, three denoised images, the output
    DN_TRY(dn->frame.ensure(px * (4 + 3 * SPK_DN_FEATURES + 3 * 4 + 4)), "frame scratch");
    float *half_a = dn->frame.p, *feat = half_a + 4 * px, *feat_a = feat + SPK_DN_FEATURES * px,
          *feat_b = feat_a + SPK_DN_FEATURES * px, *den = feat_b + SPK_DN_FEATURES * px, *den_a = den + 4 * px,
          *den_b = den_a + 4 * px, *out = den_b + 4 * px;
    void *fb = nullptr, *img = nullptr, *nd = nullptr, *alb = nullptr;
    const uint32_t half = spp / 2;
    if (half >= 1) {
        if ((st = spk_render(ctx, half)) != SPK_OK || (st = spk_synchronize(ctx)) != SPK_OK ||
            (st = spk_framebuffer_device(ctx, &fb, &img)) != SPK_OK)
            return dn_fail(dn, st, "render (first half): %s", spk_last_error(ctx));
        DN_TRY(cudaMemcpyAsync(half_a, fb, px * 4 * sizeof(float), cudaMemcpyDeviceToDevice, dn->stream), "half copy");
        DN_TRY(cudaStreamSynchronize(dn->stream), "synchronize");
    }
    if ((st = spk_render(ctx, spp - half)) != SPK_OK || (st = spk_render_guides(ctx)) != SPK_OK ||
        (st = spk_synchronize(ctx)) != SPK_OK || (st = spk_framebuffer_device(ctx, &fb, &img)) != SPK_OK ||
        (st = spk_guides_device(ctx, &nd, &alb)) != SPK_OK)
        return dn_fail(dn, st, "render: %s", spk_last_error(ctx));
    const auto *ffb = static_cast<const float *>(fb), *fnd = static_cast<const float *>(nd),
               *falb = static_cast<const float *>(alb);
    // The mean and the two halves are consecutive images of one feature batch (feat, feat_a, feat_b) and
    // come out as consecutive images (den, den_a, den_b): one inference of three images, whose coarse
    // levels then give the GPU three times the tiles. Each image's result is the same as alone.
    if ((st = spk_dn_pack_features(dn, ffb, fnd, falb, 1, h, w, feat)) != SPK_OK) return st;
    if (half >= 1 && (st = spk_dn_pack_halves(dn, ffb, half_a, fnd, falb, 1, h, w, feat_a, feat_b)) != SPK_OK)
        return st;
    if ((st = spk_dn_infer(dn, feat, half >= 1 ? 3u : 1u, h, w, den)) != SPK_OK) return st;
    uint32_t tiles = 0;
    const float *result = den;
    if (half >= 1) {
        if ((st = spk_dn_fallback(dn, den, den_a, den_b, ffb, h, w, tile, threshold, out, &tiles)) != SPK_OK)
            return st;
        result = out;
    }
    DN_TRY(cudaMemcpyAsync(denoised_rgba, result, px * 4 * sizeof(float), cudaMemcpyDefault, dn->stream), "output");
    DN_TRY(cudaStreamSynchronize(dn->stream), "synchronize");
    if (fallback_tiles) *fallback_tiles = tiles;
    return SPK_OK;
} catch (const std::bad_alloc &) {
    return dn_fail(dn, SPK_ERR_OUT_OF_MEMORY, "host memory exhausted");
}

spk_status spk_dn_debug_wait_timeout(spk_denoiser *dn) {
    if (!dn) return SPK_ERR_INVALID_ARGUMENT;
    cudaSetDevice(dn->device);
    DN_TRY(conv_wait_probe(dn->err.p, dn->stream), "wait probe");
    return check_errors(dn);
}

spk_status spk_dn_pack_features(spk_denoiser *dn, const float *d_hdr, const float *d_nd, const float *d_alb,
                                uint32_t n, uint32_t h, uint32_t w, float *d_features) {
    if (!dn || !d_hdr || !d_nd || !d_alb || !d_features) return SPK_ERR_INVALID_ARGUMENT;
    cudaSetDevice(dn->device);
    const size_t total = static_cast<size_t>(n) * h * w;
    if (total == 0) return SPK_OK;
    k_pack_features<<<blocks_for(total, 256), 256, 0, dn->stream>>>(reinterpret_cast<const float4 *>(d_hdr),
                                                                      reinterpret_cast<const float4 *>(d_nd),
                                                                      reinterpret_cast<const float4 *>(d_alb),
                                                                      d_features, total);
    DN_TRY(cudaGetLastError(), "feature packing");
    return SPK_OK;
}

spk_status spk_dn_pack_halves(spk_denoiser *dn, const float *d_full, const float *d_half_a, const float *d_nd,
                              const float *d_alb, uint32_t n, uint32_t h, uint32_t w, float *d_feat_a,
                              float *d_feat_b) {
    if (!dn || !d_full || !d_half_a || !d_nd || !d_alb || !d_feat_a || !d_feat_b) return SPK_ERR_INVALID_ARGUMENT;
    cudaSetDevice(dn->device);
    const size_t total = static_cast<size_t>(n) * h * w;
    if (total == 0) return SPK_OK;
    k_pack_halves<<<blocks_for(total, 256), 256, 0, dn->stream>>>(
        reinterpret_cast<const float4 *>(d_full), reinterpret_cast<const float4 *>(d_half_a),
        reinterpret_cast<const float4 *>(d_nd), reinterpret_cast<const float4 *>(d_alb), d_feat_a, d_feat_b, total);
    DN_TRY(cudaGetLastError(), "half feature packing");
    return SPK_OK;
}

spk_status spk_dn_gradients(spk_denoiser *dn, const float *d_features, const float *d_target, uint32_t n, uint32_t h,
                            uint32_t w, float *loss, float *host_grad, uint64_t count) {
    if (!dn) return SPK_ERR_INVALID_ARGUMENT;
    if (host_grad && count != dn->nparams)
        return dn_fail(dn, SPK_ERR_INVALID_ARGUMENT, "expected %zu gradient entries", dn->nparams);
    cudaSetDevice(dn->device);
    const spk_status st = loss_and_grads(dn, d_features, d_target, n, h, w, loss);
    if (st != SPK_OK) return st;
    if (host_grad) {
        DN_TRY(cudaMemcpyAsync(host_grad, dn->grads.p, count * sizeof(float), cudaMemcpyDeviceToHost, dn->stream),
               "gradient read");
        DN_TRY(cudaStreamSynchronize(dn->stream), "synchronize");
    }
    return SPK_OK;
}

spk_status spk_dn_train_step(spk_denoiser *dn, const float *d_features, const float *d_target, uint32_t n, uint32_t h,
                             uint32_t w, float lr, float *loss) {
    const DnRange range("spk_dn_train_step");
    if (!dn) return SPK_ERR_INVALID_ARGUMENT;
    if (!(lr > 0.f)) return dn_fail(dn, SPK_ERR_INVALID_ARGUMENT, "learning rate must be positive");
    cudaSetDevice(dn->device);
    spk_status st = loss_and_grads(dn, d_features, d_target, n, h, w, loss);
    if (st != SPK_OK) return st;
    ++dn->adam_t;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.f - static_cast<float>(std::pow(b1, static_cast<double>(dn->adam_t)));
    const float bc2 = 1.f - static_cast<float>(std::pow(b2, static_cast<double>(dn->adam_t)));
    k_adam<<<blocks_for(dn->nparams, 256), 256, 0, dn->stream>>>(dn->params.p, dn->grads.p, dn->adam_m.p, dn->adam_v.p,
                                                                  dn->nparams, lr, b1, b2, 1e-8f, bc1, bc2);
    DN_TRY(cudaGetLastError(), "adam");
    DN_TRY(refresh_weights(dn), "weight conversion");
    DN_TRY(cudaEventRecord(dn->ev1, dn->stream), "event");
    return SPK_OK;
}

spk_status spk_dn_infer(spk_denoiser *dn, const float *d_features, uint32_t n, uint32_t h, uint32_t w, float *d_out) {
    const DnRange range("spk_dn_infer");
    if (!dn || !d_features || !d_out || n == 0 || h == 0 || w == 0) return SPK_ERR_INVALID_ARGUMENT;
    cudaSetDevice(dn->device);
    const uint32_t hp = (h + SPK_DN_ALIGN - 1) / SPK_DN_ALIGN * SPK_DN_ALIGN;
    const uint32_t wp = (w + SPK_DN_ALIGN - 1) / SPK_DN_ALIGN * SPK_DN_ALIGN;
    DN_TRY(ensure_buffers(dn, n, hp, wp, false), "activation buffers");
    if (dn->weights_dirty) DN_TRY(refresh_weights(dn), "weight conversion");
    DN_TRY(cudaEventRecord(dn->ev0, dn->stream), "event");
    DN_TRY(forward(dn, d_features, n, h, w, hp, wp), "forward");
    const size_t total = static_cast<size_t>(n) * h * w;
    k_decode<<<blocks_for(total, 256), 256, 0, dn->stream>>>(dn->out.p, reinterpret_cast<float4 *>(d_out), n, h, w, hp,
                                                              wp);
    DN_TRY(cudaGetLastError(), "decode");
    DN_TRY(cudaEventRecord(dn->ev1, dn->stream), "event");
    return SPK_OK;
}

spk_status spk_dn_fallback(spk_denoiser *dn, const float *d_denoised, const float *d_den_a, const float *d_den_b,
                           const float *d_plain, uint32_t h, uint32_t w, uint32_t tile, float threshold, float *d_out,
                           uint32_t *fallback_tiles) {
    if (!dn || !d_denoised || !d_den_a || !d_den_b || !d_plain || !d_out || tile == 0 || h == 0 || w == 0)
        return SPK_ERR_INVALID_ARGUMENT;
    cudaSetDevice(dn->device);
    DN_TRY(dn->err.ensure(1), "scratch");
    unsigned int *count = nullptr;
    DN_TRY(cudaMallocAsync(reinterpret_cast<void **>(&count), sizeof(unsigned int), dn->stream), "scratch");
    DN_TRY(cudaMemsetAsync(count, 0, sizeof(unsigned int), dn->stream), "scratch");
    const uint32_t tiles = ((w + tile - 1) / tile) * ((h + tile - 1) / tile);
    k_fallback<<<tiles, 256, 0, dn->stream>>>(reinterpret_cast<const float4 *>(d_denoised),
                                              reinterpret_cast<const float4 *>(d_den_a),
                                              reinterpret_cast<const float4 *>(d_den_b),
                                              reinterpret_cast<const float4 *>(d_plain), reinterpret_cast<float4 *>(d_out),
                                              h, w, tile, threshold, count);
    unsigned int c = 0;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&c, count, sizeof(unsigned int), cudaMemcpyDeviceToHost, dn->stream);
    cudaFreeAsync(count, dn->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(dn->stream);
    if (e != cudaSuccess) return dn_cuda(dn, e, "fallback");
    if (fallback_tiles) *fallback_tiles = c;
    return SPK_OK;
}

spk_status spk_dn_synchronize(spk_denoiser *dn) {
    if (!dn) return SPK_ERR_INVALID_ARGUMENT;
    cudaSetDevice(dn->device);
    DN_TRY(cudaStreamSynchronize(dn->stream), "synchronize");
    return SPK_OK;
}

spk_status spk_dn_last_ms(spk_denoiser *dn, float *ms) {
    if (!dn || !ms) return SPK_ERR_INVALID_ARGUMENT;
    cudaSetDevice(dn->device);
    DN_TRY(cudaEventSynchronize(dn->ev1), "event");
    DN_TRY(cudaEventElapsedTime(ms, dn->ev0, dn->ev1), "event");
    return SPK_OK;
}

spk_status spk_dn_conv3x3(spk_denoiser *dn, int32_t op, const void *d_x, uint32_t x_channels, uint32_t x_ld,
                          const void *d_w, const float *d_bias, void *d_y, uint32_t y_channels, uint32_t y_ld,
                          uint32_t n, uint32_t h, uint32_t w, int32_t relu, const void *d_mask, uint32_t mask_ld,
                          float *d_dw) {
    if (!dn || !d_x || !d_y) return SPK_ERR_INVALID_ARGUMENT;
    cudaSetDevice(dn->device);
    const NhwcView x{const_cast<void *>(d_x), x_channels, x_ld}, y{d_y, y_channels, y_ld};
    const ConvGeom g{n, h, w};
    cudaError_t e;
    if (op == 0 || op == 1) {
        if (!d_w) return SPK_ERR_INVALID_ARGUMENT;
        ConvEpilogue epi;
        epi.bias = d_bias;
        epi.relu = relu != 0;
        if (d_mask) epi.mask = NhwcView{const_cast<void *>(d_mask), y_channels, mask_ld};
        const void *wts = d_w;
        if (op == 1) {  // dgrad: x is the output gradient (cout = x_channels), y the input gradient (cin)
            const size_t nw = static_cast<size_t>(x_channels) * 9 * y_channels;
            DN_TRY(dn->conv_wt_scratch.ensure(nw), "scratch");
            DN_TRY(conv3x3_transpose_weights(d_w, dn->conv_wt_scratch.p, x_channels, y_channels, dn->stream),
                   "transpose");
            wts = dn->conv_wt_scratch.p;
        }
        e = conv3x3_forward(x, wts, y_channels, y, g, epi, dn->err.p, dn->stream);
    } else if (op == 2) {
        if (!d_dw) return SPK_ERR_INVALID_ARGUMENT;
        e = conv3x3_wgrad(x, y, d_dw, g, dn->err.p, dn->stream);
    } else {
        return dn_fail(dn, SPK_ERR_INVALID_ARGUMENT, "unknown conv op %d", op);
    }
    if (e == cudaErrorInvalidValue) return dn_fail(dn, SPK_ERR_INVALID_ARGUMENT, "unsupported conv shape or alignment");
    if (e != cudaSuccess) return dn_cuda(dn, e, "conv3x3");
    return check_errors(dn);
}

}  // extern "C"
