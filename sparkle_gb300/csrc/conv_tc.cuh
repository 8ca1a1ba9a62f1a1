// conv_tc.cuh -- 3x3 convolutions (stride 1, zero padding 1) on NHWC BF16 tensors with FP32 accumulation
// on the tcgen05 tensor cores, the compute of the denoiser's U-Net.
//
//   forward : y[p][co]  = sum_{tap, ci} x[p + tap][ci] * w[co][tap][ci]           (+ bias, ReLU, mask)
//   dgrad   : the forward with the weights transposed and flipped (wt[ci][8 - tap][co])
//   wgrad   : dw[co][tap][ci] += sum_p dy[p][co] * x[p + tap][ci]                  (FP32, atomically)
//
// A tensor view is (base pointer, channels, pixel stride in elements): channel slices of a wider buffer
// (the U-Net's skip concatenations) are views with an offset base. Channels are multiples of 32 and
// pixel strides multiples of 8 elements (16 bytes, the TMA stride rule).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace spk {

struct NhwcView {
    void *ptr = nullptr;  // bf16
    uint32_t channels = 0;
    uint32_t ld = 0;      // elements between consecutive pixels
};

struct ConvGeom {
    uint32_t n = 0, h = 0, w = 0;
};

// Epilogue of the forward kernel: out = mask ? (acc + bias) * (mask > 0) : act(acc + bias).
struct ConvEpilogue {
    const float *bias = nullptr;  // cout floats or null
    bool relu = false;
    NhwcView mask{};              // optional: multiply by (mask > 0) (ReLU backward of the layer below)
    // optional: also write the 2x2 average pooling of the (BF16) output, dense [n][h/2][w/2][cout] (h, w even)
    void *pool = nullptr;
};

// y = conv3x3(x, w) over geometry g. `w` is bf16 [cout][9][cin]. `err` is a device word for error bits.
cudaError_t conv3x3_forward(const NhwcView &x, const void *w, uint32_t cout, const NhwcView &y, const ConvGeom &g,
                            const ConvEpilogue &epi, uint32_t *err, cudaStream_t stream);

// dw (fp32 [cout][9][cin]) += wgrad(dy, x). dw must be zeroed by the caller before the first call.
cudaError_t conv3x3_wgrad(const NhwcView &x, const NhwcView &dy, float *dw, const ConvGeom &g, uint32_t *err,
                          cudaStream_t stream);

// One CTA waits on an mbarrier nothing arrives at; the wait gives up after 1 s and ORs kErrWaitTimeout into
// *err (tests of the bounded-wait failure path).
cudaError_t conv_wait_probe(uint32_t *err, cudaStream_t stream);

// wt[ci][tap][co] = w[co][8 - tap][ci] (bf16), the dgrad weights.
cudaError_t conv3x3_transpose_weights(const void *w, void *wt, uint32_t cout, uint32_t cin, cudaStream_t stream);

}  // namespace spk
