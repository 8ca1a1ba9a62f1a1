/*
 * spk_denoise.h -- C ABI of the learned denoiser: a 5-level U-Net of 3x3 convolutions trained and run on
 * the tcgen05 tensor cores (BF16 weights and activations, FP32 accumulation), with albedo, normal and
 * depth guides from the primary hit.
 *
 * The reference has no learned denoiser: its cpu pipeline's only denoiser is the spatial fill of
 * CPURenderer::DenoisePass (CPURenderer.cpp:452-526, spatial_denoise cvar), and its GPU pipeline runs NRD
 * on the G-buffer that ray_trace.cs.slang:282-351 writes (WritePrimaryHitGBuffer). These entry points
 * add the learned denoiser beside them; the guides follow WritePrimaryHitGBuffer (spk_render_guides in
 * spk.h).
 *
 * Network (fixed): input features (10) = log1p(HDR rgb) (3), albedo (3), normal (3), depth feature (1),
 * zero-padded to 32 channels. Encoder levels of widths 32, 64, 96, 128, 128, two 3x3 conv + ReLU each,
 * 2x2 average pooling between levels; decoder of nearest 2x upsampling, skip concatenation and two 3x3
 * conv + ReLU per level; a final 3x3 conv to 3 (padded 32) channels predicting log1p(HDR rgb).
 * Loss: relMSE = mean((expm1(o) - t)^2 / (t^2 + 0.01)) over pixels and colour channels. Adam.
 *
 * Conventions as in spk.h: spk_status return codes, never abort, device pointers are the caller's.
 */
#ifndef SPK_DENOISE_H_
#define SPK_DENOISE_H_

#include <stddef.h>
#include <stdint.h>

#include "spk.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct spk_denoiser spk_denoiser;

#define SPK_DN_FEATURES 10u /* log1p rgb, albedo, normal, depth */
#define SPK_DN_ALIGN 16u    /* train_step image sides must be multiples of this (4 poolings) */

/* Creates a denoiser on CUDA device `device` with He-normal weights from `seed`. */
spk_status spk_dn_create(int32_t device, uint64_t seed, spk_denoiser **out);
spk_status spk_dn_destroy(spk_denoiser *dn);
const char *spk_dn_last_error(const spk_denoiser *dn);

/* Re-initialises the weights (He normal from `seed`, zero biases) and clears the Adam state. */
spk_status spk_dn_init(spk_denoiser *dn, uint64_t seed);

/* Number of FP32 parameters (weights [cout][3][3][cin] then bias [cout], layer by layer). */
spk_status spk_dn_num_params(const spk_denoiser *dn, uint64_t *count);
spk_status spk_dn_get_params(spk_denoiser *dn, float *host, uint64_t count);
spk_status spk_dn_set_params(spk_denoiser *dn, const float *host, uint64_t count);

/* Packs denoiser input features (device, n*h*w*10 floats) from device images of n*h*w float4 each:
 * `hdr` (linear radiance, rgb), `normal_depth` (world normal xyz, linear depth w) and `albedo` (rgb). */
spk_status spk_dn_pack_features(spk_denoiser *dn, const float *d_hdr, const float *d_normal_depth,
                                const float *d_albedo, uint32_t n, uint32_t h, uint32_t w, float *d_features);

/* Features of the two sample halves of a render: half A's mean `d_half_a` and half B's mean
 * 2 * d_full - d_half_a (equal halves), into d_feat_a and d_feat_b (n*h*w*10 floats each). */
spk_status spk_dn_pack_halves(spk_denoiser *dn, const float *d_full, const float *d_half_a,
                              const float *d_normal_depth, const float *d_albedo, uint32_t n, uint32_t h,
                              uint32_t w, float *d_feat_a, float *d_feat_b);

/* One Adam step (learning rate `lr`, beta 0.9/0.999, eps 1e-8) on a batch. d_features: n*h*w*10 floats,
 * d_target: n*h*w*3 floats (linear HDR); h and w multiples of SPK_DN_ALIGN. *loss receives the batch
 * relMSE before the update (the call waits for it). */
spk_status spk_dn_train_step(spk_denoiser *dn, const float *d_features, const float *d_target, uint32_t n,
                             uint32_t h, uint32_t w, float lr, float *loss);

/* Same forward and backward as a train step without the update: *loss and the FP32 gradient of every
 * parameter (host, spk_dn_num_params floats, same order as spk_dn_get_params). */
spk_status spk_dn_gradients(spk_denoiser *dn, const float *d_features, const float *d_target, uint32_t n,
                            uint32_t h, uint32_t w, float *loss, float *host_grad, uint64_t count);

/* Inference: d_out receives n*h*w float4 (denoised linear rgb, 1). Any h, w (padded internally to
 * multiples of SPK_DN_ALIGN with edge replication). Asynchronous on the denoiser's stream. */
spk_status spk_dn_infer(spk_denoiser *dn, const float *d_features, uint32_t n, uint32_t h, uint32_t w,
                        float *d_out);

/* Per-tile fallback to the plain path tracer. The samples of a render are split into two halves, each
 * half is denoised on its own (d_den_a, d_den_b), and for each `tile` x `tile` block the half-buffer
 * variance estimate v = mean(((den_a - den_b) / 2)^2) / (mean(denoised)^2 + 1e-4) (over the tile's pixels
 * and colour channels) is compared with `threshold`: where the two denoised halves disagree by more, the
 * network is not trusted and the tile takes `d_plain` (the path-traced mean of all samples) instead of
 * `d_denoised` (the denoised mean). d_out may alias d_denoised. *fallback_tiles receives the count (the
 * call waits for it). All images are h*w float4 rows. */
spk_status spk_dn_fallback(spk_denoiser *dn, const float *d_denoised, const float *d_den_a, const float *d_den_b,
                           const float *d_plain, uint32_t h, uint32_t w, uint32_t tile, float threshold,
                           float *d_out, uint32_t *fallback_tiles);

/* The denoised frame of sparkle_gb300/denoise.py's render_denoised in one call: renders `spp` samples per
 * pixel on `ctx` (camera, config and scene set; the accumulation continues as spk_render's does) in two
 * halves, renders the primary-hit guides, denoises the full mean and, when spp >= 2, each half, and
 * replaces the tiles (tile x tile pixels) whose two denoised halves disagree by more than `threshold` with
 * the plain mean (spk_dn_fallback). `denoised_rgba` (width*height float4, rows bottom up like the frame
 * buffer, host or device) receives the result and *fallback_tiles (may be NULL) the replaced tiles. */
spk_status spk_render_denoised(spk_ctx *ctx, spk_denoiser *dn, uint32_t spp, uint32_t tile, float threshold,
                               float *denoised_rgba, uint32_t *fallback_tiles);

/* Training checkpoint: the FP32 parameters, both Adam moments and the step count (spk_dn_state_size
 * bytes, host buffer), so that training stops and resumes where it was. */
spk_status spk_dn_state_size(const spk_denoiser *dn, uint64_t *bytes);
spk_status spk_dn_save_state(spk_denoiser *dn, void *host, uint64_t size);
spk_status spk_dn_load_state(spk_denoiser *dn, const void *host, uint64_t size);

/* Test hook: one kernel waits on an mbarrier that nothing arrives at. Its bounded wait gives up after 1 s
 * like every tensor-core kernel's; the call returns SPK_ERR_DEVICE_LIMIT with the time-out bit and the
 * denoiser stays usable. */
spk_status spk_dn_debug_wait_timeout(spk_denoiser *dn);

/* Waits for the denoiser's stream. */
spk_status spk_dn_synchronize(spk_denoiser *dn);

/* Device time (CUDA events on the denoiser's stream) of the last spk_dn_infer / spk_dn_train_step, ms. */
spk_status spk_dn_last_ms(spk_denoiser *dn, float *ms);

/* Low-level 3x3 convolution on device BF16 NHWC tensors (used by the tests against the CPU oracle).
 *   op 0 forward: y = conv(x, w) (+ bias) (ReLU if relu) (* (mask > 0) if mask);
 *   op 1 dgrad:   y = conv(x, flip(w)^T), i.e. the input gradient for output gradient x of a conv with w;
 *   op 2 wgrad:   dw (FP32 [cout][9][cin], device) += sum_p x2[p + tap] (x) y[p], with x2 = `x` the
 *                 layer input and `y` the output gradient.
 * Channels: multiples of 32; ld: elements between pixels, multiples of 8. w: BF16 [cout][9][cin]. */
spk_status spk_dn_conv3x3(spk_denoiser *dn, int32_t op, const void *d_x, uint32_t x_channels, uint32_t x_ld,
                          const void *d_w, const float *d_bias, void *d_y, uint32_t y_channels, uint32_t y_ld,
                          uint32_t n, uint32_t h, uint32_t w, int32_t relu, const void *d_mask, uint32_t mask_ld,
                          float *d_dw);

#ifdef __cplusplus
}
#endif

#endif /* SPK_DENOISE_H_ */
