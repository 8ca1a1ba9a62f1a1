// image_io.h -- image output: the reference's screenshot conversion and file encoders.
//
// Sparkle's screenshot path (Renderer::RequestSaveScreenshot / ReadbackFinalOutputIfRequested,
// Renderer.cpp:94-181) reads back the RGBA16F final output, converts it to 8-bit sRGB with
// Image2D::CreateFromRawPixels (ConvertPixelsToRGBA8, Image.cpp:30-67: clamp to [0, 1], pow 0.45 per
// colour channel (utilities::LinearToSrgb, Utilities.h:411-414), lround(x * 255)) and writes a PNG through
// Image2D::WriteToFile (Image.cpp:221-275; HDR images go to Radiance .hdr there). The conversion here is a
// 65,536-entry table indexed by the half's bits, filled with exactly that arithmetic, so the device and the
// host give the same bytes. The encoders are this library's own: PNG (zlib stream of fixed-Huffman deflate
// blocks with LZ77 matches, per-row filter by least absolute residual), Radiance RGBE with run-length
// scanlines, and uncompressed scanline OpenEXR with half channels.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace spk {

// RGBA8 byte of one half-float channel: colour channels (srgb = true) take the pow-0.45 encode, alpha not.
const uint8_t *rgba8_table(bool srgb);  // 65,536 entries

// Converts `pixels` RGBA16F texels to RGBA8 on the host.
void rgba16f_to_rgba8(const uint16_t *rgba16f, uint64_t pixels, uint8_t *rgba8);

// Device conversion: `tables` = the colour table followed by the alpha table (2 x 65,536 bytes, device).
cudaError_t launch_rgba16f_to_rgba8(const ushort4 *in, uint64_t pixels, const uint8_t *tables, uchar4 *out,
                                    cudaStream_t stream);
// Linear frame buffer (bottom row first) to RGBA16F rows top first (round to nearest even).
cudaError_t launch_fb_to_half(const float4 *fb, uint32_t width, uint32_t height, ushort4 *out, cudaStream_t stream);

// Encoders; each returns false (with a message in `err`) when the file cannot be written.
std::vector<uint8_t> encode_png(const uint8_t *rgba8, uint32_t width, uint32_t height);
std::vector<uint8_t> encode_hdr(const float *rgba, uint32_t width, uint32_t height);  // rows top first
std::vector<uint8_t> encode_exr(const uint16_t *rgba16f, uint32_t width, uint32_t height);
bool write_file(const std::string &path, const std::vector<uint8_t> &bytes, std::string &err);

}  // namespace spk
