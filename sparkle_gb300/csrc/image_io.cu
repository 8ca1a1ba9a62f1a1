// image_io.cu -- screenshot conversion tables and kernels, PNG / Radiance HDR / OpenEXR encoders.
#include "image_io.h"

#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

namespace spk {
namespace {

// IEEE binary16 -> binary32 (exact).
float half_to_float(uint16_t h) {
    const uint32_t sign = static_cast<uint32_t>(h & 0x8000u) << 16;
    const uint32_t exp = (h >> 10) & 0x1Fu, man = h & 0x3FFu;
    uint32_t bits;
    if (exp == 0) {
        if (man == 0) {
            bits = sign;
        } else {  // subnormal: normalise
            int e = -1;
            uint32_t m = man;
            do {
                ++e;
                m <<= 1;
            } while ((m & 0x400u) == 0);
            bits = sign | ((127 - 15 - e) << 23) | ((m & 0x3FFu) << 13);
        }
    } else if (exp == 31) {
        bits = sign | 0x7F800000u | (man << 13);
    } else {
        bits = sign | ((exp + 127 - 15) << 23) | (man << 13);
    }
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}

// FloatToUint8 (Image.cpp:31-34): lround(clamp(v, 0, 1) * 255); a NaN gives 0.
uint8_t float_to_u8(float v) {
    if (std::isnan(v)) return 0;
    return static_cast<uint8_t>(std::lround(std::clamp(v, 0.f, 1.f) * 255.f));
}

struct Tables {
    uint8_t colour[65536], alpha[65536];
    Tables() {
        for (uint32_t h = 0; h < 65536; ++h) {
            const float v = half_to_float(static_cast<uint16_t>(h));
            // rgb.cwiseMax(0).cwiseMin(1), LinearToSrgb = pow(x, 0.45f), FloatToUint8 (Image.cpp:57-62)
            float c = std::isnan(v) ? v : std::min(std::max(v, 0.f), 1.f);
            c = std::pow(c, 0.45f);
            colour[h] = float_to_u8(c);
            alpha[h] = float_to_u8(v);
        }
    }
};

const Tables &tables() {
    static Tables t;
    return t;
}

__global__ void k_rgba16f_to_rgba8(const ushort4 *in, uint64_t n, const uint8_t *tab, uchar4 *out) {
    const uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const ushort4 h = in[i];
    out[i] = make_uchar4(__ldg(tab + h.x), __ldg(tab + h.y), __ldg(tab + h.z), __ldg(tab + 65536 + h.w));
}

__global__ void k_fb_to_half(const float4 *fb, uint32_t w, uint32_t h, ushort4 *out) {
    const uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    if (i >= static_cast<uint64_t>(w) * h) return;
    const uint32_t x = static_cast<uint32_t>(i % w), y = static_cast<uint32_t>(i / w);
    const float4 v = fb[static_cast<uint64_t>(h - 1 - y) * w + x];
    out[i] = make_ushort4(__half_as_ushort(__float2half_rn(v.x)), __half_as_ushort(__float2half_rn(v.y)),
                          __half_as_ushort(__float2half_rn(v.z)), __half_as_ushort(__float2half_rn(v.w)));
}

// ---- PNG ----------------------------------------------------------------------------------------------

uint32_t crc32(const uint8_t *p, size_t n, uint32_t crc = 0) {
    static uint32_t table[256];
    static std::once_flag once;
    std::call_once(once, [] {
        for (uint32_t k = 0; k < 256; ++k) {
            uint32_t c = k;
            for (int b = 0; b < 8; ++b) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            table[k] = c;
        }
    });
    crc = ~crc;
    for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
    return ~crc;
}

uint32_t adler32(const uint8_t *p, size_t n) {
    uint32_t a = 1, b = 0;
    while (n > 0) {
        const size_t k = std::min<size_t>(n, 5552);
        for (size_t i = 0; i < k; ++i) {
            a += p[i];
            b += a;
        }
        a %= 65521u;
        b %= 65521u;
        p += k;
        n -= k;
    }
    return (b << 16) | a;
}

// LSB-first bit writer (RFC 1951 3.1.1); Huffman codes are written most significant bit first.
struct BitWriter {
    std::vector<uint8_t> &out;
    uint64_t acc = 0;
    int bits = 0;
    explicit BitWriter(std::vector<uint8_t> &o) : out(o) {}
    void put(uint32_t v, int n) {
        acc |= static_cast<uint64_t>(v) << bits;
        bits += n;
        while (bits >= 8) {
            out.push_back(static_cast<uint8_t>(acc));
            acc >>= 8;
            bits -= 8;
        }
    }
    void put_code(uint32_t code, int n) {  // reverse into LSB-first order
        uint32_t r = 0;
        for (int i = 0; i < n; ++i) r |= ((code >> i) & 1u) << (n - 1 - i);
        put(r, n);
    }
    void flush() {
        if (bits > 0) out.push_back(static_cast<uint8_t>(acc));
        acc = 0;
        bits = 0;
    }
};

// Fixed literal/length code of symbol s (RFC 1951 3.2.6).
void put_litlen(BitWriter &w, uint32_t s) {
    if (s < 144) {
        w.put_code(0x30 + s, 8);
    } else if (s < 256) {
        w.put_code(0x190 + (s - 144), 9);
    } else if (s < 280) {
        w.put_code(s - 256, 7);
    } else {
        w.put_code(0xC0 + (s - 280), 8);
    }
}

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11,
                                12, 12, 13, 13};

void put_match(BitWriter &w, uint32_t len, uint32_t dist) {
    int l = 28;
    while (kLenBase[l] > len) --l;
    put_litlen(w, 257 + l);
    if (kLenExtra[l]) w.put(len - kLenBase[l], kLenExtra[l]);
    int d = 29;
    while (kDistBase[d] > dist) --d;
    w.put_code(static_cast<uint32_t>(d), 5);
    if (kDistExtra[d]) w.put(dist - kDistBase[d], kDistExtra[d]);
}

// zlib stream (RFC 1950) of one fixed-Huffman deflate block with hash-chain LZ77 matches.
std::vector<uint8_t> zlib_compress(const std::vector<uint8_t> &in) {
    std::vector<uint8_t> out{0x78, 0x01};
    BitWriter w(out);
    w.put(1, 1);  // BFINAL
    w.put(1, 2);  // BTYPE = fixed Huffman
    constexpr uint32_t kWindow = 32768, kHashBits = 15, kMaxChain = 24;
    std::vector<int32_t> head(1u << kHashBits, -1), prev(kWindow, -1);
    const size_t n = in.size();
    auto hash = [&](size_t i) {
        const uint32_t v = static_cast<uint32_t>(in[i]) | (static_cast<uint32_t>(in[i + 1]) << 8) |
                           (static_cast<uint32_t>(in[i + 2]) << 16);
        return (v * 2654435761u) >> (32 - kHashBits);
    };
    auto insert = [&](size_t i) {
        if (i + 2 >= n) return;
        const uint32_t h = hash(i);
        prev[i & (kWindow - 1)] = head[h];
        head[h] = static_cast<int32_t>(i);
    };
    size_t i = 0;
    while (i < n) {
        uint32_t best_len = 0, best_dist = 0;
        if (i + 2 < n) {
            int32_t cand = head[hash(i)];
            const uint32_t max_len = static_cast<uint32_t>(std::min<size_t>(258, n - i));
            for (uint32_t chain = 0; cand >= 0 && chain < kMaxChain; ++chain) {
                const size_t c = static_cast<size_t>(cand);
                if (i - c > kWindow - 1) break;
                uint32_t l = 0;
                while (l < max_len && in[c + l] == in[i + l]) ++l;
                if (l > best_len) {
                    best_len = l;
                    best_dist = static_cast<uint32_t>(i - c);
                    if (l == max_len) break;
                }
                const int32_t nxt = prev[c & (kWindow - 1)];
                if (nxt >= cand) break;  // stale entry from an older window
                cand = nxt;
            }
        }
        if (best_len >= 3) {
            put_match(w, best_len, best_dist);
            for (uint32_t k = 0; k < best_len; ++k) insert(i + k);
            i += best_len;
        } else {
            put_litlen(w, in[i]);
            insert(i);
            ++i;
        }
    }
    put_litlen(w, 256);
    w.flush();
    const uint32_t a = adler32(in.data(), n);
    for (int s = 24; s >= 0; s -= 8) out.push_back(static_cast<uint8_t>(a >> s));
    return out;
}

void put_be32(std::vector<uint8_t> &o, uint32_t v) {
    for (int s = 24; s >= 0; s -= 8) o.push_back(static_cast<uint8_t>(v >> s));
}

void png_chunk(std::vector<uint8_t> &o, const char *type, const std::vector<uint8_t> &data) {
    put_be32(o, static_cast<uint32_t>(data.size()));
    const size_t start = o.size();
    o.insert(o.end(), type, type + 4);
    o.insert(o.end(), data.begin(), data.end());
    put_be32(o, crc32(o.data() + start, o.size() - start));
}

inline uint8_t paeth(int a, int b, int c) {
    const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    return static_cast<uint8_t>(pa <= pb && pa <= pc ? a : (pb <= pc ? b : c));
}

// ---- Radiance RGBE ------------------------------------------------------------------------------------

// Ward's shared-exponent encoding: e = frexp exponent of max(r, g, b), mantissas truncated to 8 bits.
void rgbe(const float *c, uint8_t *o) {
    const float r = std::max(c[0], 0.f), g = std::max(c[1], 0.f), b = std::max(c[2], 0.f);
    const float v = std::max(r, std::max(g, b));
    if (!(v >= 1e-32f) || !std::isfinite(v)) {
        o[0] = o[1] = o[2] = o[3] = 0;
        return;
    }
    int e;
    const float m = std::frexp(v, &e);
    const float s = m * 256.f / v;
    o[0] = static_cast<uint8_t>(r * s);
    o[1] = static_cast<uint8_t>(g * s);
    o[2] = static_cast<uint8_t>(b * s);
    o[3] = static_cast<uint8_t>(e + 128);
}

// One component of a new-style run-length scanline: runs of >= 3 equal bytes as (128 + n, v), n <= 127;
// the rest as literal dumps (n, bytes...), n <= 128.
void rle_component(std::vector<uint8_t> &o, const uint8_t *d, uint32_t w) {
    uint32_t i = 0;
    while (i < w) {
        uint32_t run = 1;
        while (i + run < w && run < 127 && d[i + run] == d[i]) ++run;
        if (run >= 3) {
            o.push_back(static_cast<uint8_t>(128 + run));
            o.push_back(d[i]);
            i += run;
            continue;
        }
        uint32_t j = i;  // literal until the next run of 3
        while (j < w && j - i < 128) {
            if (j + 2 < w && d[j] == d[j + 1] && d[j] == d[j + 2]) break;
            ++j;
        }
        if (j == i) j = i + 1;
        o.push_back(static_cast<uint8_t>(j - i));
        o.insert(o.end(), d + i, d + j);
        i = j;
    }
}

// ---- OpenEXR ------------------------------------------------------------------------------------------

void put_le32(std::vector<uint8_t> &o, uint32_t v) {
    for (int s = 0; s < 32; s += 8) o.push_back(static_cast<uint8_t>(v >> s));
}
void put_le64(std::vector<uint8_t> &o, uint64_t v) {
    for (int s = 0; s < 64; s += 8) o.push_back(static_cast<uint8_t>(v >> s));
}
void put_str(std::vector<uint8_t> &o, const char *s) { o.insert(o.end(), s, s + std::strlen(s) + 1); }
void exr_attr(std::vector<uint8_t> &o, const char *name, const char *type, const std::vector<uint8_t> &v) {
    put_str(o, name);
    put_str(o, type);
    put_le32(o, static_cast<uint32_t>(v.size()));
    o.insert(o.end(), v.begin(), v.end());
}

}  // namespace

const uint8_t *rgba8_table(bool srgb) { return srgb ? tables().colour : tables().alpha; }

void rgba16f_to_rgba8(const uint16_t *in, uint64_t pixels, uint8_t *out) {
    const Tables &t = tables();
    for (uint64_t i = 0; i < pixels; ++i) {
        out[4 * i + 0] = t.colour[in[4 * i + 0]];
        out[4 * i + 1] = t.colour[in[4 * i + 1]];
        out[4 * i + 2] = t.colour[in[4 * i + 2]];
        out[4 * i + 3] = t.alpha[in[4 * i + 3]];
    }
}

cudaError_t launch_rgba16f_to_rgba8(const ushort4 *in, uint64_t pixels, const uint8_t *tab, uchar4 *out,
                                    cudaStream_t stream) {
    if (pixels == 0) return cudaSuccess;
    k_rgba16f_to_rgba8<<<static_cast<unsigned>((pixels + 255) / 256), 256, 0, stream>>>(in, pixels, tab, out);
    return cudaGetLastError();
}

cudaError_t launch_fb_to_half(const float4 *fb, uint32_t width, uint32_t height, ushort4 *out, cudaStream_t stream) {
    const uint64_t n = static_cast<uint64_t>(width) * height;
    if (n == 0) return cudaSuccess;
    k_fb_to_half<<<static_cast<unsigned>((n + 255) / 256), 256, 0, stream>>>(fb, width, height, out);
    return cudaGetLastError();
}

std::vector<uint8_t> encode_png(const uint8_t *rgba8, uint32_t width, uint32_t height) {
    const size_t stride = 4ull * width;
    std::vector<uint8_t> raw;
    raw.reserve((stride + 1) * height);
    std::vector<uint8_t> cand[5];
    for (auto &c : cand) c.resize(stride);
    for (uint32_t y = 0; y < height; ++y) {
        const uint8_t *row = rgba8 + y * stride;
        const uint8_t *up = y > 0 ? rgba8 + (y - 1) * stride : nullptr;
        uint64_t best_cost = ~0ull;
        int best = 0;
        for (int f = 0; f < 5; ++f) {
            uint64_t cost = 0;
            for (size_t x = 0; x < stride; ++x) {
                const int a = x >= 4 ? row[x - 4] : 0, b = up ? up[x] : 0, c = (x >= 4 && up) ? up[x - 4] : 0;
                int pred = 0;
                switch (f) {
                case 1: pred = a; break;
                case 2: pred = b; break;
                case 3: pred = (a + b) >> 1; break;
                case 4: pred = paeth(a, b, c); break;
                default: break;
                }
                const uint8_t r = static_cast<uint8_t>(row[x] - pred);
                cand[f][x] = r;
                cost += static_cast<uint64_t>(std::abs(static_cast<int8_t>(r)));
            }
            if (cost < best_cost) {
                best_cost = cost;
                best = f;
            }
        }
        raw.push_back(static_cast<uint8_t>(best));
        raw.insert(raw.end(), cand[best].begin(), cand[best].end());
    }
    std::vector<uint8_t> o{0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, width);
    put_be32(ihdr, height);
    ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});  // 8-bit RGBA, deflate, adaptive filters, no interlace
    png_chunk(o, "IHDR", ihdr);
    png_chunk(o, "IDAT", zlib_compress(raw));
    png_chunk(o, "IEND", {});
    return o;
}

std::vector<uint8_t> encode_hdr(const float *rgba, uint32_t width, uint32_t height) {
    std::vector<uint8_t> o;
    char head[128];
    const int n = std::snprintf(head, sizeof(head), "#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y %u +X %u\n", height, width);
    o.insert(o.end(), head, head + n);
    std::vector<uint8_t> px(4ull * width), comp(width);
    const bool rle = width >= 8 && width < 32768;
    for (uint32_t y = 0; y < height; ++y) {
        for (uint32_t x = 0; x < width; ++x) rgbe(rgba + 4ull * (static_cast<uint64_t>(y) * width + x), &px[4ull * x]);
        if (!rle) {
            o.insert(o.end(), px.begin(), px.end());
            continue;
        }
        o.insert(o.end(), {2, 2, static_cast<uint8_t>(width >> 8), static_cast<uint8_t>(width & 255)});
        for (int c = 0; c < 4; ++c) {
            for (uint32_t x = 0; x < width; ++x) comp[x] = px[4ull * x + c];
            rle_component(o, comp.data(), width);
        }
    }
    return o;
}

std::vector<uint8_t> encode_exr(const uint16_t *rgba16f, uint32_t width, uint32_t height) {
    std::vector<uint8_t> o{0x76, 0x2F, 0x31, 0x01, 2, 0, 0, 0};  // magic, version 2, scanline file
    std::vector<uint8_t> ch;
    for (const char *name : {"A", "B", "G", "R"}) {  // channels sorted by name
        put_str(ch, name);
        put_le32(ch, 1);  // HALF
        ch.insert(ch.end(), {0, 0, 0, 0});  // pLinear + reserved
        put_le32(ch, 1);
        put_le32(ch, 1);
    }
    ch.push_back(0);
    exr_attr(o, "channels", "chlist", ch);
    exr_attr(o, "compression", "compression", {0});
    std::vector<uint8_t> box;
    put_le32(box, 0);
    put_le32(box, 0);
    put_le32(box, width - 1);
    put_le32(box, height - 1);
    exr_attr(o, "dataWindow", "box2i", box);
    exr_attr(o, "displayWindow", "box2i", box);
    exr_attr(o, "lineOrder", "lineOrder", {0});
    std::vector<uint8_t> one;
    put_le32(one, 0x3F800000u);
    exr_attr(o, "pixelAspectRatio", "float", one);
    exr_attr(o, "screenWindowCenter", "v2f", std::vector<uint8_t>(8, 0));
    exr_attr(o, "screenWindowWidth", "float", one);
    o.push_back(0);
    const uint64_t line_bytes = 8ull * width;
    const uint64_t table_at = o.size();
    for (uint32_t y = 0; y < height; ++y) put_le64(o, table_at + 8ull * height + y * (8 + line_bytes));
    for (uint32_t y = 0; y < height; ++y) {
        put_le32(o, y);
        put_le32(o, static_cast<uint32_t>(line_bytes));
        for (int c : {3, 2, 1, 0}) {  // A, B, G, R
            for (uint32_t x = 0; x < width; ++x) {
                const uint16_t h = rgba16f[4ull * (static_cast<uint64_t>(y) * width + x) + c];
                o.push_back(static_cast<uint8_t>(h));
                o.push_back(static_cast<uint8_t>(h >> 8));
            }
        }
    }
    return o;
}

bool write_file(const std::string &path, const std::vector<uint8_t> &bytes, std::string &err) {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) {
        err = "cannot open " + path + " for writing";
        return false;
    }
    const size_t n = std::fwrite(bytes.data(), 1, bytes.size(), f);
    const bool ok = n == bytes.size() && std::fclose(f) == 0;
    if (!ok) err = "cannot write " + path;
    return ok;
}

}  // namespace spk
