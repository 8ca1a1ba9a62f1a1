// conv_tc.cu -- tcgen05 implicit-GEMM 3x3 convolutions (see conv_tc.cuh).
//
// Forward / dgrad (one CTA per output tile of tw x (mt * th) pixels: mt M tiles of tw x th = 128 pixels
// stacked vertically, tw a multiple of 8, 4 warps):
//   warp 0 lane 0  TMA producer: per K block (column tap dx, 32-channel chunk) one 4-D tiled load of the
//                  input box {32 ch, tw px, mt * th + 2 rows, 1 image} shifted by dx and reaching one row
//                  above and below the tile (zero fill outside the image = the conv's padding), and three
//                  2-D loads of the weight slices {32, cout} of the taps (dy, dx), dy = -1, 0, 1, into a
//                  ring of 2-4 stages;
//   warp 1 lane 0  MMA issuer: per stage, row tap dy and M tile m, two kind::f16 MMAs (K = 16 each) whose A
//                  operand starts (m * th + dy + 1) * tw rows into the input box -- a whole number of 8-row
//                  swizzle atoms, so one box serves all three row taps of all M tiles and one weight slice
//                  serves all M tiles -- into M tile m's 128 x cout FP32 accumulator in TMEM (columns
//                  m * cout ...), committing each stage back to the producer;
//   all 4 warps    epilogue: tcgen05.ld of the pixel rows (warp w owns TMEM lanes 32w..32w+31), bias,
//                  ReLU or ReLU-backward mask, BF16 pack, 16-byte stores.
// Wgrad (one CTA per (128 rows of (tap, ci), pixel range)): TMA loads of the shifted input and the output
// gradient as they lie in NHWC memory (MN-major operands, 64-byte swizzle), MMAs that read them MN-major,
// and the FP32 partial sums added to dw with atomics. (SPK_CONV_WGRAD_TMA=0 keeps the earlier form: all
// threads gather and transpose both operands into K-major swizzled tiles.)
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>

#include "conv_tc.cuh"
#include "tc_common.cuh"

namespace spk {
namespace {

using namespace tc;

constexpr uint32_t kTileM = 128;
constexpr uint32_t kStages = 4;
constexpr uint32_t kATileBytes = kTileM * 64;  // 128 rows x 32 bf16
constexpr uint32_t kMaxCout = 256;
#ifndef SPK_CONV_STAGE_BUDGET_KB
#define SPK_CONV_STAGE_BUDGET_KB 32  // shared memory for the forward kernel's ring (KB): 2 stages, more CTAs per SM
#endif
constexpr uint32_t kStageBudget = SPK_CONV_STAGE_BUDGET_KB;

#ifndef SPK_CONV_TMA_STORE
#define SPK_CONV_TMA_STORE 1  // 1: forward epilogue staged in shared memory and written by TMA stores
#endif
#ifndef SPK_CONV_MTILES
#define SPK_CONV_MTILES 0  // M tiles (128 pixels each) per forward CTA: 1, 2 or 4; 0 = chosen per layer
#endif

// Where and how the forward kernels write a pixel's output channels.
struct OutSpec {
    __nv_bfloat16 *out;
    uint32_t out_ld;
    const float *bias;
    uint32_t relu;
    const __nv_bfloat16 *mask;
    uint32_t mask_ld;
    __nv_bfloat16 *pool;  // dense [n][h/2][w/2][cout]: 2x2 average of the output, or null
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&v);
}

// 2x2 average pooling of the packed BF16 outputs (channels col0..col0+15) of the four pixels of a 2x2 block,
// which sit in lanes l, l ^ 1 (next column) and l ^ tw, l ^ tw ^ 1 (next row) of the warp; every lane of the
// warp calls it. The lane holding the block's top-left pixel writes the pooled channels when that pixel is
// inside the image. Sum order per channel: top-left, top-right, bottom-left, bottom-right from 0, times 0.25,
// rounded to BF16 -- the order and rounding of the pooling kernel it replaces.
__device__ __forceinline__ void epilogue_pool(const OutSpec &O, const uint32_t (&pk)[8], uint32_t lane, uint32_t tw,
                                              bool inb, uint32_t img, uint32_t px, uint32_t py, uint32_t h,
                                              uint32_t w, uint32_t cout, uint32_t col0) {
    uint32_t b[8], c[8], d[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        b[e] = __shfl_xor_sync(0xFFFFFFFFu, pk[e], 1);
        c[e] = __shfl_xor_sync(0xFFFFFFFFu, pk[e], tw);
        d[e] = __shfl_xor_sync(0xFFFFFFFFu, pk[e], tw ^ 1u);
    }
    if ((lane & 1u) || (lane & tw) || !inb) return;
    uint32_t q[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        float lo = 0.f, hi = 0.f;
        const uint32_t words[4] = {pk[e], b[e], c[e], d[e]};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const __nv_bfloat162 v = *reinterpret_cast<const __nv_bfloat162 *>(&words[k]);
            lo += __low2float(v);
            hi += __high2float(v);
        }
        q[e] = pack_bf16(0.25f * lo, 0.25f * hi);
    }
    const size_t dst = ((static_cast<size_t>(img) * (h / 2) + py / 2) * (w / 2) + px / 2) * cout + col0;
    uint4 *op = reinterpret_cast<uint4 *>(O.pool + dst);
    op[0] = make_uint4(q[0], q[1], q[2], q[3]);
    op[1] = make_uint4(q[4], q[5], q[6], q[7]);
}

struct FwdParams {
    uint32_t n, h, w;
    uint32_t cin, cout;
    uint32_t tw, th, mt, tiles_x, tiles_y;  // M tile tw x th; mt M tiles per CTA; CTA tiles of tw x mt*th
    uint32_t stages, a_bytes, stage_bytes;  // ring depth; input box and stage sizes (1024-byte multiples)
    uint32_t stage_out;                     // 1: epilogue through shared memory and TMA stores
    OutSpec out_spec;
    uint32_t *err;
};

// Input box {32 ch, tw, rows + 2} (rows = mt * th) and the three weight slices of one column tap, each
// 1024-byte aligned.
__host__ __device__ constexpr uint32_t fwd_a_bytes(uint32_t tw, uint32_t rows) {
    return (64u * tw * (rows + 2u) + 1023u) & ~1023u;
}
__host__ __device__ constexpr uint32_t fwd_stage_bytes(uint32_t tw, uint32_t rows, uint32_t cout) {
    return fwd_a_bytes(tw, rows) + ((3u * cout * 64u + 1023u) & ~1023u);
}

__host__ __device__ constexpr uint32_t tmem_columns(uint32_t n) {
    return n <= 32 ? 32 : n <= 64 ? 64 : n <= 128 ? 128 : 256;
}

__device__ __forceinline__ uint8_t *align1024(uint8_t *raw) {
    const uint32_t a = smem_u32(raw);
    return raw + (((a + 1023u) & ~1023u) - a);
}


// Output channels col0..col0+15 of pixel `pix` from 16 FP32 accumulator columns: + bias (`bias16`, or
// none), then the ReLU-backward mask (keep where mask > 0; read only for pixels inside the image) or ReLU,
// packed to BF16 pairs.
__device__ __forceinline__ void epilogue_pack(const OutSpec &O, const uint32_t (&v)[16], const float *bias16,
                                              size_t pix, uint32_t col0, bool inb, uint32_t (&pk)[8]) {
    float f[16];
#pragma unroll
    for (int e = 0; e < 16; ++e) f[e] = __uint_as_float(v[e]) + (bias16 ? bias16[e] : 0.f);
    if (O.mask && inb) {
        const uint4 *mp = reinterpret_cast<const uint4 *>(O.mask + pix * O.mask_ld + col0);
        const uint4 m0 = mp[0], m1 = mp[1];
        const uint32_t mw[8] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w};
#pragma unroll
        for (int e = 0; e < 16; ++e) {
            const uint32_t bits = (mw[e >> 1] >> (16 * (e & 1))) & 0xFFFFu;
            // bf16 > 0: sign bit clear and not +0
            if ((bits & 0x8000u) || bits == 0u) f[e] = 0.f;
        }
    } else if (O.relu) {
#pragma unroll
        for (int e = 0; e < 16; ++e) f[e] = fmaxf(f[e], 0.f);
    }
#pragma unroll
    for (int e = 0; e < 8; ++e) pk[e] = pack_bf16(f[2 * e], f[2 * e + 1]);
}

#ifndef SPK_CONV_EPI_WARPS
#define SPK_CONV_EPI_WARPS 8  // warps per forward CTA (4 or 8); all of them drain TMEM in the epilogue
#endif
constexpr uint32_t kFwdThreads = 32u * SPK_CONV_EPI_WARPS;
static_assert(SPK_CONV_EPI_WARPS == 4 || SPK_CONV_EPI_WARPS == 8, "4 or 8 warps");

template <bool kPool>
__global__ void __launch_bounds__(kFwdThreads, 1)
    k_conv_fwd(const __grid_constant__ CUtensorMap tmx, const __grid_constant__ CUtensorMap tmw,
               const __grid_constant__ CUtensorMap tmy, FwdParams P) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = align1024(smem_raw);
    const uint32_t b_bytes = P.cout * 64u;  // one weight slice
    const uint32_t stage_bytes = P.stage_bytes, nst = P.stages;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + nst * stage_bytes);
    uint64_t *full = bars, *empty = bars + kStages, *accum = bars + 2 * kStages;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * kStages + 1);
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t ncols = tmem_columns(P.mt * P.cout);
    const uint32_t rows = P.mt * P.th;  // output rows of the CTA tile

    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < nst; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(accum, 1);
        fence_mbar_init();
        tma_prefetch_desc(&tmx);
        tma_prefetch_desc(&tmw);
    }
    if (warp == 0) tmem_alloc(tmem_slot, ncols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    uint32_t t = blockIdx.x;
    const uint32_t tx = t % P.tiles_x;
    t /= P.tiles_x;
    const uint32_t ty = t % P.tiles_y;
    const uint32_t img = t / P.tiles_y;
    const int x0 = static_cast<int>(tx * P.tw), y0 = static_cast<int>(ty * rows);
    const uint32_t nch = P.cin / 32u, nk = 3u * nch;  // K blocks: (column tap, channel chunk)

    if (warp == 0 && lane == 0) {
        for (uint32_t kb = 0; kb < nk; ++kb) {
            const uint32_t s = kb % nst, u = kb / nst;
            if (u > 0 && !mbar_wait(&empty[s], (u - 1) & 1u, P.err)) break;
            uint8_t *a = smem + s * stage_bytes;
            uint8_t *b = a + P.a_bytes;
            mbar_arrive_expect_tx(&full[s], 64u * P.tw * (rows + 2u) + 3u * b_bytes);
            const uint32_t dx3 = kb / nch, c = kb - dx3 * nch;
            tma_load_4d(a, &tmx, &full[s], static_cast<int>(c * 32u), x0 + static_cast<int>(dx3) - 1, y0 - 1,
                        static_cast<int>(img));
            for (uint32_t dy3 = 0; dy3 < 3; ++dy3)
                tma_load_2d(b + dy3 * b_bytes, &tmw, &full[s], static_cast<int>((dy3 * 3u + dx3) * P.cin + c * 32u), 0);
        }
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = idesc_bf16(kTileM, P.cout);
        bool ok = true;
        for (uint32_t kb = 0; kb < nk; ++kb) {
            const uint32_t s = kb % nst, u = kb / nst;
            if (!mbar_wait(&full[s], u & 1u, P.err)) {
                ok = false;
                break;
            }
            tc_fence_after();
            const uint32_t a = smem_u32(smem + s * stage_bytes), b = a + P.a_bytes;
#pragma unroll
            for (uint32_t dy3 = 0; dy3 < 3; ++dy3) {
                const uint32_t bd = b + dy3 * b_bytes;
                for (uint32_t m = 0; m < P.mt; ++m) {
                    const uint32_t ad = a + (m * P.th + dy3) * P.tw * 64u;
#pragma unroll
                    for (uint32_t k2 = 0; k2 < 2; ++k2)
                        mma_bf16(tmem + m * P.cout, smem_desc_sw64(ad + 32u * k2), smem_desc_sw64(bd + 32u * k2),
                                 idesc, (kb | dy3 | k2) != 0u);
                }
            }
            mma_commit(&empty[s]);
        }
        if (ok) mma_commit(accum);
    }
    __syncwarp();

    // Epilogue.
    bool ready = mbar_wait(accum, 0, P.err);
    ready = __all_sync(0xFFFFFFFFu, ready);
    tc_fence_after();
    // With P.stage_out the tile goes through shared memory (the ring, idle once every MMA has completed):
    // per M tile and 32-channel chunk a 128-row x 64-byte region in the 64-byte-swizzled layout (rows =
    // pixels of the M tile in box order), written by a 4-D TMA store that writes whole lines and drops the
    // pixels outside the image. Otherwise each thread stores its pixel's channels itself.
    // Warp w reads TMEM lane group w % 4 (the lanes it may access). With 8 warps the second four take the
    // odd M tiles, or (one M tile) the upper half of the output channels.
    const uint32_t lgrp = warp & 3u, part = warp >> 2, nparts = SPK_CONV_EPI_WARPS / 4u;
    const uint32_t r = lgrp * 32u + lane;
    const uint32_t chunks = P.cout / 32u;
    const uint32_t m_step = P.mt >= nparts ? nparts : 1u;
    const uint32_t m_first = P.mt >= nparts ? part : 0u;
    const uint32_t j_count = P.mt >= nparts ? P.cout / 16u : P.cout / 16u / nparts;
    const uint32_t j_first = P.mt >= nparts ? 0u : part * j_count;
    for (uint32_t m = m_first; ready && m < P.mt; m += m_step) {
        const uint32_t px = static_cast<uint32_t>(x0) + (r % P.tw);
        const uint32_t py = static_cast<uint32_t>(y0) + m * P.th + (r / P.tw);
        const bool inb = px < P.w && py < P.h;
        const size_t pix = (static_cast<size_t>(img) * P.h + py) * P.w + px;
        for (uint32_t j = j_first; j < j_first + j_count; ++j) {
            uint32_t v[16], pk[8];
            tmem_ld16(tmem + ((lgrp * 32u) << 16) + m * P.cout + j * 16u, v);
            epilogue_pack(P.out_spec, v, P.out_spec.bias ? P.out_spec.bias + j * 16u : nullptr, pix, j * 16u, inb,
                          pk);
            if (kPool)
                epilogue_pool(P.out_spec, pk, lane, P.tw, inb, img, px, py, P.h, P.w, P.cout, j * 16u);
            if (P.stage_out) {
                uint8_t *region = smem + (m * chunks + (j >> 1)) * (kTileM * 64u);
                const uint32_t c0 = (j & 1u) * 2u;
                *reinterpret_cast<uint4 *>(region + sw64_offset(r, c0)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                *reinterpret_cast<uint4 *>(region + sw64_offset(r, c0 + 1u)) = make_uint4(pk[4], pk[5], pk[6], pk[7]);
            } else if (inb) {
                uint4 *op = reinterpret_cast<uint4 *>(P.out_spec.out + pix * P.out_spec.out_ld + j * 16u);
                op[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                op[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
            }
        }
    }
    if (P.stage_out) {
        fence_proxy_async_smem();
        __syncthreads();
        if (threadIdx.x == 0 && ready) {
            for (uint32_t m = 0; m < P.mt; ++m)
                for (uint32_t cc = 0; cc < chunks; ++cc)
                    tma_store_4d(&tmy, smem + (m * chunks + cc) * (kTileM * 64u), static_cast<int>(cc * 32u), x0,
                                 y0 + static_cast<int>(m * P.th), static_cast<int>(img));
            tma_store_commit();
            tma_store_wait_read();
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, ncols);
    }
}

// ------------------------------------------------------------------------------------------------
// wgrad
// ------------------------------------------------------------------------------------------------
constexpr uint32_t kWgStages = 2;
constexpr uint32_t kWgKPix = 32;  // pixels per K block

struct WgradParams {
    uint32_t n, h, w, cin, cout;
    const __nv_bfloat16 *x;
    uint32_t x_ld;
    const __nv_bfloat16 *dy;
    uint32_t dy_ld;
    float *dw;
    uint32_t kblocks;    // K blocks per CTA
    uint32_t row_tiles;  // ceil(9 * cin / 128)
    unsigned long long npix;
    uint32_t *err;
};

__host__ __device__ constexpr uint32_t wg_stage_bytes(uint32_t cout) {
    return (kATileBytes + cout * 64u + 1023u) & ~1023u;
}

// Writes 8 bf16 (one 16-byte vector: channels c..c+7 of one pixel) as column `k` of rows row0..row0+7.
__device__ __forceinline__ void scatter_column(uint8_t *tile, uint32_t row0, uint32_t k, uint4 v) {
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (uint32_t e = 0; e < 8; ++e) {
        const uint16_t h = static_cast<uint16_t>((w[e >> 1] >> (16u * (e & 1u))) & 0xFFFFu);
        *reinterpret_cast<uint16_t *>(tile + sw64_offset(row0 + e, k >> 3) + (k & 7u) * 2u) = h;
    }
}

__global__ void __launch_bounds__(128, 1) k_conv_wgrad(WgradParams P) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = align1024(smem_raw);
    const uint32_t stage_bytes = wg_stage_bytes(P.cout);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kWgStages * stage_bytes);
    uint64_t *full = bars, *empty = bars + kWgStages, *accum = bars + 2 * kWgStages;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * kWgStages + 1);
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    const uint32_t ncols = tmem_columns(P.cout);

    if (tid == 0) {
        for (uint32_t s = 0; s < kWgStages; ++s) {
            mbar_init(&full[s], 128);
            mbar_init(&empty[s], 1);
        }
        mbar_init(accum, 1);
        fence_mbar_init();
    }
    if (warp == 0) tmem_alloc(tmem_slot, ncols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    const uint32_t rt = blockIdx.x % P.row_tiles, split = blockIdx.x / P.row_tiles;
    const uint32_t krows = 9u * P.cin;
    const unsigned long long pbase = static_cast<unsigned long long>(split) * P.kblocks * kWgKPix;
    const uint32_t hw = P.h * P.w;
    const uint32_t idesc = idesc_bf16(kTileM, P.cout);
    // Lane layout of the gathers: 4 channel groups of 8 x 8 pixels per warp pass (64 contiguous bytes
    // of each pixel's channels).
    const uint32_t cg = lane & 3u, kk = lane >> 2;
    // `ok` turns false on a wait timeout; the loop leaves only at a barrier, where every thread agrees.
    bool ok = true;
    for (uint32_t kb = 0; kb < P.kblocks; ++kb) {
        const uint32_t s = kb % kWgStages, u = kb / kWgStages;
        if (u > 0 && ok) ok = mbar_wait(&empty[s], (u - 1) & 1u, P.err);
        ok = __syncthreads_and(ok);
        if (!ok) break;
        uint8_t *a = smem + s * stage_bytes, *b = a + kATileBytes;
        // A: rows g = (tap, ci) of this row tile, column k = pixel pbase + kb*32 + k, value x[p + tap][ci].
        for (uint32_t it = warp; it < 16u; it += 4u) {  // 16 passes: 4 channel-group quads x 4 pixel octets
            const uint32_t group = (it >> 2) * 4u + cg;  // 8-row group 0..15
            const uint32_t k = (it & 3u) * 8u + kk;
            const uint32_t g0 = rt * kTileM + group * 8u;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            const unsigned long long p = pbase + static_cast<unsigned long long>(kb) * kWgKPix + k;
            if (g0 < krows && p < P.npix) {
                const uint32_t tap = g0 / P.cin, ci0 = g0 - tap * P.cin;
                const uint32_t img = static_cast<uint32_t>(p / hw), rem = static_cast<uint32_t>(p - static_cast<unsigned long long>(img) * hw);
                const int y = static_cast<int>(rem / P.w) + static_cast<int>(tap / 3u) - 1;
                const int xx = static_cast<int>(rem % P.w) + static_cast<int>(tap % 3u) - 1;
                if (y >= 0 && y < static_cast<int>(P.h) && xx >= 0 && xx < static_cast<int>(P.w)) {
                    const size_t q = (static_cast<size_t>(img) * P.h + static_cast<uint32_t>(y)) * P.w + static_cast<uint32_t>(xx);
                    v = *reinterpret_cast<const uint4 *>(P.x + q * P.x_ld + ci0);
                }
            }
            scatter_column(a, group * 8u, k, v);
        }
        // B: rows co, column k, value dy[p][co].
        const uint32_t bgroups = P.cout / 8u;  // 8-row groups; cout % 32 == 0, so bgroups passes
        for (uint32_t it = warp; it < bgroups; it += 4u) {
            const uint32_t group = (it >> 2) * 4u + cg;
            const uint32_t k = (it & 3u) * 8u + kk;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            const unsigned long long p = pbase + static_cast<unsigned long long>(kb) * kWgKPix + k;
            if (p < P.npix) v = *reinterpret_cast<const uint4 *>(P.dy + static_cast<size_t>(p) * P.dy_ld + group * 8u);
            scatter_column(b, group * 8u, k, v);
        }
        fence_proxy_async_smem();
        mbar_arrive(&full[s]);
        if (tid == 0) {
            if (!mbar_wait(&full[s], u & 1u, P.err)) {
                ok = false;
            } else {
                tc_fence_after();
                const uint32_t sa = smem_u32(a), sb = smem_u32(b);
#pragma unroll
                for (uint32_t k2 = 0; k2 < 2; ++k2)
                    mma_bf16(tmem, smem_desc_sw64(sa + 32u * k2), smem_desc_sw64(sb + 32u * k2), idesc,
                             (kb | k2) != 0u);
                mma_commit(&empty[s]);
            }
        }
    }
    ok = __syncthreads_and(ok);
    if (tid == 0 && ok) mma_commit(accum);
    bool ready = ok && mbar_wait(accum, 0, P.err);
    ready = __all_sync(0xFFFFFFFFu, ready);
    tc_fence_after();
    if (ready) {
        const uint32_t g = rt * kTileM + warp * 32u + lane;
        for (uint32_t j = 0; j < P.cout / 16u; ++j) {
            uint32_t v[16];
            tmem_ld16(tmem + ((warp * 32u) << 16) + j * 16u, v);
            if (g >= krows) continue;
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                const float f = __uint_as_float(v[e]);
                if (f != 0.f) atomicAdd(P.dw + static_cast<size_t>(j * 16u + e) * krows + g, f);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, ncols);
    }
}

// ------------------------------------------------------------------------------------------------
// wgrad with TMA-fed MN-major operands
// ------------------------------------------------------------------------------------------------
// GEMM dw[g][co] = sum_p x[p + tap(g)][ci(g)] * dy[p][co], rows g = (tap, ci) in M tiles of 128, N = cout,
// K = pixels in blocks of a tw x th = 64-pixel tile. In NHWC memory both operands have M (N) contiguous and
// K strided, so they are loaded as they lie: per K block, warp 0 issues one 4-D TMA load per 32-row span of
// the M tile (the input box {32 ch, tw, th, 1} of that span's channel chunk, shifted by its tap; zero fill
// outside the image is the padding) and one per 32-channel span of dy (unshifted), each landing as 64 rows
// (pixels) x 64 bytes in the 64-byte-swizzled layout; warp 1 issues four kind::f16 MMAs (K = 16 pixels
// each) that read both tiles MN-major. The FP32 partial sums of the CTA's pixel range are then added to dw.
constexpr uint32_t kWgtStages = 4;
constexpr uint32_t kWgtPix = 64;                 // pixels per K block
constexpr uint32_t kWgtSpanBytes = kWgtPix * 64;  // one 32-channel span of a K block: 64 rows x 64 B
// Slack after the ring, before the barriers: every MMA read stays inside its stage for the descriptor
// offsets above; the slack keeps it inside the CTA's shared memory even if the two offsets were read the
// other way round (8-row groups 4 KB apart, spans 512 B apart).
constexpr uint32_t kWgtSlack = 8192;

struct WgradTmaParams {
    uint32_t n, h, w, cin, cout;
    uint32_t tw, th, tiles_x, tiles_y;  // K-block pixel tile and tiles per image row / column
    uint32_t krows;                     // 9 * cin
    uint32_t m_tiles;                   // ceil(krows / 128)
    uint32_t kblocks;                   // K blocks (pixel tiles) per CTA
    uint32_t ktotal;                    // pixel tiles in all images
    uint32_t stages, stage_bytes;
    float *dw;
    uint32_t *err;
};

__host__ __device__ constexpr uint32_t wgt_stage_bytes(uint32_t cout) { return 4u * kWgtSpanBytes + (cout / 32u) * kWgtSpanBytes; }

__global__ void __launch_bounds__(128, 1)
    k_conv_wgrad_tma(const __grid_constant__ CUtensorMap tmx, const __grid_constant__ CUtensorMap tmdy, WgradTmaParams P) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = align1024(smem_raw);
    const uint32_t nst = P.stages, stage_bytes = P.stage_bytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + nst * stage_bytes + kWgtSlack);
    uint64_t *full = bars, *empty = bars + kWgtStages, *accum = bars + 2 * kWgtStages;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * kWgtStages + 1);
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t ncols = tmem_columns(P.cout);

    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < nst; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(accum, 1);
        fence_mbar_init();
        tma_prefetch_desc(&tmx);
        tma_prefetch_desc(&tmdy);
    }
    if (warp == 0) tmem_alloc(tmem_slot, ncols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    const uint32_t mtile = blockIdx.x % P.m_tiles, split = blockIdx.x / P.m_tiles;
    const uint32_t kb0 = split * P.kblocks;
    const uint32_t nkb = kb0 < P.ktotal ? min(P.kblocks, P.ktotal - kb0) : 0u;
    const uint32_t cspans = P.cout / 32u;
    // Spans of this M tile that hold rows < krows (the rest of the A tile is never loaded; its rows of the
    // accumulator are not written out).
    const uint32_t g_first = mtile * kTileM;
    const uint32_t aspans = min(4u, (P.krows - g_first + 31u) / 32u);

    if (warp == 0 && lane == 0) {
        const uint32_t tx_bytes = (aspans + cspans) * kWgtSpanBytes;
        for (uint32_t i = 0; i < nkb; ++i) {
            const uint32_t s = i % nst, u = i / nst;
            if (u > 0 && !mbar_wait(&empty[s], (u - 1) & 1u, P.err)) break;
            uint32_t t = kb0 + i;
            const uint32_t tx = t % P.tiles_x;
            t /= P.tiles_x;
            const uint32_t ty = t % P.tiles_y;
            const int img = static_cast<int>(t / P.tiles_y);
            const int x0 = static_cast<int>(tx * P.tw), y0 = static_cast<int>(ty * P.th);
            uint8_t *a = smem + s * stage_bytes;
            uint8_t *b = a + 4u * kWgtSpanBytes;
            mbar_arrive_expect_tx(&full[s], tx_bytes);
            for (uint32_t sp = 0; sp < aspans; ++sp) {
                const uint32_t g0 = g_first + sp * 32u;
                const uint32_t tap = g0 / P.cin, ci0 = g0 - tap * P.cin;
                tma_load_4d(a + sp * kWgtSpanBytes, &tmx, &full[s], static_cast<int>(ci0),
                            x0 + static_cast<int>(tap % 3u) - 1, y0 + static_cast<int>(tap / 3u) - 1, img);
            }
            for (uint32_t sp = 0; sp < cspans; ++sp)
                tma_load_4d(b + sp * kWgtSpanBytes, &tmdy, &full[s], static_cast<int>(sp * 32u), x0, y0, img);
        }
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = idesc_bf16(kTileM, P.cout, true, true);
        bool ok = true;
        for (uint32_t i = 0; i < nkb; ++i) {
            const uint32_t s = i % nst, u = i / nst;
            if (!mbar_wait(&full[s], u & 1u, P.err)) {
                ok = false;
                break;
            }
            tc_fence_after();
            const uint32_t a = smem_u32(smem + s * stage_bytes), b = a + 4u * kWgtSpanBytes;
#pragma unroll
            for (uint32_t k16 = 0; k16 < kWgtPix / 16u; ++k16)
                mma_bf16(tmem, smem_desc_mn_sw64(a + k16 * 1024u, kWgtSpanBytes),
                         smem_desc_mn_sw64(b + k16 * 1024u, kWgtSpanBytes), idesc, (i | k16) != 0u);
            mma_commit(&empty[s]);
        }
        if (ok && nkb > 0) mma_commit(accum);
    }
    __syncwarp();

    bool ready = nkb > 0 && mbar_wait(accum, 0, P.err);
    ready = __all_sync(0xFFFFFFFFu, ready);
    tc_fence_after();
    if (ready) {
        const uint32_t g = g_first + warp * 32u + lane;
        for (uint32_t j = 0; j < P.cout / 16u; ++j) {
            uint32_t v[16];
            tmem_ld16(tmem + ((warp * 32u) << 16) + j * 16u, v);
            if (g >= P.krows) continue;
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                const float f = __uint_as_float(v[e]);
                if (f != 0.f) atomicAdd(P.dw + static_cast<size_t>(j * 16u + e) * P.krows + g, f);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, ncols);
    }
}

__global__ void k_transpose_weights(const __nv_bfloat16 *w, __nv_bfloat16 *wt, uint32_t cout, uint32_t cin) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;  // index into wt [cin][9][cout]
    if (i >= cout * cin * 9u) return;
    const uint32_t co = i % cout, tap = (i / cout) % 9u, ci = i / (9u * cout);
    wt[i] = w[(static_cast<size_t>(co) * 9u + (8u - tap)) * cin + ci];
}

// ------------------------------------------------------------------------------------------------
// Host: tensor maps through the driver entry point (no libcuda link dependency).
// ------------------------------------------------------------------------------------------------
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

constexpr int kMaxDynSmem = 227 * 1024;

// Dynamic shared memory of a launch: what the kernel uses, raised so that the CTAs resident on one SM
// never ask for more than the SM's 512 TMEM columns (an allocation beyond that would wait for another
// CTA to finish). 0 when the kernel would use more than a CTA may have: the caller refuses the launch.
size_t launch_smem(size_t used, uint32_t tmem_cols) {
    if (used > static_cast<size_t>(kMaxDynSmem)) return 0;
    const size_t per_sm = 228u * 1024u;
    const size_t ctas = 512u / tmem_cols;
    const size_t floor_bytes = per_sm / (ctas + 1u) - 1024u + 1u;  // the SM reserves 1 KB per CTA: ctas + 1 do not fit
    return std::min<size_t>(kMaxDynSmem, std::max(used, floor_bytes));
}

// Waits on an mbarrier that nothing arrives at: the bounded wait gives up after 1 s and sets
// kErrWaitTimeout, the failure path every tensor-core kernel takes when its pipeline stalls.
__global__ void k_wait_probe(uint32_t *err) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) mbar_wait(&bar, 0, err);
    __syncthreads();
}

int device_sms() {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

// M tiles per forward CTA. Two M tiles share each weight slice and each input box row between more
// pixels (fewer bytes staged per pixel, fewer CTAs paying the fixed set-up and epilogue), as long as the
// accumulators fit 256 TMEM columns and the layer still gives every SM several CTAs. Four (explicit
// SPK_CONV_MTILES=4 only) leave too few CTAs per SM to hide each CTA's load latency: slower on GB300.
uint32_t conv_mtiles(const ConvGeom &g, uint32_t tw, uint32_t th, uint32_t cout) {
    const unsigned long long tiles_x = (g.w + tw - 1) / tw;
    if (SPK_CONV_MTILES == 1 || SPK_CONV_MTILES == 2 || SPK_CONV_MTILES == 4)
        return (SPK_CONV_MTILES * cout <= 256u) ? SPK_CONV_MTILES : 1u;
    static const int sms = device_sms();
    for (uint32_t mt = 2; mt > 1; mt /= 2) {
        const unsigned long long ctas = tiles_x * ((g.h + mt * th - 1) / (mt * th)) * g.n;
        if (mt * cout <= 256u && ctas >= 4ull * static_cast<unsigned long long>(sms)) return mt;
    }
    return 1;
}

OutSpec out_spec(const NhwcView &y, const ConvEpilogue &epi) {
    OutSpec o{};
    o.out = static_cast<__nv_bfloat16 *>(y.ptr);
    o.out_ld = y.ld;
    o.bias = epi.bias;
    o.relu = epi.relu ? 1u : 0u;
    o.mask = static_cast<const __nv_bfloat16 *>(epi.mask.ptr);
    o.mask_ld = epi.mask.ld;
    o.pool = static_cast<__nv_bfloat16 *>(epi.pool);
    return o;
}

}  // namespace

cudaError_t conv_wait_probe(uint32_t *err, cudaStream_t stream) {
    k_wait_probe<<<1, 32, 0, stream>>>(err);
    return cudaGetLastError();
}

cudaError_t conv3x3_forward(const NhwcView &x, const void *w, uint32_t cout, const NhwcView &y, const ConvGeom &g,
                            const ConvEpilogue &epi, uint32_t *err, cudaStream_t stream) {
    if (x.channels == 0 || x.channels % 32u || cout == 0 || cout % 32u || cout > kMaxCout || y.channels != cout ||
        x.ld % 8u || y.ld % 8u || x.ld < x.channels || y.ld < y.channels || !aligned16(x.ptr) || !aligned16(y.ptr) ||
        !aligned16(w) || g.n == 0 || g.h == 0 || g.w == 0)
        return cudaErrorInvalidValue;
    if (epi.mask.ptr && (epi.mask.channels != cout || epi.mask.ld % 8u || !aligned16(epi.mask.ptr)))
        return cudaErrorInvalidValue;
    if (epi.pool && ((g.h | g.w) & 1u || !aligned16(epi.pool))) return cudaErrorInvalidValue;
    EncodeTiledFn enc = encode_fn();
    if (!enc) return cudaErrorNotSupported;
    // Tiles of 16 x 8 pixels (8 x 16 below 16 columns): a multiple of 8 columns, so that the row taps'
    // A operands start on 8-row swizzle atoms of the shared input box.
    const uint32_t tw = g.w >= 16u ? 16u : 8u;
    const uint32_t th = kTileM / tw;
    const uint32_t mt = conv_mtiles(g, tw, th, cout);
    const uint32_t rows = mt * th;
    CUtensorMap tmx, tmw;
    {
        const cuuint64_t dims[4] = {x.channels, g.w, g.h, g.n};
        const cuuint64_t strides[3] = {static_cast<cuuint64_t>(x.ld) * 2u, static_cast<cuuint64_t>(x.ld) * 2u * g.w,
                                       static_cast<cuuint64_t>(x.ld) * 2u * g.w * g.h};
        const cuuint32_t box[4] = {32u, tw, rows + 2u, 1u};
        const cuuint32_t es[4] = {1u, 1u, 1u, 1u};
        if (enc(&tmx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, x.ptr, dims, strides, box, es,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return cudaErrorInvalidValue;
    }
    {
        const cuuint64_t dims[2] = {9u * x.channels, cout};
        const cuuint64_t strides[1] = {9u * x.channels * 2u};
        const cuuint32_t box[2] = {32u, cout};
        const cuuint32_t es[2] = {1u, 1u};
        if (enc(&tmw, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(w), dims, strides, box, es,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return cudaErrorInvalidValue;
    }
    CUtensorMap tmy;
    {
        const cuuint64_t dims[4] = {cout, g.w, g.h, g.n};
        const cuuint64_t strides[3] = {static_cast<cuuint64_t>(y.ld) * 2u, static_cast<cuuint64_t>(y.ld) * 2u * g.w,
                                       static_cast<cuuint64_t>(y.ld) * 2u * g.w * g.h};
        const cuuint32_t box[4] = {32u, tw, th, 1u};
        const cuuint32_t es[4] = {1u, 1u, 1u, 1u};
        if (enc(&tmy, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, y.ptr, dims, strides, box, es,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return cudaErrorInvalidValue;
    }
    FwdParams P{};
    P.n = g.n;
    P.h = g.h;
    P.w = g.w;
    P.cin = x.channels;
    P.cout = cout;
    P.tw = tw;
    P.th = th;
    P.mt = mt;
    P.tiles_x = (g.w + tw - 1) / tw;
    P.tiles_y = (g.h + rows - 1) / rows;
    P.a_bytes = fwd_a_bytes(tw, rows);
    P.stage_bytes = fwd_stage_bytes(tw, rows, cout);
    // Ring depth: up to 4 stages within the stage budget, never more than the K blocks of a tile (3 per 32
    // channels). A smaller ring leaves room for more CTAs per SM.
    P.stages = std::max(2u, std::min({kStages, 3u * (x.channels / 32u), (kStageBudget * 1024u) / P.stage_bytes}));
    P.out_spec = out_spec(y, epi);
    // The staged tile (mt x 128 pixels x cout BF16) must fit in the ring it reuses.
    P.stage_out = (SPK_CONV_TMA_STORE && kTileM * 2u * mt * cout <= P.stages * P.stage_bytes) ? 1u : 0u;
    P.err = err;
    static std::once_flag attr;
    std::call_once(attr, [] {
        cudaFuncSetAttribute(k_conv_fwd<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem);
        cudaFuncSetAttribute(k_conv_fwd<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem);
    });
    const unsigned long long tiles = static_cast<unsigned long long>(P.tiles_x) * P.tiles_y * g.n;
    if (tiles > 0x7FFFFFFFull) return cudaErrorInvalidValue;
    const size_t smem = launch_smem(P.stages * P.stage_bytes + 1024 + 256, tmem_columns(mt * cout));
    if (smem == 0) return cudaErrorInvalidConfiguration;
    auto *kern = P.out_spec.pool ? k_conv_fwd<true> : k_conv_fwd<false>;
    kern<<<static_cast<unsigned>(tiles), kFwdThreads, smem, stream>>>(tmx, tmw, tmy, P);
    return cudaGetLastError();
}

#ifndef SPK_CONV_WGRAD_TMA
#define SPK_CONV_WGRAD_TMA 1  // 1: weight gradient from TMA-loaded MN-major operands; 0: thread-gathered K-major tiles
#endif

namespace {
cudaError_t wgrad_tma(const NhwcView &x, const NhwcView &dy, float *dw, const ConvGeom &g, uint32_t *err,
                      cudaStream_t stream) {
    EncodeTiledFn enc = encode_fn();
    if (!enc) return cudaErrorNotSupported;
    WgradTmaParams P{};
    P.n = g.n;
    P.h = g.h;
    P.w = g.w;
    P.cin = x.channels;
    P.cout = dy.channels;
    P.tw = g.w >= 16u ? 16u : 8u;
    P.th = kWgtPix / P.tw;
    P.tiles_x = (g.w + P.tw - 1) / P.tw;
    P.tiles_y = (g.h + P.th - 1) / P.th;
    P.krows = 9u * P.cin;
    P.m_tiles = (P.krows + kTileM - 1) / kTileM;
    const unsigned long long ktotal = static_cast<unsigned long long>(P.tiles_x) * P.tiles_y * g.n;
    if (ktotal > 0x7FFFFFFFull) return cudaErrorInvalidValue;
    P.ktotal = static_cast<uint32_t>(ktotal);
    P.dw = dw;
    P.err = err;
    P.stage_bytes = wgt_stage_bytes(P.cout);
    P.stages = std::min<uint32_t>(kWgtStages, (200u * 1024u) / P.stage_bytes);
    if (P.stages < 2) return cudaErrorInvalidConfiguration;
    CUtensorMap tmx, tmdy;
    const NhwcView *views[2] = {&x, &dy};
    CUtensorMap *maps[2] = {&tmx, &tmdy};
    for (int k = 0; k < 2; ++k) {
        const NhwcView &v = *views[k];
        const cuuint64_t dims[4] = {v.channels, g.w, g.h, g.n};
        const cuuint64_t strides[3] = {static_cast<cuuint64_t>(v.ld) * 2u, static_cast<cuuint64_t>(v.ld) * 2u * g.w,
                                       static_cast<cuuint64_t>(v.ld) * 2u * g.w * g.h};
        const cuuint32_t box[4] = {32u, P.tw, P.th, 1u};
        const cuuint32_t es[4] = {1u, 1u, 1u, 1u};
        if (enc(maps[k], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, v.ptr, dims, strides, box, es,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return cudaErrorInvalidValue;
    }
    // About two CTAs per SM in total, at least 8 K blocks each (fewer splits: fewer atomic partial sums).
    static const int sms = device_sms();
    unsigned long long splits = std::max<unsigned long long>(1ull, (2ull * sms) / P.m_tiles);
    splits = std::min<unsigned long long>(splits, (ktotal + 7) / 8);
    splits = std::max<unsigned long long>(splits, 1ull);
    P.kblocks = static_cast<uint32_t>((ktotal + splits - 1) / splits);
    splits = (ktotal + P.kblocks - 1) / P.kblocks;
    const size_t smem = launch_smem(P.stages * P.stage_bytes + kWgtSlack + 1024 + 256, tmem_columns(P.cout));
    if (smem == 0) return cudaErrorInvalidConfiguration;
    static std::once_flag attr;
    std::call_once(attr, [] {
        cudaFuncSetAttribute(k_conv_wgrad_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem);
    });
    k_conv_wgrad_tma<<<static_cast<unsigned>(splits * P.m_tiles), 128, smem, stream>>>(tmx, tmdy, P);
    return cudaGetLastError();
}
}  // namespace

cudaError_t conv3x3_wgrad(const NhwcView &x, const NhwcView &dy, float *dw, const ConvGeom &g, uint32_t *err,
                          cudaStream_t stream) {
    if (x.channels == 0 || x.channels % 32u || dy.channels == 0 || dy.channels % 32u || dy.channels > kMaxCout ||
        x.ld % 8u || dy.ld % 8u || !aligned16(x.ptr) || !aligned16(dy.ptr) || g.n == 0 || g.h == 0 || g.w == 0)
        return cudaErrorInvalidValue;
    if (SPK_CONV_WGRAD_TMA) return wgrad_tma(x, dy, dw, g, err, stream);
    WgradParams P{};
    P.n = g.n;
    P.h = g.h;
    P.w = g.w;
    P.cin = x.channels;
    P.cout = dy.channels;
    P.x = static_cast<const __nv_bfloat16 *>(x.ptr);
    P.x_ld = x.ld;
    P.dy = static_cast<const __nv_bfloat16 *>(dy.ptr);
    P.dy_ld = dy.ld;
    P.dw = dw;
    P.npix = static_cast<unsigned long long>(g.n) * g.h * g.w;
    P.row_tiles = (9u * P.cin + kTileM - 1) / kTileM;
    P.err = err;
    const unsigned long long kblocks_total = (P.npix + kWgKPix - 1) / kWgKPix;
    // About 4 CTAs per SM in total, at least 8 K blocks each.
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    unsigned long long splits = std::max<unsigned long long>(1ull, (4ull * sms) / P.row_tiles);
    splits = std::min<unsigned long long>(splits, (kblocks_total + 7) / 8);
    splits = std::max<unsigned long long>(splits, 1ull);
    P.kblocks = static_cast<uint32_t>((kblocks_total + splits - 1) / splits);
    splits = (kblocks_total + P.kblocks - 1) / P.kblocks;
    const size_t smem = launch_smem(kWgStages * wg_stage_bytes(P.cout) + 1024 + 256, tmem_columns(P.cout));
    if (smem == 0) return cudaErrorInvalidConfiguration;
    static std::once_flag attr;
    std::call_once(attr, [] {
        cudaFuncSetAttribute(k_conv_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem);
    });
    k_conv_wgrad<<<static_cast<unsigned>(splits * P.row_tiles), 128, smem, stream>>>(P);
    return cudaGetLastError();
}

cudaError_t conv3x3_transpose_weights(const void *w, void *wt, uint32_t cout, uint32_t cin, cudaStream_t stream) {
    const uint32_t n = cout * cin * 9u;
    k_transpose_weights<<<(n + 255) / 256, 256, 0, stream>>>(static_cast<const __nv_bfloat16 *>(w),
                                                            static_cast<__nv_bfloat16 *>(wt), cout, cin);
    return cudaGetLastError();
}

}  // namespace spk
