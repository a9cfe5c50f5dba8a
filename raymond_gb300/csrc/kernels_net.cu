// The learned denoiser's kernels: 3×3 convolutions as implicit GEMMs on the
// fifth-generation tensor cores (tcgen05.mma, BF16 operands, FP32
// accumulators in tensor memory) for the forward pass, the input gradient
// and the weight gradient, plus the element-wise kernels around them
// (input features, 2×2 pooling, the gradient split at skip connections,
// the loss, Adam and the display composite).
//
// Tensors are NHWC BF16 with a channel stride that is a multiple of 8, so a
// 16-byte cp.async moves 8 channels of one pixel. Weights are [cout][9][cin]
// (tap-major rows, cin a multiple of 16).
//
// GEMM views (M × N × K):
//   forward        M = pixels,    N = cout, K = 9·cin   A K-major  (input taps),   B K-major  (weights)
//   input grad     M = pixels,    N = cin,  K = 9·cout  A K-major  (flipped taps), B MN-major (weights)
//   weight grad    M = 9·cin + 1, N = cout, K = pixels  A MN-major (shifted input), B MN-major (dy)
// Three kernels: k_conv_halo (forward and input gradient on 8×16-pixel
// tiles whose halo is staged once per channel chunk and read by all nine
// taps; the default), k_conv_ws (the same two on 128-pixel row tiles whose
// taps are gathered as im2col rows) and k_conv (the weight gradient, split
// over pixels, FP32 atomics). The weight gradient's extra row is all ones,
// so its result row is the bias gradient. A kernel that waits too long on
// its mbarrier records NET_STATUS_TIMEOUT and returns after freeing its
// tensor memory.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdint>
#include <cstring>

#include "dev_tcgen05.cuh"
#include "dev_tma.cuh"
#include "net.cuh"

namespace rmd {
namespace net {

using bf16 = __nv_bfloat16;

constexpr int kThreads = 256;
constexpr int kStages = 3;
constexpr int kTileM = 128;
constexpr int kChunk = 64;                       // K elements per stage
constexpr uint32_t kABytes = kTileM * kChunk * 2;  // 16 KB
constexpr uint32_t kLBO = 128;                   // K-direction core-matrix stride
constexpr uint32_t kSBO = 1024;                  // M/N-direction core-matrix stride (8 k-groups)

__host__ __device__ inline uint32_t tmem_cols_for(int n) {
    return n <= 32 ? 32u : n <= 64 ? 64u : n <= 128 ? 128u : n <= 256 ? 256u : 512u;
}
__host__ __device__ inline uint32_t stage_bytes_for(int n) { return kABytes + uint32_t(n) * 128u; }

struct Pixel {
    int img, y, x;
    bool valid;
};
__device__ __forceinline__ Pixel decode(int p, int total, int h, int w) {
    Pixel px;
    px.valid = p < total;
    const int hw = h * w;
    px.img = p / hw;
    const int r = p - px.img * hw;
    px.y = r / w;
    px.x = r - px.y * w;
    return px;
}

// Address of channel c at pixel (img, yy, xx) of the level, read from the
// concatenated sources; false outside the image.
__device__ __forceinline__ bool source_at(const ConvArgs& a, int img, int yy, int xx, int c, const bf16*& ptr) {
    if (yy < 0 || xx < 0 || yy >= a.h || xx >= a.w) return false;
    const ConvSrc& s = c < a.src[0].channels ? a.src[0] : a.src[1];
    const int cc = c < a.src[0].channels ? c : c - a.src[0].channels;
    const int sh = s.shift, sw = a.w >> sh, shh = a.h >> sh;
    const size_t pix = (size_t(img) * shh + (yy >> sh)) * sw + (xx >> sh);
    ptr = s.ptr + pix * size_t(s.stride) + cc;
    return true;
}

__device__ __forceinline__ float slope(float v) { return v > 0.0f ? 1.0f : kLeak; }

__device__ __forceinline__ void unpack8(uint4 u, float* f) {
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float2 t = __bfloat1622float2(h[i]);
        f[2 * i] = t.x;
        f[2 * i + 1] = t.y;
    }
}
__device__ __forceinline__ uint4 pack8(const float* f) {
    uint4 u;
    __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&u);
#pragma unroll
    for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
    return u;
}

template <int MODE>
__device__ __forceinline__ void load_chunk(const ConvArgs& a, int N, int K, int m0, int k0, int kend, unsigned char* sa,
                                           unsigned char* sb, const Pixel& row_px, int total_pixels) {
    const int tid = threadIdx.x;
    if (MODE == FWD || MODE == BWD_DATA) {
        // A: thread owns one pixel row, four of the eight k-groups.
        const int r = tid & (kTileM - 1);
        const int cdiv = MODE == FWD ? a.cin : a.cout;
        for (int j = 0; j < 4; ++j) {
            const int g = (tid >> 7) + 2 * j;
            const int k = k0 + 8 * g;
            if (k >= kend) continue;
            const int tap = k / cdiv;
            const int c = k - tap * cdiv;
            const int ty = tap / 3, tx = tap - 3 * ty;
            const bf16* src = a.wt;
            bool ok = false;
            if (row_px.valid) {
                if (MODE == FWD) {
                    ok = source_at(a, row_px.img, row_px.y + ty - 1, row_px.x + tx - 1, c, src);
                } else {
                    const int yy = row_px.y - (ty - 1), xx = row_px.x - (tx - 1);
                    if (yy >= 0 && xx >= 0 && yy < a.h && xx < a.w) {
                        src = a.dy + ((size_t(row_px.img) * a.h + yy) * a.w + xx) * size_t(a.dy_stride) + c;
                        ok = true;
                    }
                }
            }
            tc::cp_async16(sa + tc::core_offset(r, g, 8), ok ? src : a.wt, ok ? 16u : 0u);
        }
        // B
        if (MODE == FWD) {
            for (int idx = tid; idx < N * 8; idx += kThreads) {
                const int row = idx >> 3, g = idx & 7;
                const int k = k0 + 8 * g;
                if (k < kend) tc::cp_async16(sb + tc::core_offset(row, g, 8), a.wt + size_t(row) * K + k, 16u);
            }
        } else {
            const int kin = 9 * a.cin;
            for (int idx = tid; idx < (N >> 3) * kChunk; idx += kThreads) {
                const int kl = idx & (kChunk - 1), ng = idx >> 6;
                const int k = k0 + kl;
                if (k >= kend) continue;
                const int tap = k / a.cout;
                const int co = k - tap * a.cout;
                tc::cp_async16(sb + ng * kSBO + kl * 16, a.wt + size_t(co) * kin + tap * a.cin + 8 * ng, 16u);
            }
        }
    } else {
        // Weight gradient. A: thread owns one pixel (k) and four 8-row groups.
        const int kl = tid & (kChunk - 1);
        const Pixel px = decode(k0 + kl, kend, a.h, a.w);
        const int rows = 9 * a.cin;
        for (int j = 0; j < 4; ++j) {
            const int mg = (tid >> 6) + 4 * j;
            const int m = m0 + 8 * mg;
            unsigned char* dst = sa + mg * kSBO + kl * 16;
            if (m < rows) {
                const int tap = m / a.cin;
                const int ci = m - tap * a.cin;
                const int ty = tap / 3, tx = tap - 3 * ty;
                const bf16* src = a.wt;
                const bool ok = px.valid && source_at(a, px.img, px.y + ty - 1, px.x + tx - 1, ci, src);
                tc::cp_async16(dst, ok ? src : a.wt, ok ? 16u : 0u);
            } else {
                uint4 v = make_uint4(0u, 0u, 0u, 0u);
                if (m == rows && px.valid) v.x = 0x3F80u;  // bf16 1.0 in the group's first row
                *reinterpret_cast<uint4*>(dst) = v;
            }
        }
        // B: dy, 8 output channels of one pixel per piece.
        for (int idx = tid; idx < (N >> 3) * kChunk; idx += kThreads) {
            const int l = idx & (kChunk - 1), ng = idx >> 6;
            const int p = k0 + l;
            const bool ok = p < kend;
            tc::cp_async16(sb + ng * kSBO + l * 16, ok ? a.dy + size_t(p) * a.dy_stride + 8 * ng : a.dy, ok ? 16u : 0u);
        }
    }
    (void)total_pixels;
}

template <int MODE>
__global__ void __launch_bounds__(kThreads) k_conv(ConvArgs a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t bars[kStages];
    __shared__ uint32_t tslot;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int pixels = a.n * a.h * a.w;
    const int N = MODE == BWD_DATA ? a.cin : a.cout;
    const int K = MODE == FWD ? 9 * a.cin : MODE == BWD_DATA ? 9 * a.cout : pixels;
    const uint32_t sbytes = stage_bytes_for(N);
    const uint32_t tcols = tmem_cols_for(N);
    const int m0 = blockIdx.x * kTileM;
    int kbeg = 0, kend = K;
    if (MODE == BWD_WEIGHT) {
        kbeg = blockIdx.y * a.pixels_per_cta;
        kend = min(K, kbeg + a.pixels_per_cta);
    }
    const int nchunks = (kend - kbeg + kChunk - 1) / kChunk;

    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) tc::mbar_init(&bars[s], 1);
        tc::fence_barrier_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(&tslot, tcols);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before_sync();
    __syncthreads();
    tc::tc_fence_after_sync();
    const uint32_t tbase = tslot;

    Pixel row_px{0, 0, 0, false};
    if (MODE != BWD_WEIGHT) row_px = decode(m0 + (tid & (kTileM - 1)), pixels, a.h, a.w);

    uint32_t idesc = tc::idesc_bf16(kTileM, N);
    if (MODE == BWD_DATA) idesc |= 1u << 16;
    if (MODE == BWD_WEIGHT) idesc |= (1u << 15) | (1u << 16);

    for (int c = 0; c < kStages - 1; ++c) {
        if (c < nchunks) {
            unsigned char* st = smem + c * sbytes;
            load_chunk<MODE>(a, N, K, m0, kbeg + c * kChunk, kend, st, st + kABytes, row_px, pixels);
        }
        tc::cp_async_commit();
    }

    bool failed = false;
    for (int i = 0; i < nchunks; ++i) {
        asm volatile("cp.async.wait_group %0;" ::"n"(kStages - 2) : "memory");
        tc::fence_proxy_async_smem();
        if (__syncthreads_or(failed)) {
            failed = true;
            break;
        }
        const int s = i % kStages;
        if (tid == 0) {
            tc::tc_fence_after_sync();
            const uint32_t sa = tc::smem_u32(smem + s * sbytes);
            const uint32_t sb = sa + kABytes;
            const int kleft = kend - (kbeg + i * kChunk);
            const int slices = min(kChunk, kleft + 15) / 16;
            for (int j = 0; j < slices; ++j) {
                const uint64_t ad = tc::smem_desc(sa + j * 256, kLBO, kSBO);
                const uint64_t bd = tc::smem_desc(sb + j * 256, kLBO, kSBO);
                tc::mma_bf16(tbase, ad, bd, idesc, (i > 0 || j > 0) ? 1u : 0u);
            }
            tc::mma_commit(&bars[s]);
        }
        const int next = i + kStages - 1;
        if (next < nchunks) {
            if (i >= 1) {
                const int prev = i - 1;
                if (!tc::mbar_wait(&bars[prev % kStages], (prev / kStages) & 1)) failed = true;
            }
            if (!failed) {
                unsigned char* st = smem + (next % kStages) * sbytes;
                load_chunk<MODE>(a, N, K, m0, kbeg + next * kChunk, kend, st, st + kABytes, row_px, pixels);
            }
        }
        tc::cp_async_commit();
    }
    tc::cp_async_wait_all();

    // Completion of the last chunk's MMAs (and so of all of them).
    bool done = false;
    if (!failed) {
        const int last = nchunks - 1;
        done = tc::mbar_wait(&bars[last % kStages], (last / kStages) & 1);
    }
    const bool ok = !__syncthreads_or(!done);
    if (!ok && tid == 0) atomicOr(a.status, NET_STATUS_TIMEOUT);
    tc::tc_fence_after_sync();

    if (ok) {
        const int quarter = warp & 3;
        const int row = m0 + 32 * quarter + lane;
        const uint32_t lane_addr = tbase + (uint32_t(32 * quarter) << 16);
        for (int c = (warp >> 2) * 16; c < N; c += 32) {
            float v[16];
            tc::tmem_ld16(lane_addr + uint32_t(c), v);
            if (MODE == FWD) {
                if (row < pixels) {
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        float t = v[i] + a.bias[c + i];
                        if (a.act) t = t > 0.0f ? t : kLeak * t;
                        v[i] = t;
                    }
                    if (a.out_f32) {
                        float4* o = reinterpret_cast<float4*>(a.out_f32 + size_t(row) * a.out_stride + c);
#pragma unroll
                        for (int i = 0; i < 4; ++i) o[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
                    } else {
                        uint4* o = reinterpret_cast<uint4*>(a.out + size_t(row) * a.out_stride + c);
                        o[0] = pack8(v);
                        o[1] = pack8(v + 8);
                    }
                }
            } else if (MODE == BWD_DATA) {
                if (row < pixels) {
                    if (a.mask) {
                        const uint4* mk = reinterpret_cast<const uint4*>(a.mask + size_t(row) * a.mask_stride + c);
                        float mv[16];
                        unpack8(mk[0], mv);
                        unpack8(mk[1], mv + 8);
#pragma unroll
                        for (int i = 0; i < 16; ++i) v[i] *= slope(mv[i]);
                    }
                    uint4* o = reinterpret_cast<uint4*>(a.out + size_t(row) * a.out_stride + c);
                    o[0] = pack8(v);
                    o[1] = pack8(v + 8);
                }
            } else {
                const int rows = 9 * a.cin;
                if (row < rows) {
#pragma unroll
                    for (int i = 0; i < 16; ++i) atomicAdd(a.dw + size_t(c + i) * rows + row, v[i]);
                } else if (row == rows) {
#pragma unroll
                    for (int i = 0; i < 16; ++i) atomicAdd(a.db + c + i, v[i]);
                }
            }
        }
    } else {
        // MMAs may still be in flight: give them a bounded time before the
        // tensor memory is released.
        if (tid == 0) {
            for (int s = 0; s < kStages; ++s) tc::mbar_wait(&bars[s], 0);
        }
    }
    tc::tc_fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::tc_fence_after_sync();
        tc::tmem_dealloc(tbase, tcols);
    }
}

// ---------------------------------------------------------------- warp-specialised forward / input gradient

// Roles of k_conv_ws's 13 warps: 0-3 drain accumulators (warp w reads the
// tensor-memory lanes 32·w…), 4-11 load stages, 12 issues the MMAs.
constexpr int kWsEpilogueWarps = 4, kWsLoadWarps = 8;
constexpr int kWsLoaders = kWsLoadWarps * 32;
constexpr int kWsMmaWarp = kWsEpilogueWarps + kWsLoadWarps;
constexpr int kWsThreads = (kWsMmaWarp + 1) * 32;

// Stage loads for loader thread p (0..255): A rows as k_conv's load_chunk
// (row p & 127, four k-groups), B pieces strided over the loaders.
template <int MODE>
__device__ __forceinline__ void ws_load(const ConvArgs& a, int p, int N, int K, const Pixel& px, int k0,
                                        unsigned char* sa, unsigned char* sb) {
    const int r = p & (kTileM - 1);
    const int cdiv = MODE == FWD ? a.cin : a.cout;
    for (int j = 0; j < 4; ++j) {
        const int g = (p >> 7) + 2 * j;
        const int k = k0 + 8 * g;
        if (k >= K) continue;
        const int tap = k / cdiv;
        const int c = k - tap * cdiv;
        const int ty = tap / 3, tx = tap - 3 * ty;
        const bf16* src = a.wt;
        bool ok = false;
        if (px.valid) {
            if (MODE == FWD) {
                ok = source_at(a, px.img, px.y + ty - 1, px.x + tx - 1, c, src);
            } else {
                const int yy = px.y - (ty - 1), xx = px.x - (tx - 1);
                if (yy >= 0 && xx >= 0 && yy < a.h && xx < a.w) {
                    src = a.dy + ((size_t(px.img) * a.h + yy) * a.w + xx) * size_t(a.dy_stride) + c;
                    ok = true;
                }
            }
        }
        tc::cp_async16(sa + tc::core_offset(r, g, 8), ok ? src : a.wt, ok ? 16u : 0u);
    }
    if (MODE == FWD) {
        for (int idx = p; idx < N * 8; idx += kWsLoaders) {
            const int row = idx >> 3, g = idx & 7;
            const int k = k0 + 8 * g;
            if (k < K) tc::cp_async16(sb + tc::core_offset(row, g, 8), a.wt + size_t(row) * K + k, 16u);
        }
    } else {
        const int kin = 9 * a.cin;
        for (int idx = p; idx < (N >> 3) * kChunk; idx += kWsLoaders) {
            const int kl = idx & (kChunk - 1), ng = idx >> 6;
            const int k = k0 + kl;
            if (k >= K) continue;
            const int tap = k / a.cout;
            const int co = k - tap * a.cout;
            tc::cp_async16(sb + ng * kSBO + kl * 16, a.wt + size_t(co) * kin + tap * a.cin + 8 * ng, 16u);
        }
    }
}

// Forward and input gradient as persistent, warp-specialised CTAs over
// pixel tiles (blockIdx.x, + gridDim.x, …). Loaders fill a ring of stages
// and signal each with cp.async's own mbarrier arrival; the MMA thread
// consumes stages into one of two tensor-memory accumulators and frees each
// stage by tcgen05.commit; the epilogue warps drain an accumulator while the
// next tile accumulates in the other. Every wait is bounded: a wait that
// runs out records NET_STATUS_TIMEOUT and its role stops, so every role
// reaches the end (the others' waits run out in turn) and the tensor memory
// is freed.
template <int MODE>
__global__ void __launch_bounds__(kWsThreads) k_conv_ws(ConvArgs a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t full[kStages], empty[kStages], acc_full[2], acc_empty[2];
    __shared__ uint32_t tslot;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int pixels = a.n * a.h * a.w;
    const int N = MODE == FWD ? a.cout : a.cin;
    const int K = MODE == FWD ? 9 * a.cin : 9 * a.cout;
    const uint32_t sbytes = stage_bytes_for(N);
    const uint32_t tcols = tmem_cols_for(2 * N);
    const int ntiles = (pixels + kTileM - 1) / kTileM;
    const int nchunks = (K + kChunk - 1) / kChunk;
    const int my_tiles = int(blockIdx.x) < ntiles ? (ntiles - 1 - int(blockIdx.x)) / int(gridDim.x) + 1 : 0;

    if (tid == 0) {
        for (int st = 0; st < kStages; ++st) {
            tc::mbar_init(&full[st], kWsLoaders);
            tc::mbar_init(&empty[st], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&acc_full[b], 1);
            tc::mbar_init(&acc_empty[b], kWsEpilogueWarps);
        }
        tc::fence_barrier_init();
    }
    if (warp == kWsMmaWarp) {
        tc::tmem_alloc(&tslot, tcols);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before_sync();
    __syncthreads();
    tc::tc_fence_after_sync();
    const uint32_t tbase = tslot;
    bool ok = true;

    if (warp >= kWsEpilogueWarps && warp < kWsMmaWarp) {
        // ---- loaders
        const int p = tid - kWsEpilogueWarps * 32;
        for (int i = 0; i < my_tiles && ok; ++i) {
            const int m0 = (int(blockIdx.x) + i * int(gridDim.x)) * kTileM;
            const Pixel px = decode(m0 + (p & (kTileM - 1)), pixels, a.h, a.w);
            for (int c = 0; c < nchunks; ++c) {
                const int j = i * nchunks + c, s = j % kStages;
                if (!tc::mbar_wait(&empty[s], ((j / kStages) & 1) ^ 1)) {
                    ok = false;
                    break;
                }
                unsigned char* st = smem + s * sbytes;
                ws_load<MODE>(a, p, N, K, px, c * kChunk, st, st + kABytes);
                tc::cp_async_arrive(&full[s]);
            }
        }
        tc::cp_async_wait_all();
    } else if (warp == kWsMmaWarp) {
        // ---- MMA issue (one thread)
        if (lane == 0) {
            uint32_t idesc = tc::idesc_bf16(kTileM, N);
            if (MODE == BWD_DATA) idesc |= 1u << 16;
            for (int i = 0; i < my_tiles && ok; ++i) {
                const int b = i & 1;
                if (!tc::mbar_wait(&acc_empty[b], ((i >> 1) & 1) ^ 1)) {
                    ok = false;
                    break;
                }
                tc::tc_fence_after_sync();
                const uint32_t acc = tbase + uint32_t(b * N);
                for (int c = 0; c < nchunks; ++c) {
                    const int j = i * nchunks + c, s = j % kStages;
                    if (!tc::mbar_wait(&full[s], (j / kStages) & 1)) {
                        ok = false;
                        break;
                    }
                    // the loaders' cp.async writes, seen by the tensor core's proxy
                    tc::fence_proxy_async_smem();
                    tc::tc_fence_after_sync();
                    const uint32_t sa = tc::smem_u32(smem + s * sbytes);
                    const uint32_t sb = sa + kABytes;
                    const int slices = min(kChunk, K - c * kChunk) / 16;
                    for (int q = 0; q < slices; ++q) {
                        const uint64_t ad = tc::smem_desc(sa + q * 256, kLBO, kSBO);
                        const uint64_t bd = tc::smem_desc(sb + q * 256, kLBO, kSBO);
                        tc::mma_bf16(acc, ad, bd, idesc, (c > 0 || q > 0) ? 1u : 0u);
                    }
                    tc::mma_commit(&empty[s]);
                }
                if (!ok) break;
                tc::mma_commit(&acc_full[b]);
            }
        }
        __syncwarp();
    } else {
        // ---- epilogue: warp w reads tensor-memory lanes 32·w..32·w+31
        for (int i = 0; i < my_tiles && ok; ++i) {
            const int b = i & 1;
            if (!tc::mbar_wait(&acc_full[b], (i >> 1) & 1)) {
                ok = false;
                break;
            }
            tc::tc_fence_after_sync();
            const int row = (int(blockIdx.x) + i * int(gridDim.x)) * kTileM + 32 * warp + lane;
            const uint32_t lane_addr = tbase + (uint32_t(32 * warp) << 16) + uint32_t(b * N);
            for (int c = 0; c < N; c += 16) {
                float v[16];
                tc::tmem_ld16(lane_addr + uint32_t(c), v);  // the whole warp, every row
                if (row < pixels) {
                    if (MODE == FWD) {
#pragma unroll
                        for (int q = 0; q < 16; ++q) {
                            float t = v[q] + a.bias[c + q];
                            if (a.act) t = t > 0.0f ? t : kLeak * t;
                            v[q] = t;
                        }
                    } else if (a.mask) {
                        const uint4* mk = reinterpret_cast<const uint4*>(a.mask + size_t(row) * a.mask_stride + c);
                        float mv[16];
                        unpack8(mk[0], mv);
                        unpack8(mk[1], mv + 8);
#pragma unroll
                        for (int q = 0; q < 16; ++q) v[q] *= slope(mv[q]);
                    }
                    if (MODE == FWD && a.out_f32) {
                        float4* o = reinterpret_cast<float4*>(a.out_f32 + size_t(row) * a.out_stride + c);
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                    } else {
                        uint4* o = reinterpret_cast<uint4*>(a.out + size_t(row) * a.out_stride + c);
                        o[0] = pack8(v);
                        o[1] = pack8(v + 8);
                    }
                }
            }
            tc::tc_fence_before_sync();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&acc_empty[b]);
        }
    }
    if (!ok) atomicOr(a.status, NET_STATUS_TIMEOUT);
    tc::tc_fence_before_sync();
    __syncthreads();
    if (warp == kWsMmaWarp) {
        tc::tc_fence_after_sync();
        tc::tmem_dealloc(tbase, tcols);
    }
}

// ---------------------------------------------------------------- halo tiles, resident weights

// A tile is 8 × 16 output pixels of one image: M row m = 8·py + px, so each
// 8-row core matrix is one tile row. Its halo of 10 × 18 pixels is staged
// once per chunk of kc channels, as kc/8 columns of 180 16-byte pieces
// (pixel (hy, hx) of the halo at (10·hy + hx)·16). Tap (ty, tx)'s A operand
// is that column read from pixel ty·10 + tx with 160 bytes between core
// matrices, so the nine taps share one load instead of loading the input
// nine times. The weights are blocks per (chunk, tap) of N × kc in
// core-matrix order: all of them in shared memory for the CTA's life when
// they fit, else the nine blocks of a chunk brought with each stage.

constexpr int kTileW = 8, kTileH = 16;
constexpr int kHaloW = kTileW + 2, kHaloH = kTileH + 2, kHaloPx = kHaloW * kHaloH;
constexpr uint32_t kHaloBox = kHaloPx * 16;     // one 8-channel column: 2880 B
constexpr uint32_t kHaloCol = 23 * 128;         // its slot, 128-byte aligned for the tensor copy
constexpr uint32_t kHaloRowStep = kHaloW * 16;  // between the tile's rows (core matrices along M)
// An upsampled source's halo column comes from a 6 × 10 box of the
// half-resolution tensor (960 B, in a 1 KB slot), widened in shared memory.
constexpr int kUpW = 6, kUpH = 10;
constexpr uint32_t kUpBox = kUpW * kUpH * 16, kUpCol = 1024;
constexpr int kHaloMaxStages = 8;
// Roles of k_conv_halo's 12 warps: 0-3 epilogue (as k_conv_ws); 4 issues
// the tensor copies (lane 0), running ahead over free stages; 5-10 widen
// (where a source is upsampled, thread p < 180 of them widens halo pixel p
// of its columns once they land); 11 issues the MMAs. Warps 4-10 load the
// resident weights first.
constexpr int kHaloIssueWarp = kWsEpilogueWarps, kHaloWidenWarps = 6;
constexpr int kHaloLoadWarps = 1 + kHaloWidenWarps, kHaloLoaders = kHaloLoadWarps * 32;
constexpr int kHaloMmaWarp = kWsEpilogueWarps + kHaloLoadWarps;
constexpr int kHaloThreads = (kHaloMmaWarp + 1) * 32;
static_assert(kHaloWidenWarps * 32 >= kHaloPx, "one widening thread per halo pixel");

struct HaloPlan {
    int up;            // bit k: source k is upsampled (its columns are widened from half resolution)
    int stream;        // weights too large to stay: each stage brings its chunk's nine blocks
    int kc;            // K-side channels per stage (16, 32 or 64)
    int nchunks;       // ceil(K-side channels / kc)
    int stages;        // 2 … kHaloMaxStages
    uint32_t up_off;   // in a stage: the half-resolution boxes, after the kc/8 halo columns
    uint32_t b_off;    // in a stage (streamed weights): the nine weight blocks, after the boxes
    uint32_t a_bytes;  // one stage: kc/8 halo columns of kHaloCol bytes (+ boxes, + weight blocks)
    uint32_t b_block;  // weights of one (chunk, tap): N · kc · 2 bytes
    uint32_t b_bytes;  // resident weights: nchunks · 9 · b_block (0 when streamed)
};

// The weights into shared memory (loader thread p of kHaloLoaders): FWD as
// K-major blocks (row co, k = ci within the chunk), BWD_DATA as MN-major
// blocks (n = ci, k = co within the chunk), both with 16·kc bytes between
// 8-row groups and 128 between 8-column groups.
template <int MODE>
__device__ __forceinline__ void halo_load_weights(const ConvArgs& a, const HaloPlan& hp, int p, unsigned char* sb) {
    const int cin8 = a.cin >> 3;
    const int pieces = a.cout * 9 * cin8;  // 16-byte pieces of [cout][9][cin]
    for (int i = p; i < pieces; i += kHaloLoaders) {
        const int co = i / (9 * cin8);
        const int r = i - co * 9 * cin8;
        const int t = r / cin8, c8 = r - t * cin8;
        const bf16* src = a.wt + (size_t(co) * 9 + t) * a.cin + 8 * c8;
        uint32_t off;
        if (MODE == FWD) {
            const int ci = 8 * c8, c = ci / hp.kc, g = (ci - c * hp.kc) >> 3;
            off = uint32_t(c * 9 + t) * hp.b_block + uint32_t(((co >> 3) * (hp.kc >> 3) + g) * 128 + (co & 7) * 16);
        } else {
            const int c = co / hp.kc, kl = co - c * hp.kc;
            off = uint32_t(c * 9 + t) * hp.b_block + uint32_t(c8 * 16 * hp.kc + kl * 16);
        }
        tc::cp_async16(sb + off, src, 16u);
    }
}

// Forward and input gradient over halo tiles: the roles, rings and bounded
// waits of k_conv_ws, with the A stages holding halos and the weights
// loaded once. Tiles (img, row of tiles, column) in row-major order, so CTAs
// that run at the same time share halo rows in L2. A halo column comes as
// one tensor copy (box of 8 channels × 10 × 18 pixels, zero outside the
// image) from map0 (source 0, or dy) or map1 (source 1); an upsampled
// source's map is of its half-resolution tensor. Streamed weights come as
// one copy per tap from mapw, whose box is a (chunk, tap) block already in
// core-matrix order.
template <int MODE>
__global__ void __launch_bounds__(kHaloThreads, 3)
    k_conv_halo(ConvArgs a, HaloPlan hp, const __grid_constant__ CUtensorMap map0,
                const __grid_constant__ CUtensorMap map1, const __grid_constant__ CUtensorMap mapw) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t full[kHaloMaxStages], empty[kHaloMaxStages], upb[kHaloMaxStages], acc_full[2], acc_empty[2];
    __shared__ uint32_t tslot;
    __shared__ __align__(16) float sbias[256];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int N = MODE == FWD ? a.cout : a.cin;
    const int CK = MODE == FWD ? a.cin : a.cout;  // K-side channels of one tap
    const uint32_t tcols = tmem_cols_for(2 * N);
    const int tiles_x = (a.w + kTileW - 1) / kTileW, tiles_y = (a.h + kTileH - 1) / kTileH;
    const int per_img = tiles_x * tiles_y;
    const int ntiles = a.n * per_img;
    const int my_tiles = int(blockIdx.x) < ntiles ? (ntiles - 1 - int(blockIdx.x)) / int(gridDim.x) + 1 : 0;
    const int S = hp.stages;
    unsigned char* sb = smem;
    unsigned char* sa0 = smem + hp.b_bytes;

    if (tid == 0) {
        for (int st = 0; st < S; ++st) {
            tc::mbar_init(&full[st], hp.up ? kHaloWidenWarps + 1 : 1);
            tc::mbar_init(&empty[st], 1);
            tc::mbar_init(&upb[st], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&acc_full[b], 1);
            tc::mbar_init(&acc_empty[b], kWsEpilogueWarps);
        }
        tc::fence_barrier_init();
    }
    if (!hp.stream && warp >= kWsEpilogueWarps && warp < kHaloMmaWarp) {
        halo_load_weights<MODE>(a, hp, tid - kWsEpilogueWarps * 32, sb);
        tc::cp_async_wait_all();
        tc::fence_proxy_async_smem();
    }
    if (MODE == FWD && tid < N) sbias[tid] = a.bias[tid];
    if (warp == kHaloMmaWarp) {
        tc::tmem_alloc(&tslot, tcols);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before_sync();
    __syncthreads();
    tc::tc_fence_after_sync();
    const uint32_t tbase = tslot;
    bool ok = true;

    const int c0 = MODE == FWD ? a.src[0].channels : CK;
    if (warp == kHaloIssueWarp) {
        // ---- tensor copies (lane 0): a stage's halo columns and streamed
        // weights arrive on full[s] with their bytes, half-resolution boxes
        // on upb[s]; the next stage is issued as soon as it is free
        for (int i = 0; i < my_tiles && ok && lane == 0; ++i) {
            const int tile = int(blockIdx.x) + i * int(gridDim.x);
            const int img = tile / per_img, r = tile - img * per_img;
            const int y0 = (r / tiles_x) * kTileH, x0 = (r - (r / tiles_x) * tiles_x) * kTileW;
            for (int c = 0; c < hp.nchunks; ++c) {
                const int j = i * hp.nchunks + c, s = j % S;
                if (!tc::mbar_wait(&empty[s], ((j / S) & 1) ^ 1)) {
                    ok = false;
                    break;
                }
                unsigned char* st = sa0 + s * hp.a_bytes;
                const int cols = min(hp.kc, CK - c * hp.kc) >> 3;
                uint32_t direct = 0, up = 0;
                for (int g = 0; g < cols; ++g) {
                    if ((hp.up >> (c * hp.kc + 8 * g < c0 ? 0 : 1)) & 1)
                        up += kUpBox;
                    else
                        direct += kHaloBox;
                }
                if (hp.up) mbar_expect_tx(&upb[s], up);
                mbar_expect_tx(&full[s], direct + (hp.stream ? 9u * hp.b_block : 0u));
                if (hp.stream) {
                    for (int t = 0; t < 9; ++t) {
                        if (MODE == FWD)  // (ch, row in group, channel group, tap, row group)
                            tma_load_5d(st + hp.b_off + t * hp.b_block, &mapw, 0, 0, c * (hp.kc >> 3), t, 0, &full[s]);
                        else  // (ch, k = output channel, channel group, tap)
                            tma_load_4d(st + hp.b_off + t * hp.b_block, &mapw, 0, c * hp.kc, 0, t, &full[s]);
                    }
                }
                for (int g = 0; g < cols; ++g) {
                    const int cb = c * hp.kc + 8 * g, src = cb < c0 ? 0 : 1, grp = (cb - src * c0) >> 3;
                    const CUtensorMap* m = src ? &map1 : &map0;
                    if ((hp.up >> src) & 1)
                        tma_load_5d(st + hp.up_off + g * kUpCol, m, 0, grp, (x0 >> 1) - 1, (y0 >> 1) - 1, img,
                                    &upb[s]);
                    else
                        tma_load_5d(st + g * kHaloCol, m, 0, grp, x0 - 1, y0 - 1, img, &full[s]);
                }
            }
        }
        __syncwarp();
    } else if (warp > kHaloIssueWarp && warp < kHaloMmaWarp) {
        // ---- widening (upsampled sources only): once a stage's boxes land,
        // halo pixel (hy, hx) copies pixel ((hy+1)/2, (hx+1)/2) of its box
        // into the column, then each warp arrives once on full[s]
        const int p = tid - (kHaloIssueWarp + 1) * 32;
        const bool owner = p < kHaloPx;
        const int hy = p / kHaloW, hx = p - hy * kHaloW;
        const uint32_t from = uint32_t(((hy + 1) >> 1) * kUpW + ((hx + 1) >> 1)) * 16u;
        for (int i = 0; i < my_tiles && ok && hp.up; ++i) {
            for (int c = 0; c < hp.nchunks; ++c) {
                const int j = i * hp.nchunks + c, s = j % S;
                // upb[s] completes after the copies into this stage, so after its release
                if (!__all_sync(0xFFFFFFFFu, tc::mbar_wait(&upb[s], (j / S) & 1))) {
                    ok = false;
                    break;
                }
                unsigned char* st = sa0 + s * hp.a_bytes;
                const int cols = min(hp.kc, CK - c * hp.kc) >> 3;
                for (int g = 0; g < cols && owner; ++g) {
                    if (!((hp.up >> (c * hp.kc + 8 * g < c0 ? 0 : 1)) & 1)) continue;
                    const uint4 v = *reinterpret_cast<const uint4*>(st + hp.up_off + g * kUpCol + from);
                    *reinterpret_cast<uint4*>(st + g * kHaloCol + p * 16) = v;
                }
                // each writer's stores to the async proxy, then one arrival per warp
                tc::fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&full[s]);
            }
        }
    } else if (warp == kHaloMmaWarp) {
        // ---- MMA issue (one thread): 9 taps × kc/16 slices per stage. The
        // descriptors are built once; an MMA adds its operands' offsets in
        // 16-byte units to their address fields.
        if (lane == 0) {
            uint32_t idesc = tc::idesc_bf16(kTileM, N);
            if (MODE == BWD_DATA) idesc |= 1u << 16;
            const uint64_t a0 = tc::smem_desc(tc::smem_u32(sa0), kHaloCol, kHaloRowStep);
            // resident weights: block (c, t) at sb; streamed: block t of the stage
            const uint64_t b0 = tc::smem_desc(tc::smem_u32(hp.stream ? sa0 + hp.b_off : sb), 128, uint32_t(16 * hp.kc));
            const uint32_t a_stage16 = hp.a_bytes >> 4, b_block16 = hp.b_block >> 4;
            for (int i = 0; i < my_tiles && ok; ++i) {
                const int b = i & 1;
                if (!tc::mbar_wait(&acc_empty[b], ((i >> 1) & 1) ^ 1)) {
                    ok = false;
                    break;
                }
                tc::tc_fence_after_sync();
                const uint32_t acc = tbase + uint32_t(b * N);
                for (int c = 0; c < hp.nchunks; ++c) {
                    const int j = i * hp.nchunks + c, s = j % S;
                    if (!tc::mbar_wait(&full[s], (j / S) & 1)) {
                        ok = false;
                        break;
                    }
                    tc::fence_proxy_async_smem();
                    tc::tc_fence_after_sync();
                    const uint64_t as = a0 + uint64_t(uint32_t(s) * a_stage16);
                    const uint64_t bc = b0 + uint64_t(hp.stream ? uint32_t(s) * a_stage16 : uint32_t(c * 9) * b_block16);
                    const int slices = min(hp.kc, CK - c * hp.kc) >> 4;
#pragma unroll
                    for (int t = 0; t < 9; ++t) {
                        // forward reads x(p + tap − 1); the input gradient reads dy(p − tap + 1)
                        const int ty = t / 3, tx = t % 3;
                        const uint32_t pix = MODE == FWD ? ty * kHaloW + tx : (2 - ty) * kHaloW + (2 - tx);
                        const uint64_t at = as + pix;
                        const uint64_t bt = bc + uint64_t(uint32_t(t) * b_block16);
                        for (int q = 0; q < slices; ++q)
                            tc::mma_bf16(acc, at + uint64_t(q * (2 * kHaloCol / 16)), bt + uint64_t(q * 16), idesc,
                                         (c > 0 || t > 0 || q > 0) ? 1u : 0u);
                    }
                    tc::mma_commit(&empty[s]);
                }
                if (!ok) break;
                tc::mma_commit(&acc_full[b]);
            }
        }
        __syncwarp();
    } else {
        // ---- epilogue: warp w holds tile rows 4w … 4w+3 (tensor-memory lanes 32·w …)
        const int py = 4 * warp + (lane >> 3), px = lane & 7;
        for (int i = 0; i < my_tiles && ok; ++i) {
            const int b = i & 1;
            if (!tc::mbar_wait(&acc_full[b], (i >> 1) & 1)) {
                ok = false;
                break;
            }
            tc::tc_fence_after_sync();
            const int tile = int(blockIdx.x) + i * int(gridDim.x);
            const int img = tile / per_img, r = tile - img * per_img;
            const int y = (r / tiles_x) * kTileH + py, x = (r - (r / tiles_x) * tiles_x) * kTileW + px;
            const bool valid = y < a.h && x < a.w;
            const size_t row = (size_t(img) * a.h + y) * a.w + x;
            const uint32_t lane_addr = tbase + (uint32_t(32 * warp) << 16) + uint32_t(b * N);
            for (int c = 0; c < N; c += 16) {
                float v[16];
                tc::tmem_ld16(lane_addr + uint32_t(c), v);  // the whole warp, every row
                if (valid) {
                    if (MODE == FWD) {
#pragma unroll
                        for (int q = 0; q < 16; ++q) {
                            float t = v[q] + sbias[c + q];
                            if (a.act) t = t > 0.0f ? t : kLeak * t;
                            v[q] = t;
                        }
                    } else if (a.mask) {
                        const uint4* mk = reinterpret_cast<const uint4*>(a.mask + row * a.mask_stride + c);
                        float mv[16];
                        unpack8(mk[0], mv);
                        unpack8(mk[1], mv + 8);
#pragma unroll
                        for (int q = 0; q < 16; ++q) v[q] *= slope(mv[q]);
                    }
                    if (MODE == FWD && a.out_f32) {
                        float4* o = reinterpret_cast<float4*>(a.out_f32 + row * a.out_stride + c);
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                    } else {
                        uint4* o = reinterpret_cast<uint4*>(a.out + row * a.out_stride + c);
                        o[0] = pack8(v);
                        o[1] = pack8(v + 8);
                    }
                }
            }
            tc::tc_fence_before_sync();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&acc_empty[b]);
        }
    }
    if (!ok) atomicOr(a.status, NET_STATUS_TIMEOUT);
    tc::tc_fence_before_sync();
    __syncthreads();
    if (warp == kHaloMmaWarp) {
        tc::tc_fence_after_sync();
        tc::tmem_dealloc(tbase, tcols);
    }
}

// ---------------------------------------------------------------- launchers

static int smem_for(int n) { return int(kStages * stage_bytes_for(n)); }

// The halo kernel's stage size and weight blocks for N output columns and
// CK K-side channels: of the chunk widths (32 or 64 channels, 16 where CK
// is 16) whose weights and at least two stages fit in a CTA, and of the
// resident-CTA counts up to `limit` (the other resources' bound), the one
// with the most CTAs (each brings its own MMA issuer and epilogue), then
// the widest chunk, with as many stages as fit. When the weights fit for no
// width, the stages bring their chunk's weights instead (32 or 16
// channels). False when even that does not fit.
static bool plan_halo(int N, int CK, bool up, int static_bytes, int limit, HaloPlan& hp, int& ctas) {
    const int per_sm = 233472, per_cta = 232448 - static_bytes;
    bool found = false;
    long best = 0;
    ctas = 0;
    // chunks below 32 channels only where the K side has fewer: a stage's
    // MMAs are then too few to cover its hand-over
    const int kc_min = CK >= 32 ? 32 : 16;
    for (int stream = 0; stream < 2 && !found; ++stream) {
        for (int kc = stream ? 32 : 64; kc >= (stream ? 16 : kc_min); kc >>= 1) {
            if (kc > CK && kc > 16) continue;
            HaloPlan q{};
            q.stream = stream;
            q.kc = kc;
            q.nchunks = (CK + kc - 1) / kc;
            q.up_off = uint32_t(kc / 8) * kHaloCol;
            q.b_off = q.up_off + (up ? uint32_t(kc / 8) * kUpCol : 0u);
            q.b_block = uint32_t(N) * uint32_t(kc) * 2u;
            q.b_bytes = stream ? 0u : uint32_t(q.nchunks) * 9u * q.b_block;
            q.a_bytes = q.b_off + (stream ? 9u * q.b_block : 0u);
            for (int t = limit; t >= 1; --t) {
                const int room = std::min(per_cta, per_sm / t - static_bytes - 1024) - int(q.b_bytes);
                const int stages = room > 0 ? std::min(kHaloMaxStages, room / int(q.a_bytes)) : 0;
                const long score = long(t) * 1000 + kc;
                if (stages >= 2 && score > best) {
                    q.stages = stages;
                    hp = q;
                    ctas = t;
                    best = score;
                    found = true;
                }
            }
        }
    }
    return found;
}

// Dynamic shared memory and resident CTAs of the halo kernel, counted from
// its resources as configure_ws does; fits is false when the weights do not
// fit in shared memory.
template <int MODE>
static cudaError_t configure_halo(int N, int CK, bool up, HaloPlan& hp, int& smem, int& ctas, bool& fits) {
    cudaFuncAttributes attr{};
    cudaError_t e = cudaFuncGetAttributes(&attr, k_conv_halo<MODE>);
    if (e != cudaSuccess) return e;
    const int by_threads = 2048 / kHaloThreads;
    const int regs_per_cta = ((attr.numRegs * 32 + 255) / 256 * 256) * (kHaloThreads / 32);
    const int by_regs = 65536 / regs_per_cta;
    const int max_tmem = 512 / int(tmem_cols_for(2 * N));
    const int limit = std::min(std::min(by_threads, by_regs), max_tmem);
    fits = limit >= 1 && plan_halo(N, CK, up, int(attr.sharedSizeBytes), limit, hp, ctas);
    if (!fits) return cudaSuccess;
    // a smaller request could let more CTAs reside than tensor memory allows: grow it
    smem = int(hp.b_bytes + uint32_t(hp.stages) * hp.a_bytes);
    while (233472 / (smem + int(attr.sharedSizeBytes) + 1024) > max_tmem) smem += 4096;
    return cudaFuncSetAttribute(k_conv_halo<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}


// The warp-specialised kernel's dynamic shared memory and resident CTAs per
// SM, counted from its resources (shared memory with the per-CTA reserve,
// threads, registers); its two accumulators need 2·n tensor-memory columns,
// so the shared-memory request grows until the resident CTAs fit in 512.
template <int MODE>
static cudaError_t configure_ws(int n, int& smem, int& ctas) {
    cudaFuncAttributes attr{};
    cudaError_t e = cudaFuncGetAttributes(&attr, k_conv_ws<MODE>);
    if (e != cudaSuccess) return e;
    const int by_threads = 2048 / kWsThreads;
    const int regs_per_cta = ((attr.numRegs * 32 + 255) / 256 * 256) * (kWsThreads / 32);
    const int by_regs = 65536 / regs_per_cta;
    const int max_tmem = 512 / int(tmem_cols_for(2 * n));
    smem = smem_for(n);
    for (;;) {
        const int by_smem = 233472 / (smem + int(attr.sharedSizeBytes) + 1024);
        ctas = std::min(std::min(by_threads, by_regs), by_smem);
        if (ctas <= max_tmem) break;
        smem += 4096;
    }
    if (ctas < 1) return cudaErrorInvalidConfiguration;
    return cudaFuncSetAttribute(k_conv_ws<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

template <int MODE>
static cudaError_t configure(int n, int& smem) {
    smem = smem_for(n);
    // Tensor memory: the CTAs that fit on an SM must not ask for more than
    // its 512 columns, or an allocation would wait for another CTA to end.
    const int per_sm_smem = 233472;  // 228 KB per SM
    const int cols = int(tmem_cols_for(n));
    const int max_ctas = 512 / cols;
    while (per_sm_smem / (smem + 2048) > max_ctas) smem += 4096;  // + static and reserved smem
    return cudaFuncSetAttribute(k_conv<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

static bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

const char* check_conv(const ConvArgs& a, int mode) {
    if (a.n <= 0 || a.h <= 0 || a.w <= 0) return "conv: empty geometry";
    if (a.cin % 16 || a.cout % 16 || a.cin < 16 || a.cout < 16) return "conv: channel counts must be multiples of 16";
    if (a.cin > 256 || a.cout > 256) return "conv: at most 256 channels";
    for (int i = 0; i < 2 && mode != BWD_DATA; ++i) {
        if (i == 0 && a.src[0].channels + a.src[1].channels != a.cin) return "conv: source channels do not add up to cin";
        const ConvSrc& s = a.src[i];
        if (s.channels == 0) continue;
        if (s.channels % 8 || s.stride % 8 || s.stride < s.channels) return "conv: source stride must cover its channels in multiples of 8";
        if (s.shift < 0 || s.shift > 1) return "conv: source shift must be 0 or 1";
        if (s.shift && ((a.h & 1) || (a.w & 1))) return "conv: an upsampled source needs even sizes";
        if (!s.ptr || !aligned16(s.ptr)) return "conv: source must be 16-byte aligned";
    }
    if (!a.wt || !aligned16(a.wt)) return "conv: weights must be 16-byte aligned";
    if (!a.status) return "conv: no status word";
    const size_t pixels = size_t(a.n) * a.h * a.w;
    if (pixels >= (size_t(1) << 31)) return "conv: too many pixels";
    if (mode == FWD) {
        if (!a.bias) return "conv: forward needs a bias";
        if (a.out_f32) {
            if (a.out_stride < a.cout || a.out_stride % 4 || !aligned16(a.out_f32)) return "conv: bad fp32 output";
        } else if (!a.out || a.out_stride < a.cout || a.out_stride % 8 || !aligned16(a.out)) {
            return "conv: bad output";
        }
    } else {
        if (!a.dy || a.dy_stride < a.cout || a.dy_stride % 8 || !aligned16(a.dy)) return "conv: bad output gradient";
    }
    if (mode == BWD_DATA) {
        if (!a.out || a.out_stride < a.cin || a.out_stride % 8 || !aligned16(a.out)) return "conv: bad input gradient";
        if (a.mask && (a.mask_stride < a.cin || a.mask_stride % 8 || !aligned16(a.mask))) return "conv: bad mask";
    }
    if (mode == BWD_WEIGHT) {
        if (!a.dw || !a.db) return "conv: weight gradient needs dw and db";
        if (a.pixels_per_cta <= 0 || a.pixels_per_cta % kChunk) return "conv: pixels per CTA must be a multiple of 64";
    }
    return nullptr;
}

bool conv_halo_fits(const ConvArgs& a, int mode) {
    if (mode != FWD && mode != BWD_DATA) return false;
    HaloPlan hp{};
    int smem = 0, ctas = 0;
    bool fits = false;
    const bool up = mode == FWD && (a.src[0].shift || (a.src[1].channels && a.src[1].shift));
    const cudaError_t e = mode == FWD ? configure_halo<FWD>(a.cout, a.cin, up, hp, smem, ctas, fits)
                                      : configure_halo<BWD_DATA>(a.cin, a.cout, false, hp, smem, ctas, fits);
    return e == cudaSuccess && fits;
}

// A BF16 NHWC tensor as a rank-5 tensor map (8 channels, channel groups,
// x, y, image) whose box is 8 channels × bw × bh pixels: one halo column,
// or the half-resolution box an upsampled column is widened from.
static bool encode_halo_map(CUtensorMap* m, const bf16* base, int channels, int stride, int w, int h, int n, int bw,
                            int bh) {
    auto enc = tensor_map_encoder();
    if (!enc || channels % 8 || stride % 8) return false;
    const cuuint64_t pix = cuuint64_t(stride) * 2;
    const cuuint64_t dims[5] = {8, cuuint64_t(channels / 8), cuuint64_t(w), cuuint64_t(h), cuuint64_t(n)};
    const cuuint64_t strides[4] = {16, pix, pix * cuuint64_t(w), pix * cuuint64_t(w) * cuuint64_t(h)};
    const cuuint32_t box[5] = {8, 1, cuuint32_t(bw), cuuint32_t(bh), 1};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The weights [cout][9][cin] as a tensor map whose box is one (chunk, tap)
// block of the halo kernel in core-matrix order: forward (K-major, rows =
// output channels) dims (8 channels, 8 rows, cin/8 groups, 9 taps, cout/8
// row groups); input gradient (MN-major, k = output channel) dims (8
// channels, cout, cin/8 groups, 9 taps).
template <int MODE>
static bool encode_weight_map(CUtensorMap* m, const bf16* wt, int cin, int cout, int kc) {
    auto enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t row = cuuint64_t(9) * cin * 2, tap = cuuint64_t(cin) * 2;
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    if (MODE == FWD) {
        const cuuint64_t dims[5] = {8, 8, cuuint64_t(cin / 8), 9, cuuint64_t(cout / 8)};
        const cuuint64_t strides[4] = {row, 16, tap, row * 8};
        const cuuint32_t box[5] = {8, 8, cuuint32_t(kc / 8), 1, cuuint32_t(cout / 8)};
        return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16*>(wt), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    }
    const cuuint64_t dims[4] = {8, cuuint64_t(cout), cuuint64_t(cin / 8), 9};
    const cuuint64_t strides[3] = {row, 16, tap};
    const cuuint32_t box[4] = {8, cuuint32_t(kc), cuuint32_t(cin / 8), 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16*>(wt), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Forward or input gradient: the halo kernel unless the caller asked for
// pixel-row tiles or the weights do not fit (then CONV_HALO is an error).
// Sources come by tensor copies (an upsampled one from its half-resolution
// tensor); if a map cannot be made the pixel-row kernel runs instead.
template <int MODE>
static cudaError_t launch_fwd_or_data(const ConvArgs& a, int num_sms, cudaStream_t st) {
    const int N = MODE == FWD ? a.cout : a.cin, CK = MODE == FWD ? a.cin : a.cout;
    int smem = 0, ctas = 0;
    cudaError_t e;
    if (a.kernel != CONV_ROWS) {
        HaloPlan hp{};
        bool fits = false;
        const bool up = MODE == FWD && (a.src[0].shift || (a.src[1].channels && a.src[1].shift));
        if ((e = configure_halo<MODE>(N, CK, up, hp, smem, ctas, fits)) != cudaSuccess) return e;
        CUtensorMap m[3];
        std::memset(m, 0, sizeof m);
        bool mapped = true;
        if (fits && MODE == FWD) {
            for (int k = 0; k < 2 && mapped; ++k) {
                const ConvSrc& src = a.src[k];
                if (src.channels == 0) continue;
                mapped = encode_halo_map(&m[k], src.ptr, src.channels, src.stride, a.w >> src.shift,
                                         a.h >> src.shift, a.n, src.shift ? kUpW : kHaloW, src.shift ? kUpH : kHaloH);
                if (src.shift) hp.up |= 1 << k;
            }
        } else if (fits) {
            mapped = encode_halo_map(&m[0], a.dy, a.cout, a.dy_stride, a.w, a.h, a.n, kHaloW, kHaloH);
        }
        if (fits && mapped && hp.stream) mapped = encode_weight_map<MODE>(&m[2], a.wt, a.cin, a.cout, hp.kc);
        if (fits && mapped) {
            const int ntiles = a.n * ((a.w + kTileW - 1) / kTileW) * ((a.h + kTileH - 1) / kTileH);
            k_conv_halo<MODE><<<std::min(ntiles, ctas * num_sms), kHaloThreads, smem, st>>>(a, hp, m[0], m[1], m[2]);
            return cudaGetLastError();
        }
        if (a.kernel == CONV_HALO) return fits ? cudaErrorNotSupported : cudaErrorInvalidValue;
    }
    if ((e = configure_ws<MODE>(N, smem, ctas)) != cudaSuccess) return e;
    const int ntiles = (a.n * a.h * a.w + kTileM - 1) / kTileM;
    k_conv_ws<MODE><<<std::min(ntiles, ctas * num_sms), kWsThreads, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_conv(ConvArgs a, int mode, int num_sms, cudaStream_t st) {
    if (mode == FWD) return launch_fwd_or_data<FWD>(a, num_sms, st);
    if (mode == BWD_DATA) return launch_fwd_or_data<BWD_DATA>(a, num_sms, st);
    const int pixels = a.n * a.h * a.w;
    int smem = 0;
    cudaError_t e;
    if ((e = configure<BWD_WEIGHT>(a.cout, smem)) != cudaSuccess) return e;
    const int mtiles = (9 * a.cin + 1 + kTileM - 1) / kTileM;
    if (a.pixels_per_cta <= 0) {
        // About two waves of CTAs over the SMs, at least 8 chunks each.
        const int want = std::max(1, 2 * num_sms / mtiles);
        int per = (pixels + want - 1) / want;
        per = std::max(per, 8 * kChunk);
        a.pixels_per_cta = (per + kChunk - 1) / kChunk * kChunk;
    }
    const int ksplit = (pixels + a.pixels_per_cta - 1) / a.pixels_per_cta;
    k_conv<BWD_WEIGHT><<<dim3(mtiles, ksplit), kThreads, smem, st>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- element-wise kernels

__device__ __forceinline__ float lum3(float r, float g, float b) { return r * 0.2126f + g * 0.7152f + b * 0.0722f; }

// The displayed radiance of one pixel from the network's output: a
// prediction p = a·e^o (o = out[0..2] clamped to ±kMaxLog, so p > 0) blended
// with the running average m: f = α·p + (1 − α)·m, α = sigmoid(out[3])·g.
// The guard g = v/(v + τ²) (v the average's relative variance of the mean
// luminance, from the Σ luminance² channel; τ the network's setting,
// about its own relative error) goes to zero as the average converges, so
// the display converges with it whatever the network predicts; the network
// learns α within that bound. Below kGuardMinSamples the per-pixel variance
// says too little and g = 1.
struct Blend {
    float a[3], m[3], pred[3], fin[3], alpha, gate, guard;
};
__device__ __forceinline__ Blend blend_at(const float* out, const float4& ac, const float4& al, float n, float tau) {
    Blend b;
    b.a[0] = fmaxf(al.x / n, 0.01f);
    b.a[1] = fmaxf(al.y / n, 0.01f);
    b.a[2] = fmaxf(al.z / n, 0.01f);
    b.m[0] = fmaxf(ac.x / n, 0.0f);
    b.m[1] = fmaxf(ac.y / n, 0.0f);
    b.m[2] = fmaxf(ac.z / n, 0.0f);
    const float ml = lum3(b.m[0], b.m[1], b.m[2]);
    const float var_mean = fmaxf(ac.w / n - ml * ml, 0.0f) / n;
    const float v = var_mean / (ml * ml + 1e-4f);
    b.guard = n < kGuardMinSamples ? 1.0f : v / (v + tau * tau);
    b.gate = 1.0f / (1.0f + expf(-fminf(fmaxf(out[3], -20.0f), 20.0f)));
    b.alpha = b.gate * b.guard;
    for (int c = 0; c < 3; ++c) {
        b.pred[c] = expf(fminf(fmaxf(out[c], -kMaxLog), kMaxLog)) * b.a[c];
        b.fin[c] = b.alpha * b.pred[c] + (1.0f - b.alpha) * b.m[c];
    }
    return b;
}

// d(loss)/d(value) of one channel's value v against target t:
// w_log · |log(1 + v/a) − log(1 + t/a)| + w_rel · (v − t)² / (v̂² + ε),
// v̂ = v held constant; adds the loss into *l.
__device__ __forceinline__ float loss_grad(float v, float t, float a, float w_log, float w_rel, float eps, float* l) {
    const float d = log1pf(v / a) - log1pf(fmaxf(t / a, 0.0f));
    const float e = v - t;
    const float den = v * v + eps;
    *l += w_log * fabsf(d) + w_rel * e * e / den;
    return w_log * (d > 0.0f ? 1.0f : d < 0.0f ? -1.0f : 0.0f) / (a + v) + w_rel * 2.0f * e / den;
}

// Input features of one pixel from the renderer's sums over n samples:
// log radiance over albedo (the à-trous filter's demodulation), albedo,
// unit normal, log depth, log standard error of the mean luminance,
// 1/sqrt(n), and four zero channels.
__global__ void k_features(FeatureArgs f) {
    const int total = f.n * f.h * f.w;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= total) return;
    const int hw = f.h * f.w;
    const int img = p / hw, r = p - img * hw, y = r / f.w, x = r - y * f.w;
    float v[16] = {};
    if (y < f.src_h && x < f.src_w) {
        const size_t i = (size_t(img) * f.src_h + y) * f.src_w + x;
        const float n = fmaxf(f.samples ? f.samples[img] : f.samples_all, 1.0f);
        const float4 ac = f.accum[i], al = f.albedo[i], nr = f.normal[i];
        const float ax = fmaxf(al.x / n, 0.01f), ay = fmaxf(al.y / n, 0.01f), az = fmaxf(al.z / n, 0.01f);
        const float mr = ac.x / n, mg = ac.y / n, mb = ac.z / n;
        v[0] = log1pf(fmaxf(mr / ax, 0.0f));
        v[1] = log1pf(fmaxf(mg / ay, 0.0f));
        v[2] = log1pf(fmaxf(mb / az, 0.0f));
        v[3] = ax;
        v[4] = ay;
        v[5] = az;
        const float d2 = nr.x * nr.x + nr.y * nr.y + nr.z * nr.z;
        if (d2 > 0.0f) {
            const float il = rsqrtf(d2);
            v[6] = nr.x * il;
            v[7] = nr.y * il;
            v[8] = nr.z * il;
        }
        v[9] = log1pf(fmaxf(nr.w / n, 0.0f));
        const float m = lum3(mr, mg, mb);
        const float var = fmaxf(ac.w / n - m * m, 0.0f) / n;
        v[10] = log1pf(sqrtf(var));
        v[11] = rsqrtf(n);
        if (!(isfinite(v[0]) && isfinite(v[1]) && isfinite(v[2]) && isfinite(v[9]) && isfinite(v[10]))) {
            for (int c = 0; c < 16; ++c) v[c] = 0.0f;
        }
    }
    uint4* o = reinterpret_cast<uint4*>(f.out + size_t(p) * 16);
    o[0] = pack8(v);
    o[1] = pack8(v + 8);
}

// 2×2 average pooling, 8 channels per thread.
__global__ void k_pool(const bf16* __restrict__ in, bf16* __restrict__ out, int n, int h, int w, int c) {
    const int oh = h >> 1, ow = w >> 1, groups = c >> 3;
    const size_t total = size_t(n) * oh * ow * groups;
    const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int g = int(t % groups);
    const size_t op = t / groups;
    const int x = int(op % ow), y = int((op / ow) % oh), img = int(op / (size_t(ow) * oh));
    float s[8] = {}, f[8];
    for (int dy = 0; dy < 2; ++dy)
        for (int dx = 0; dx < 2; ++dx) {
            const size_t ip = (size_t(img) * h + 2 * y + dy) * w + 2 * x + dx;
            unpack8(*reinterpret_cast<const uint4*>(in + ip * c + 8 * g), f);
            for (int i = 0; i < 8; ++i) s[i] += f[i];
        }
    for (int i = 0; i < 8; ++i) s[i] *= 0.25f;
    *reinterpret_cast<uint4*>(out + op * c + 8 * g) = pack8(s);
}

// Gradient of an upsampled source: the sum over each 2×2 block of the
// concatenation gradient's first `cup` channels, times the activation slope
// of the coarse tensor.
__global__ void k_split_up(const bf16* __restrict__ dcat, int cat_stride, bf16* __restrict__ g_coarse,
                           const bf16* __restrict__ coarse, int n, int h, int w, int cup) {
    const int oh = h >> 1, ow = w >> 1, groups = cup >> 3;
    const size_t total = size_t(n) * oh * ow * groups;
    const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int g = int(t % groups);
    const size_t op = t / groups;
    const int x = int(op % ow), y = int((op / ow) % oh), img = int(op / (size_t(ow) * oh));
    float s[8] = {}, f[8];
    for (int dy = 0; dy < 2; ++dy)
        for (int dx = 0; dx < 2; ++dx) {
            const size_t ip = (size_t(img) * h + 2 * y + dy) * w + 2 * x + dx;
            unpack8(*reinterpret_cast<const uint4*>(dcat + ip * cat_stride + 8 * g), f);
            for (int i = 0; i < 8; ++i) s[i] += f[i];
        }
    unpack8(*reinterpret_cast<const uint4*>(coarse + op * cup + 8 * g), f);
    for (int i = 0; i < 8; ++i) s[i] *= slope(f[i]);
    *reinterpret_cast<uint4*>(g_coarse + op * cup + 8 * g) = pack8(s);
}

// Gradient of an encoder output that feeds both a skip connection and the
// pooling below it: (skip gradient + pooled gradient / 4) × slope.
__global__ void k_merge(const bf16* __restrict__ skip, int skip_stride, const bf16* __restrict__ g_pool,
                        const bf16* __restrict__ act, bf16* __restrict__ out, int n, int h, int w, int c) {
    const int groups = c >> 3;
    const size_t total = size_t(n) * h * w * groups;
    const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int g = int(t % groups);
    const size_t p = t / groups;
    const int x = int(p % w), y = int((p / w) % h), img = int(p / (size_t(w) * h));
    const size_t cp = (size_t(img) * (h >> 1) + (y >> 1)) * (w >> 1) + (x >> 1);
    float s[8], q[8], f[8];
    unpack8(*reinterpret_cast<const uint4*>(skip + p * skip_stride + 8 * g), s);
    unpack8(*reinterpret_cast<const uint4*>(g_pool + cp * c + 8 * g), q);
    unpack8(*reinterpret_cast<const uint4*>(act + p * c + 8 * g), f);
    for (int i = 0; i < 8; ++i) s[i] = (s[i] + 0.25f * q[i]) * slope(f[i]);
    *reinterpret_cast<uint4*>(out + p * c + 8 * g) = pack8(s);
}

// Loss of one pixel: loss_grad of the display f (blend_at) plus loss_grad
// of the prediction p itself, so the prediction keeps learning whatever the
// blend weight does; and its gradient with respect to the network's output
// (bf16, 16 channels: three predictions and the blend logit, zero past the
// fourth; through the exponent's clamp as if unclamped). Each element is
// clipped to ±kMaxGrad, so one bright pixel cannot swamp a step.
__global__ void k_loss(LossArgs L) {
    const int total = L.n * L.h * L.w;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    float part = 0.0f;
    if (p < total) {
        const int hw = L.h * L.w;
        const int img = p / hw, r = p - img * hw, y = r / L.w, x = r - y * L.w;
        float g[16] = {};
        if (y < L.src_h && x < L.src_w) {
            const size_t i = (size_t(img) * L.src_h + y) * L.src_w + x;
            const float n = fmaxf(L.samples ? L.samples[img] : L.samples_all, 1.0f);
            const float* out = L.out + size_t(p) * 16;
            const Blend b = blend_at(out, L.accum[i], L.albedo[i], n, L.tau);
            const float4 tg = L.target[i];
            const float t[3] = {tg.x, tg.y, tg.z};
            float l = 0.0f, g_alpha = 0.0f, go[4];
            for (int c = 0; c < 3; ++c) {
                const float gf = loss_grad(b.fin[c], t[c], b.a[c], L.w_log, L.w_rel, L.rel_eps, &l);
                const float gp = loss_grad(b.pred[c], t[c], b.a[c], L.w_log, L.w_rel, L.rel_eps, &l);
                g_alpha += gf * (b.pred[c] - b.m[c]);
                go[c] = (gf * b.alpha + gp) * b.pred[c];
            }
            go[3] = g_alpha * b.guard * b.gate * (1.0f - b.gate);
            bool ok = isfinite(l);
            for (int c = 0; c < 4; ++c) ok = ok && isfinite(go[c]);
            if (ok) {
                part += l;
                for (int c = 0; c < 4; ++c) g[c] = fminf(fmaxf(go[c], -kMaxGrad), kMaxGrad) * L.scale;
            }
        }
        uint4* o = reinterpret_cast<uint4*>(L.grad + size_t(p) * 16);
        o[0] = pack8(g);
        o[1] = pack8(g + 8);
    }
    for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
    if ((threadIdx.x & 31) == 0 && part != 0.0f) atomicAdd(L.loss, part * L.scale);
}

// Adam on the flat parameter vector; refreshes the BF16 copy of the weights.
// A non-finite gradient element leaves its parameter and moments alone.
__global__ void k_adam(AdamArgs A) {
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.count) return;
    const float g = A.grad[i];
    if (!isfinite(g)) return;
    const float m = A.beta1 * A.m[i] + (1.0f - A.beta1) * g;
    const float v = A.beta2 * A.v[i] + (1.0f - A.beta2) * g * g;
    A.m[i] = m;
    A.v[i] = v;
    const float p = A.param[i] - A.step * m / (sqrtf(v) + A.eps_hat);
    A.param[i] = p;
    A.param_bf16[i] = __float2bfloat16_rn(p);
}

// Display image: the blend of the network's prediction and the running
// average (blend_at).
__global__ void k_compose(ComposeArgs C) {
    const int hw = C.w * C.h;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= C.n * hw) return;
    const int img = p / hw, r = p - img * hw, y = r / C.w, x = r - y * C.w;
    const float n = fmaxf(C.samples ? C.samples[img] : C.samples_all, 1.0f);
    const float* o = C.out + ((size_t(img) * C.ph + y) * C.pw + x) * 16;
    const Blend b = blend_at(o, C.accum[p], C.albedo[p], n, C.tau);
    float c[3];
    for (int k = 0; k < 3; ++k) c[k] = isfinite(b.fin[k]) ? b.fin[k] : b.m[k];
    C.dst[p] = make_float4(c[0], c[1], c[2], 1.0f);
}

static inline unsigned blocks_for(size_t n, unsigned t) { return unsigned((n + t - 1) / t); }

cudaError_t launch_features(const FeatureArgs& f, cudaStream_t st) {
    const size_t total = size_t(f.n) * f.h * f.w;
    k_features<<<blocks_for(total, 256), 256, 0, st>>>(f);
    return cudaGetLastError();
}
cudaError_t launch_pool(const bf16* in, bf16* out, int n, int h, int w, int c, cudaStream_t st) {
    const size_t total = size_t(n) * (h / 2) * (w / 2) * (c / 8);
    k_pool<<<blocks_for(total, 256), 256, 0, st>>>(in, out, n, h, w, c);
    return cudaGetLastError();
}
cudaError_t launch_split_up(const bf16* dcat, int cat_stride, bf16* g_coarse, const bf16* coarse, int n, int h, int w,
                            int cup, cudaStream_t st) {
    const size_t total = size_t(n) * (h / 2) * (w / 2) * (cup / 8);
    k_split_up<<<blocks_for(total, 256), 256, 0, st>>>(dcat, cat_stride, g_coarse, coarse, n, h, w, cup);
    return cudaGetLastError();
}
cudaError_t launch_merge(const bf16* skip, int skip_stride, const bf16* g_pool, const bf16* act, bf16* out, int n,
                         int h, int w, int c, cudaStream_t st) {
    const size_t total = size_t(n) * h * w * (c / 8);
    k_merge<<<blocks_for(total, 256), 256, 0, st>>>(skip, skip_stride, g_pool, act, out, n, h, w, c);
    return cudaGetLastError();
}
cudaError_t launch_loss(const LossArgs& L, cudaStream_t st) {
    const size_t total = size_t(L.n) * L.h * L.w;
    k_loss<<<blocks_for(total, 256), 256, 0, st>>>(L);
    return cudaGetLastError();
}
cudaError_t launch_adam(const AdamArgs& A, cudaStream_t st) {
    k_adam<<<blocks_for(A.count, 256), 256, 0, st>>>(A);
    return cudaGetLastError();
}
cudaError_t launch_compose(const ComposeArgs& C, cudaStream_t st) {
    k_compose<<<blocks_for(size_t(C.n) * C.w * C.h, 256), 256, 0, st>>>(C);
    return cudaGetLastError();
}

}  // namespace net
}  // namespace rmd
