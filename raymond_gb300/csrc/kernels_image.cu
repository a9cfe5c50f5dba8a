// The à-trous denoiser (src/shaders.mjs:1916-2098) and the display tone map
// (src/shaders.mjs:2114-2152) as sm_103a kernels on the per-pixel buffers.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "dev_tcgen05.cuh"
#include "dev_tma.cuh"
#include "kernels.cuh"

#include <mutex>

#include "../../include/raymond.h"

namespace rmd {

namespace {

__device__ __forceinline__ float3 xyz4(float4 v) { return make_float3(v.x, v.y, v.z); }
__device__ __forceinline__ float lum(float3 c) { return c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f; }

struct DenoiseView {
    const float4* accum;
    const float4* guide_albedo;
    const float4* guide_normal;
    const float4* guide_unit;  // the passes' guides, written by prepare; null: worked out per tap
    uint32_t w, h;
    float n;  // samples(): max(total_samples, 1)
};

__device__ __forceinline__ float3 albedo_at(const DenoiseView& v, uint32_t i) {
    const float4 g = v.guide_albedo[i];
    return make_float3(fmaxf(g.x / v.n, 0.01f), fmaxf(g.y / v.n, 0.01f), fmaxf(g.z / v.n, 0.01f));
}
// normal_at (src/shaders.mjs:1944-1952): the unit shading normal (zero where
// nothing was hit) and the mean depth of a guide sum. Explicitly rounded
// operations, so that prepare's copy and a per-tap recomputation agree bit
// for bit whichever kernel computes them.
__device__ __forceinline__ float4 unit_guide(float4 g, float n) {
    const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(g.x, g.x), __fmul_rn(g.y, g.y)), __fmul_rn(g.z, g.z));
    float3 u = make_float3(0.0f, 0.0f, 0.0f);
    if (d2 > 0.0f) {
        const float l = __fsqrt_rn(d2);
        u = make_float3(__fdiv_rn(g.x, l), __fdiv_rn(g.y, l), __fdiv_rn(g.z, l));
    }
    return make_float4(u.x, u.y, u.z, __fdiv_rn(g.w, n));
}
__device__ __forceinline__ float4 guide_at(const DenoiseView& v, uint32_t i) {
    return v.guide_unit ? v.guide_unit[i] : unit_guide(v.guide_normal[i], v.n);
}
__device__ __forceinline__ float3 light_at(const DenoiseView& v, uint32_t i) {
    const float4 a = v.accum[i];
    const float3 al = albedo_at(v, i);
    return make_float3(a.x / v.n / al.x, a.y / v.n / al.y, a.z / v.n / al.z);
}
// similarity (src/shaders.mjs:1958-1968): normal^64 by six squarings and the
// depth term's exponential, for prepare's variance estimate.
__device__ __forceinline__ float pow64(float x) {
    x = __fmul_rn(x, x);
    x = __fmul_rn(x, x);
    x = __fmul_rn(x, x);
    x = __fmul_rn(x, x);
    x = __fmul_rn(x, x);
    return __fmul_rn(x, x);
}
__device__ __forceinline__ float similarity(float4 p, float4 q, float step) {
    if (p.w <= 0.0f || q.w <= 0.0f) return (p.w <= 0.0f && q.w <= 0.0f) ? 1.0f : 0.0f;
    if (p.x * p.x + p.y * p.y + p.z * p.z == 0.0f) return 0.0f;
    const float wn = pow64(fmaxf(p.x * q.x + p.y * q.y + p.z * q.z, 0.0f));
    const float wz = expf(-fabsf(p.w - q.w) / (p.w * 0.02f * step + 1e-6f));
    return wn * wz;
}

__constant__ float c_kernel[3] = {0.375f, 0.25f, 0.0625f};
constexpr float LOG2E = 1.4426950408889634f;

// prepare (src/shaders.mjs:1974-2021), and the passes' guide for this pixel.
__device__ void prepare_at(const DenoiseView& v, uint32_t x, uint32_t y, float4* __restrict__ out,
                           float4* __restrict__ unit_out) {
    const uint32_t i = y * v.w + x;
    const float n = v.n;
    const float3 light = light_at(v, i);
    const float4 gp = unit_guide(v.guide_normal[i], n);
    if (unit_out) unit_out[i] = gp;
    const float a = lum(albedo_at(v, i));
    float variance;
    if (n >= 4.0f) {
        const float4 ac = v.accum[i];
        const float mean = lum(xyz4(ac)) / n;
        const float spread = fmaxf(ac.w / n - mean * mean, 0.0f) * n / (n - 1.0f);
        variance = spread / n / (a * a);
    } else {
        float sum = 0.0f, sum2 = 0.0f, weight = 0.0f;
        for (int dy = -2; dy <= 2; ++dy) {
            for (int dx = -2; dx <= 2; ++dx) {
                const int xx = int(x) + dx, yy = int(y) + dy;
                if (xx < 0 || yy < 0 || xx >= int(v.w) || yy >= int(v.h)) continue;
                const uint32_t j = uint32_t(yy) * v.w + uint32_t(xx);
                const float w = similarity(gp, unit_guide(v.guide_normal[j], n), 1.0f);
                const float l = lum(light_at(v, j));
                sum += w * l;
                sum2 += w * l * l;
                weight += w;
            }
        }
        const float mean = sum / fmaxf(weight, 1e-6f);
        variance = fmaxf(sum2 / fmaxf(weight, 1e-6f) - mean * mean, 0.0f) + 0.01f * mean * mean;
    }
    out[i] = make_float4(light.x, light.y, light.z, variance);
}
__global__ void k_prepare(DenoiseView v, float4* __restrict__ out, float4* __restrict__ unit_out) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= v.w || y >= v.h) return;
    prepare_at(v, x, y, out, unit_out);
}

// atrous (src/shaders.mjs:2023-2086) for one pixel of one pass. The centre's
// constants are worked out once: its guide, luminance, and the two
// exponentials' scales, so that a tap's weight
//   k(dx)·k(dy) · max(n_p·n_q, 0)^64 · exp(−|z_p − z_q| / (z_p·0.02·step + 1e-6)) · exp(−|l_p − l_q| / σ)
// costs six squarings and one exp2 of the two exponents' sum. LOAD(dx, dy,
// light, guide) fetches a tap (from a staged tile or from memory); INTERIOR
// drops the image-edge tests where every tap is inside. Every multiply-add
// is written out (__fmaf_rn, __fmul_rn), so the staged and the unstaged
// kernels, each instantiation compiled on its own, give the same bits.
__device__ __forceinline__ float lum_rn(float4 c) {
    return __fmaf_rn(c.z, 0.0722f, __fmaf_rn(c.y, 0.7152f, __fmul_rn(c.x, 0.2126f)));
}
__device__ __forceinline__ float dot3_rn(float4 a, float4 b) {
    return __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, __fmul_rn(a.x, b.x)));
}
struct PassCentre {
    float4 c, gp;
    float lp, kz, kl;
    bool background, flat;
};

template <bool INTERIOR, typename Load>
__device__ __forceinline__ float4 atrous_pixel(const DenoiseView& v, int x, int y, int step, Load load) {
    float4 c, gp;
    load(0, 0, c, gp);
    // σ from the 3×3 binomial blur of the variance (src/shaders.mjs:2037-2050).
    float variance = 0.0f, variance_weight = 0.0f;
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy) {
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx) {
            if (INTERIOR || (x + dx >= 0 && y + dy >= 0 && x + dx < int(v.w) && y + dy < int(v.h))) {
                const float w = __fmul_rn(c_kernel[dx < 0 ? -dx : dx], c_kernel[dy < 0 ? -dy : dy]);
                float4 q, g;
                load(dx, dy, q, g);
                variance = __fmaf_rn(w, q.w, variance);
                variance_weight = __fadd_rn(variance_weight, w);
            }
        }
    }
    const float sigma = __fmaf_rn(4.0f, __fsqrt_rn(__fdiv_rn(variance, variance_weight)), 1e-4f);
    const float lp = lum_rn(c);
    const float kl = __fdiv_rn(LOG2E, sigma);
    const float kz = __fdiv_rn(LOG2E, __fmaf_rn(__fmul_rn(gp.w, 0.02f), float(step), 1e-6f));
    const bool background = gp.w <= 0.0f;
    const bool flat = dot3_rn(gp, gp) == 0.0f;

    float3 sum = make_float3(0.0f, 0.0f, 0.0f);
    float sum_variance = 0.0f, weight = 0.0f;
#pragma unroll
    for (int dy = -2; dy <= 2; ++dy) {
#pragma unroll
        for (int dx = -2; dx <= 2; ++dx) {
            const int xx = x + dx * step, yy = y + dy * step;
            if (!INTERIOR && (xx < 0 || yy < 0 || xx >= int(v.w) || yy >= int(v.h))) continue;
            float4 q, gq;
            load(dx * step, dy * step, q, gq);
            const float k = __fmul_rn(c_kernel[dx < 0 ? -dx : dx], c_kernel[dy < 0 ? -dy : dy]);
            const float dl = fabsf(__fsub_rn(lp, lum_rn(q)));
            float w;
            if (background || gq.w <= 0.0f) {
                w = (background && gq.w <= 0.0f) ? __fmul_rn(k, exp2f(-__fmul_rn(dl, kl))) : 0.0f;
            } else if (flat) {
                w = 0.0f;
            } else {
                const float wn = pow64(fmaxf(dot3_rn(gp, gq), 0.0f));
                w = __fmul_rn(__fmul_rn(k, wn), exp2f(-__fmaf_rn(fabsf(__fsub_rn(gp.w, gq.w)), kz, __fmul_rn(dl, kl))));
            }
            sum.x = __fmaf_rn(w, q.x, sum.x);
            sum.y = __fmaf_rn(w, q.y, sum.y);
            sum.z = __fmaf_rn(w, q.z, sum.z);
            sum_variance = __fmaf_rn(__fmul_rn(w, w), q.w, sum_variance);
            weight = __fadd_rn(weight, w);
        }
    }
    if (weight > 0.0f) {
        const float w2 = __fmul_rn(weight, weight);
        return make_float4(__fdiv_rn(sum.x, weight), __fdiv_rn(sum.y, weight), __fdiv_rn(sum.z, weight),
                           __fdiv_rn(sum_variance, w2));
    }
    return c;
}

// A pass reading its taps from memory (L1/L2): the passes of the allocation-
// free entry, the batch's, and every renderer's last pass (step 16, whose
// 32-pixel halo makes a staged tile too large). With `compose`, the pass
// writes compose()'s product with the albedo (src/shaders.mjs:2088-2097)
// into out instead of the filtered light.
__device__ __forceinline__ void atrous_at(const DenoiseView& v, const float4* __restrict__ in, float4* __restrict__ out,
                                          int step, uint32_t x, uint32_t y, bool compose) {
    const uint32_t i = y * v.w + x;
    auto load = [&](int ox, int oy, float4& q, float4& g) {
        const uint32_t j = uint32_t(int(i) + oy * int(v.w) + ox);
        q = __ldg(in + j);
        g = guide_at(v, j);
    };
    const int reach = 2 * step;
    const bool interior = int(x) >= reach && int(y) >= reach && int(x) + reach < int(v.w) && int(y) + reach < int(v.h);
    const float4 l = interior ? atrous_pixel<true>(v, int(x), int(y), step, load)
                              : atrous_pixel<false>(v, int(x), int(y), step, load);
    if (compose) {
        const float3 a = albedo_at(v, i);
        out[i] = make_float4(__fmul_rn(l.x, a.x), __fmul_rn(l.y, a.y), __fmul_rn(l.z, a.z), 0.0f);
    } else {
        out[i] = l;
    }
}
__global__ void k_atrous(DenoiseView v, const float4* __restrict__ in, float4* __restrict__ out, int step, int compose) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= v.w || y >= v.h) return;
    atrous_at(v, in, out, step, x, y, compose != 0);
}

// The same pass with its input staged in shared memory by the tensor memory
// accelerator: a 32×16 block of outputs reads a (32 + 4·step) × (16 + 4·step)
// tile of the light buffer and of the passes' guide, two 2D box copies that
// complete on one mbarrier (a bounded wait; a wait that runs out sets the
// status word and the block writes nothing). Taps outside the image are
// skipped by coordinate, as in atrous_at; the box's out-of-image part is
// zero-filled and never read. Blocks whose whole tile lies inside the image
// skip the tests. Same arithmetic as atrous_at.
constexpr int ATROUS_TW = 32, ATROUS_TH = 16, ATROUS_THREADS = 256;

template <int STEP>
struct AtrousTile {
    static constexpr int halo = 2 * STEP;
    static constexpr int w = ATROUS_TW + 2 * halo, h = ATROUS_TH + 2 * halo;
    static constexpr uint32_t bytes = uint32_t(w) * h * 16;
    static constexpr uint32_t stride = (bytes + 1023u) / 1024u * 1024u;  // second tile 1 KB aligned
    static constexpr uint32_t smem = 2 * stride;
};

template <int STEP>
__global__ void __launch_bounds__(ATROUS_THREADS) k_atrous_tma(DenoiseView v, const __grid_constant__ CUtensorMap light,
                                                                const __grid_constant__ CUtensorMap guide,
                                                                float4* __restrict__ out, unsigned* status) {
    using T = AtrousTile<STEP>;
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t bar;
    const float4* s_light = reinterpret_cast<const float4*>(smem);
    const float4* s_guide = reinterpret_cast<const float4*>(smem + T::stride);
    const int bx = int(blockIdx.x) * ATROUS_TW, by = int(blockIdx.y) * ATROUS_TH;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        tc::fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_expect_tx(&bar, 2u * T::bytes);
        // x counts floats (4 per pixel): always a multiple of 16 bytes.
        tma_load_2d(smem, &light, 4 * (bx - T::halo), by - T::halo, &bar);
        tma_load_2d(smem + T::stride, &guide, 4 * (bx - T::halo), by - T::halo, &bar);
    }
    const bool arrived = tc::mbar_wait(&bar, 0);
    if (!__syncthreads_and(arrived)) {
        if (threadIdx.x == 0) {
            atomicOr(status, 1u);
            tc::mbar_wait(&bar, 0);  // bounded: the copies must land before the block's memory goes
        }
        __syncthreads();
        return;
    }
    const bool interior = bx >= T::halo && by >= T::halo && bx + ATROUS_TW + T::halo <= int(v.w) &&
                          by + ATROUS_TH + T::halo <= int(v.h);
    const int tx = int(threadIdx.x) % ATROUS_TW;
    for (int ty = int(threadIdx.x) / ATROUS_TW; ty < ATROUS_TH; ty += ATROUS_THREADS / ATROUS_TW) {
        const int x = bx + tx, y = by + ty;
        if (x >= int(v.w) || y >= int(v.h)) continue;
        const int base = (ty + T::halo) * T::w + (tx + T::halo);
        auto load = [&](int ox, int oy, float4& q, float4& g) {
            q = s_light[base + oy * T::w + ox];
            g = s_guide[base + oy * T::w + ox];
        };
        out[uint32_t(y) * v.w + uint32_t(x)] =
            interior ? atrous_pixel<true>(v, x, y, STEP, load) : atrous_pixel<false>(v, x, y, STEP, load);
    }
}

// Narkowicz's ACES fit and the sRGB OETF (src/shaders.mjs:2115-2122).
__device__ __forceinline__ float aces1(float x) {
    return fminf(fmaxf((x * (2.51f * x + 0.03f)) / (x * (2.43f * x + 0.59f) + 0.14f), 0.0f), 1.0f);
}
__device__ __forceinline__ float to_srgb1(float c) {
    const float x = fminf(fmaxf(c, 0.0f), 1.0f);
    return x <= 0.0031308f ? x * 12.92f : 1.055f * powf(x, 1.0f / 2.4f) - 0.055f;
}
__device__ __forceinline__ uint8_t unorm8(float v) {
    const float c = fminf(fmaxf(v, 0.0f), 1.0f);
    return uint8_t(__float2int_rn(c * 255.0f));
}

// fragment (src/shaders.mjs:2124-2152) into a headless RGBA8 buffer.
__device__ void tonemap_at(const Params& P, const float4* __restrict__ accum, const float4* __restrict__ denoised,
                           uchar4* __restrict__ display, uint32_t x, uint32_t y) {
    const uint32_t i = y * P.width + x;
    float3 o;
    if (P.total_samples == 0u) {
        o = make_float3(0.0f, 0.0f, 0.0f);
    } else {
        const float4 a = accum[i];
        const float n = float(P.total_samples);
        const float3 c = make_float3(a.x / n, a.y / n, a.z / n);
        if (P.view == 0u) {
            float3 shown = c;
            if (P.denoise != 0u) shown = xyz4(denoised[i]);
            o = make_float3(to_srgb1(aces1(shown.x * P.exposure)), to_srgb1(aces1(shown.y * P.exposure)),
                            to_srgb1(aces1(shown.z * P.exposure)));
        } else if (P.view == 1u) {
            o = make_float3(to_srgb1(c.x), to_srgb1(c.y), to_srgb1(c.z));
        } else if (P.view == 2u) {
            o = make_float3(c.x * 0.5f + 0.5f, c.y * 0.5f + 0.5f, c.z * 0.5f + 0.5f);
        } else {
            const float g = c.x <= 0.0f ? 0.0f : 1.0f / (1.0f + c.x / P.focus_distance);
            o = make_float3(g, g, g);
        }
    }
    display[i] = make_uchar4(unorm8(o.x), unorm8(o.y), unorm8(o.z), 255);
}
__global__ void k_tonemap(Params P, const float4* __restrict__ accum, const float4* __restrict__ denoised,
                          uchar4* __restrict__ display) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= P.width || y >= P.height) return;
    tonemap_at(P, accum, denoised, display, x, y);
}

}  // namespace

// cuTensorMapEncodeTiled, from the driver through the runtime (no -lcuda).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

namespace {

// A w×h float4 image as a 2D tensor of floats (4w × h) with a box of the
// tile for one step.
template <int STEP>
bool encode_tile_map(CUtensorMap* map, const float4* base, uint32_t w, uint32_t h) {
    auto enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t dims[2] = {cuuint64_t(w) * 4, h};
    const cuuint64_t strides[1] = {cuuint64_t(w) * 16};
    const cuuint32_t box[2] = {cuuint32_t(AtrousTile<STEP>::w * 4), cuuint32_t(AtrousTile<STEP>::h)};
    const cuuint32_t estr[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float4*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int STEP>
bool launch_atrous_tma(const DenoiseView& v, const float4* in, float4* out, unsigned* status, cudaStream_t st) {
    CUtensorMap light, guide;
    if (!v.guide_unit || !encode_tile_map<STEP>(&light, in, v.w, v.h) ||
        !encode_tile_map<STEP>(&guide, v.guide_unit, v.w, v.h))
        return false;
    static const bool configured = cudaFuncSetAttribute(k_atrous_tma<STEP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                        int(AtrousTile<STEP>::smem)) == cudaSuccess;
    if (!configured) return false;
    const dim3 grid((v.w + ATROUS_TW - 1) / ATROUS_TW, (v.h + ATROUS_TH - 1) / ATROUS_TH);
    k_atrous_tma<STEP><<<grid, ATROUS_THREADS, AtrousTile<STEP>::smem, st>>>(v, light, guide, out, status);
    return true;
}

}  // namespace

int launch_denoise(const Params& P, const PixelBuffers& px, unsigned* status, cudaStream_t st) {
    DenoiseView v{px.accum, px.guide_albedo, px.guide_normal, px.guide_unit, P.width, P.height,
                  float(P.total_samples > 1u ? P.total_samples : 1u)};
    const dim3 block(16, 8), grid((P.width + 15) / 16, (P.height + 7) / 8);
    // prepare fills light a and the passes' guide; the passes go a→b, b→a,
    // …; the last writes compose()'s product into denoised (src/Renderer.mjs:893-912).
    k_prepare<<<grid, block, 0, st>>>(v, px.light_a, px.guide_unit);
    const int steps[4] = {1, 2, 4, 8};
    float4* from = px.light_a;
    float4* to = px.light_b;
    for (int k = 0; k < 4; ++k) {
        // Steps 1-8 stage their tiles with TMA.
        bool staged = false;
        if (status) {
            switch (steps[k]) {
                case 1: staged = launch_atrous_tma<1>(v, from, to, status, st); break;
                case 2: staged = launch_atrous_tma<2>(v, from, to, status, st); break;
                case 4: staged = launch_atrous_tma<4>(v, from, to, status, st); break;
                default: staged = launch_atrous_tma<8>(v, from, to, status, st); break;
            }
        }
        if (!staged) k_atrous<<<grid, block, 0, st>>>(v, from, to, steps[k], 0);
        float4* t = from;
        from = to;
        to = t;
    }
    // Step 16's halo (32 pixels a side) would need 200 KB of tile for 512
    // outputs, so it reads L1/L2, and composes as it writes.
    k_atrous<<<grid, block, 0, st>>>(v, from, px.denoised, 16, 1);
    return 6;
}

int launch_tonemap(const Params& P, const PixelBuffers& px, cudaStream_t st) {
    const dim3 block(16, 8), grid((P.width + 15) / 16, (P.height + 7) / 8);
    k_tonemap<<<grid, block, 0, st>>>(P, px.accum, px.denoised, px.display);
    return 1;
}

namespace {
// readPixels' average: each sum divided by the sample count, correctly
// rounded (IEEE division, as the host's), before the image leaves the GPU.
__global__ void k_average(const float4* __restrict__ sums, float4* __restrict__ out, uint32_t n, float samples) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 s = sums[i];
        out[i] = make_float4(__fdiv_rn(s.x, samples), __fdiv_rn(s.y, samples), __fdiv_rn(s.z, samples),
                             __fdiv_rn(s.w, samples));
    }
}
}  // namespace

int launch_average(const float4* sums, float4* out, uint32_t n, float samples, int num_sms, cudaStream_t st) {
    const uint32_t blocks = std::min<uint32_t>((n + 255u) / 256u, uint32_t(num_sms) * 8u);
    k_average<<<blocks ? blocks : 1u, 256, 0, st>>>(sums, out, n, samples);
    return 1;
}


// ---- batched frames: the same passes over many jobs' images in one launch ----
namespace {

// The job whose pixels hold batch pixel t (segments in pixel order).
__device__ __forceinline__ uint32_t find_job(const JobPixels* seg, uint32_t n, uint32_t t) {
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) / 2;
        if (seg[mid].pixel_offset <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ DenoiseView job_view(const JobDesc& jd) {
    const Params& P = jd.params;
    return DenoiseView{jd.px.accum, jd.px.guide_albedo, jd.px.guide_normal, jd.px.guide_unit, P.width, P.height,
                       float(P.total_samples > 1u ? P.total_samples : 1u)};
}

// pass: 0 prepare, 1..4 à-trous steps 1..8, 5 step 16 composed into denoised.
__global__ void k_denoise_batch(const JobDesc* __restrict__ jobs, const JobPixels* __restrict__ seg, uint32_t n_seg,
                                uint32_t total, int pass) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const JobPixels g = seg[find_job(seg, n_seg, t)];
        const JobDesc& jd = jobs[g.job];
        if (jd.params.denoise == 0u) continue;
        const DenoiseView v = job_view(jd);
        const uint32_t i = t - g.pixel_offset;
        const uint32_t x = i % v.w, y = i / v.w;
        // prepare fills light a and the guide; passes go a→b, b→a, …; the
        // fifth reads light a and writes the composed image.
        if (pass == 0) {
            prepare_at(v, x, y, jd.px.light_a, jd.px.guide_unit);
        } else if (pass <= 4) {
            const bool even = (pass - 1) % 2 == 0;
            atrous_at(v, even ? jd.px.light_a : jd.px.light_b, even ? jd.px.light_b : jd.px.light_a,
                      1 << (pass - 1), x, y, false);
        } else {
            atrous_at(v, jd.px.light_a, jd.px.denoised, 16, x, y, true);
        }
    }
}

__global__ void k_tonemap_batch(const JobDesc* __restrict__ jobs, const JobPixels* __restrict__ seg, uint32_t n_seg,
                                uint32_t total) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const JobPixels g = seg[find_job(seg, n_seg, t)];
        const JobDesc& jd = jobs[g.job];
        const uint32_t i = t - g.pixel_offset;
        tonemap_at(jd.params, jd.px.accum, jd.px.denoised, jd.px.display, i % jd.params.width, i / jd.params.width);
    }
}

}  // namespace

int launch_image_batch(const JobDesc* d_jobs, const JobPixels* d_pix, uint32_t n_jobs, uint32_t total_pixels,
                       int num_sms, cudaStream_t st) {
    const int grid = num_sms * 8;
    for (int pass = 0; pass <= 5; ++pass) k_denoise_batch<<<grid, 256, 0, st>>>(d_jobs, d_pix, n_jobs, total_pixels, pass);
    k_tonemap_batch<<<grid, 256, 0, st>>>(d_jobs, d_pix, n_jobs, total_pixels);
    return 7;
}

// ---- Denoising into a caller's buffers without allocating ----
//
// raymond_denoise_static runs the same prepare / à-trous / compose kernels
// as a renderer's frame, but keeps the two intermediate light buffers in
// this fixed file-scope device array instead of memory the renderer
// allocates. Every GPU that loads the library holds the array until exit.
// All calls share it: two calls whose kernels overlap on the GPU (different
// streams, no ordering between them) race on it. Nothing in it needs to
// start at zero: prepare writes every pixel of the first buffer and each
// pass writes every pixel of the buffer it produces before anything reads
// it, so the previous call's contents are never seen.
namespace {

constexpr uint32_t kStaticDenoiseMaxPixels = RAYMOND_DENOISE_STATIC_MAX_PIXELS;
static __device__ __align__(256) float4 g_denoise_scratch[2 * kStaticDenoiseMaxPixels];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
float4* g_scratch_address[kMaxDevices] = {};

}  // namespace

extern "C" int raymond_denoise_static(const float* accum, const float* guide_albedo, const float* guide_normal,
                                      uint32_t width, uint32_t height, uint32_t total_samples, float* out,
                                      void* stream) {
    if (!accum || !guide_albedo || !guide_normal || !out || width == 0 || height == 0) {
        set_handleless_error("raymond_denoise_static: null buffer or empty image.");
        return RAYMOND_EINVAL;
    }
    if (uint64_t(width) * height > kStaticDenoiseMaxPixels) {
        set_handleless_error("raymond_denoise_static: the image has more pixels than the static scratch holds "
                             "(RAYMOND_DENOISE_STATIC_MAX_PIXELS).");
        return RAYMOND_ECAPACITY;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0) {
        set_handleless_error("raymond_denoise_static: no current CUDA device.");
        return RAYMOND_ECUDA;
    }
    if (dev >= kMaxDevices) {
        set_handleless_error("raymond_denoise_static: the current device's index is beyond the static scratch "
                             "table's 64 devices.");
        return RAYMOND_ECUDA;
    }
    float4* scratch;
    {
        // First call on this device: resolve the array's device address
        // (the host-side symbol is only a stand-in for it).
        std::lock_guard<std::mutex> lock(g_scratch_mutex);
        if (!g_scratch_address[dev]) {
            void* addr = nullptr;
            e = cudaGetSymbolAddress(&addr, g_denoise_scratch);
            if (e != cudaSuccess || !addr) {
                set_handleless_error("raymond_denoise_static: cudaGetSymbolAddress failed.");
                return RAYMOND_ECUDA;
            }
            g_scratch_address[dev] = static_cast<float4*>(addr);
        }
        scratch = g_scratch_address[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const uint32_t pixels = width * height;
    // No third buffer here for the passes' guide: each tap works it out from
    // guide_normal (the same bits prepare would have stored).
    DenoiseView v{reinterpret_cast<const float4*>(accum), reinterpret_cast<const float4*>(guide_albedo),
                  reinterpret_cast<const float4*>(guide_normal), nullptr, width, height,
                  float(total_samples > 1u ? total_samples : 1u)};
    const dim3 block(16, 8), grid((width + 15) / 16, (height + 7) / 8);
    float4* from = scratch;
    float4* to = scratch + pixels;
    k_prepare<<<grid, block, 0, st>>>(v, from, nullptr);
    const int steps[4] = {1, 2, 4, 8};
    for (int k = 0; k < 4; ++k) {
        k_atrous<<<grid, block, 0, st>>>(v, from, to, steps[k], 0);
        float4* t = from;
        from = to;
        to = t;
    }
    k_atrous<<<grid, block, 0, st>>>(v, from, reinterpret_cast<float4*>(out), 16, 1);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_handleless_error("raymond_denoise_static: kernel launch failed.");
        return RAYMOND_ECUDA;
    }
    return RAYMOND_OK;
}

}  // namespace rmd
