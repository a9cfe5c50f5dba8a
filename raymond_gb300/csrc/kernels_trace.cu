// Primary-ray traversal and the one-kernel path tracer for sm_103a.
#include "dev_shade.cuh"
#include "kernels.cuh"

#include <cmath>

namespace rmd {

// Closest hits for a batch of rays (6 floats each). Persistent warps pull
// 32 rays at a time from a global counter, so the grid is sized to the SMs
// and no lane waits on a slow warp elsewhere.
__global__ void __launch_bounds__(TRACE_BLOCK) k_trace_primary(Scene s, const float* __restrict__ rays, uint32_t n,
                                                                 uint32_t* __restrict__ prim_out,
                                                                 float* __restrict__ t_out,
                                                                 uint32_t* __restrict__ counter) {
    __shared__ uint32_t stack[STACK_SHARED * TRACE_BLOCK];
    const uint32_t lane = threadIdx.x & 31u;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(counter, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) return;
        const uint32_t r = base + lane;
        if (r < n) {
            const float* ray = rays + size_t(r) * 6;
            const float3 o = f3(ray[0], ray[1], ray[2]);
            const float3 d = f3(ray[3], ray[4], ray[5]);
            const Hit h = trace_ray<false>(s, o, d, INF, stack + threadIdx.x, TRACE_BLOCK);
            prim_out[r] = h.prim;
            t_out[r] = h.t;
        }
    }
}

int launch_trace_primary(const Scene& s, const float* rays, uint32_t n, uint32_t* prim, float* t,
                         uint32_t* work_counter, int num_sms, cudaStream_t st) {
    cudaMemsetAsync(work_counter, 0, sizeof(uint32_t), st);
    const uint32_t warps_needed = (n + 31u) / 32u;
    uint32_t blocks = uint32_t(num_sms) * 8u;
    const uint32_t need = (warps_needed + (TRACE_BLOCK / 32) - 1) / (TRACE_BLOCK / 32);
    if (need < blocks) blocks = need > 0 ? need : 1;
    k_trace_primary<<<blocks, TRACE_BLOCK, 0, st>>>(s, rays, n, prim, t, work_counter);
    return 1;
}

// The sample streams, drawn as the kernels draw them (camera_rng, light_rng,
// gather_rng and Rng's rand/rand2), for bit-for-bit checks. Per pair: for
// each dimension id, rand2()'s two values then rand()'s one at that
// dimension; the spectrum position; `chain` draws of the light path's and of
// the gather's PCG chains.
__global__ void k_sample_streams(const uint32_t* __restrict__ pairs, uint32_t n, const uint32_t* __restrict__ dim_ids,
                                 uint32_t dims, uint32_t chain, uint32_t seed_hash, float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t index = pairs[2 * i], sample = pairs[2 * i + 1];
    float* o = out + size_t(i) * (3u * dims + 1u + 2u * chain);
    for (uint32_t k = 0; k < dims; ++k) {
        Rng r = camera_rng(index, sample, seed_hash);
        r.dim = dim_ids[k];
        const float2 two = r.rand2();
        r.dim = dim_ids[k];
        const float one = r.rand();
        o[3 * k] = two.x;
        o[3 * k + 1] = two.y;
        o[3 * k + 2] = one;
    }
    o += 3u * dims;
    *o++ = spectrum_position(index, sample);
    Rng light = light_rng(index, sample, seed_hash);
    for (uint32_t k = 0; k < chain; ++k) *o++ = light.rand();
    Rng gather = gather_rng(index, sample, seed_hash);
    for (uint32_t k = 0; k < chain; ++k) *o++ = gather.rand();
}

int launch_sample_streams(const uint32_t* pairs, uint32_t n, const uint32_t* dim_ids, uint32_t dims, uint32_t chain,
                          uint32_t seed_hash, float* out, cudaStream_t st) {
    if (n == 0) return 0;
    k_sample_streams<<<(n + 127u) / 128u, 128, 0, st>>>(pairs, n, dim_ids, dims, chain, seed_hash, out);
    return 1;
}

// ---- the megakernel: main() (src/shaders.mjs:1838-1895), one thread per pixel ----
constexpr int MK_BLOCK_X = 16, MK_BLOCK_Y = 8, MK_BLOCK = MK_BLOCK_X * MK_BLOCK_Y;

template <uint32_t FEAT>
__global__ void __launch_bounds__(MK_BLOCK) k_megakernel(Scene s, Params P, PixelBuffers px) {
    __shared__ uint32_t stack[STACK_SHARED * MK_BLOCK];
    const uint32_t tid = threadIdx.y * MK_BLOCK_X + threadIdx.x;
    uint32_t* col = stack + tid;
    const uint32_t x = blockIdx.x * MK_BLOCK_X + threadIdx.x;
    const uint32_t y = blockIdx.y * MK_BLOCK_Y + threadIdx.y;
    if (x >= P.width || y >= P.height) return;
    const uint32_t index = y * P.width + x;

    float4 sum = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float3 sum_albedo = f3(0.0f);
    float4 sum_normal = make_float4(0.0f, 0.0f, 0.0f, 0.0f);

    for (uint32_t k = 0; k < P.samples_per_frame; ++k) {
        PathState ps;
        float3 c;
        if (P.view == VIEW_COLOR) {
            path_begin(P, s.seed_hash, x, y, k, ps);
            for (;;) {
                const Hit hit = trace_ray<false>(s, ps.o, ps.d, INF, col, MK_BLOCK);
                ShadowRay sh;
                const bool more = path_step<FEAT>(s, P, ps, hit, sh);
                if (sh.valid) {
                    const Hit occ = trace_ray<true>(s, sh.o, sh.d, sh.reach, col, MK_BLOCK);
                    if (occ.prim == NONE) ps.result += sh.contribution;
                }
                if (!more) break;
            }
            c = ps.result;
            const float peak = maxc(c);
            if (P.firefly_clamp > 0.0f && peak > P.firefly_clamp) c *= P.firefly_clamp / peak;
        } else {
            ps.g_albedo = f3(0.0f);
            ps.g_normal = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            float3 o, d;
            Rng unused{};
            camera_ray(P, make_float2(float(x) + 0.5f, float(y) + 0.5f), false, unused, o, d);
            const Hit hit = trace_ray<false>(s, o, d, INF, col, MK_BLOCK);
            c = inspect_hit<FEAT>(s, P, o, d, hit);
        }
        const float3 gn = f3(ps.g_normal.x, ps.g_normal.y, ps.g_normal.z);
        if (finite3(c) && finite3(ps.g_albedo) && finite3(gn) && finite1(ps.g_normal.w)) {
            const float l = luminance(c);
            sum.x += c.x;
            sum.y += c.y;
            sum.z += c.z;
            sum.w += l * l;
            sum_albedo += ps.g_albedo;
            sum_normal.x += ps.g_normal.x;
            sum_normal.y += ps.g_normal.y;
            sum_normal.z += ps.g_normal.z;
            sum_normal.w += ps.g_normal.w;
        }
    }

    if (P.sample_offset == 0u) {
        px.accum[index] = sum;
        px.guide_albedo[index] = make_float4(sum_albedo.x, sum_albedo.y, sum_albedo.z, 0.0f);
        px.guide_normal[index] = sum_normal;
    } else {
        float4 a = px.accum[index];
        px.accum[index] = make_float4(a.x + sum.x, a.y + sum.y, a.z + sum.z, a.w + sum.w);
        float4 g = px.guide_albedo[index];
        px.guide_albedo[index] = make_float4(g.x + sum_albedo.x, g.y + sum_albedo.y, g.z + sum_albedo.z, g.w);
        float4 n = px.guide_normal[index];
        px.guide_normal[index] =
            make_float4(n.x + sum_normal.x, n.y + sum_normal.y, n.z + sum_normal.z, n.w + sum_normal.w);
    }
}

template <uint32_t FEAT>
static void launch_mk(const Scene& s, const Params& P, const PixelBuffers& px, cudaStream_t st) {
    const dim3 block(MK_BLOCK_X, MK_BLOCK_Y);
    const dim3 grid((P.width + MK_BLOCK_X - 1) / MK_BLOCK_X, (P.height + MK_BLOCK_Y - 1) / MK_BLOCK_Y);
    k_megakernel<FEAT><<<grid, block, 0, st>>>(s, P, px);
}

// Compiled feature sets: none, each alone, and all; anything else runs
// with every feature on, as the reference falls back to its all-features
// pipeline (src/Renderer.mjs:1000-1020).
int launch_megakernel(const Scene& s, const Params& P, uint32_t features, const PixelBuffers& px, int,
                      cudaStream_t st) {
    switch (features & 15u) {
        case 0: launch_mk<0>(s, P, px, st); break;
        case F_VOLUMES: launch_mk<F_VOLUMES>(s, P, px, st); break;
        case F_TEXTURES: launch_mk<F_TEXTURES>(s, P, px, st); break;
        case F_ENVIRONMENT: launch_mk<F_ENVIRONMENT>(s, P, px, st); break;
        case F_DISPERSION: launch_mk<F_DISPERSION>(s, P, px, st); break;
        default: launch_mk<15u>(s, P, px, st); break;
    }
    return 1;
}

cudaError_t upload_srgb_table_trace() { return upload_srgb_table_here(); }

}  // namespace rmd
