// Launch-side declarations of the learned denoiser's kernels.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>

namespace rmd {
namespace net {

enum ConvMode { FWD = 0, BWD_DATA = 1, BWD_WEIGHT = 2 };

// Forward and input-gradient kernels: pixel-row tiles that gather each tap
// (any size), or 8×16 halo tiles with the weights resident in shared memory
// (when they fit); CONV_AUTO takes the halo kernel where it can.
enum ConvKernel { CONV_AUTO = 0, CONV_ROWS = 1, CONV_HALO = 2 };

constexpr float kLeak = 0.1f;  // leaky ReLU slope below zero
constexpr float kMaxLog = 8.0f;    // clamp of the prediction's exponent (radiance ≤ e⁸ × albedo)
constexpr float kMaxGrad = 64.0f;  // loss: clip of each element's gradient (before the 1/(3·pixels) scale)
constexpr float kRelEps = 0.01f;   // loss: default ε of the relative squared error
constexpr float kBlendTau = 0.1f;         // blend guard's default τ: relative error below which the average takes over
constexpr float kGuardMinSamples = 4.0f;  // blend guard: off below this many samples
constexpr unsigned NET_STATUS_TIMEOUT = 1u;

// One input tensor of a convolution whose input is a channel concatenation:
// `channels` channels at `stride` per pixel; shift 1 reads it at half
// resolution (nearest-neighbour upsampling).
struct ConvSrc {
    const __nv_bfloat16* ptr;
    int channels;
    int stride;
    int shift;
};

struct ConvArgs {
    int n, h, w;     // images and spatial size (of the output, and of every full-resolution input)
    int cin, cout;   // cin = src[0].channels + src[1].channels
    ConvSrc src[2];  // forward and weight-gradient input
    const __nv_bfloat16* wt;  // [cout][9][cin]
    const float* bias;        // [cout]
    const __nv_bfloat16* dy;  // gradient at the convolution's output (before the activation)
    int dy_stride;
    __nv_bfloat16* out;  // forward output or input gradient
    int out_stride;
    float* out_f32;  // forward output in FP32 instead of `out`
    const __nv_bfloat16* mask;  // input gradient: times the activation slope of this tensor
    int mask_stride;
    float* dw;  // weight gradient, accumulated: [cout][9][cin]
    float* db;  // bias gradient, accumulated
    int act;    // forward: apply the leaky ReLU
    int pixels_per_cta;  // weight gradient: K split (0 picks one)
    unsigned* status;
    int kernel;  // forward and input gradient: CONV_AUTO, CONV_ROWS or CONV_HALO
};

struct FeatureArgs {
    const float4* accum;
    const float4* albedo;
    const float4* normal;
    const float* samples;  // per image, device; null uses samples_all
    float samples_all;
    int n, h, w;          // padded size of the feature tensor
    int src_h, src_w;     // size of the source images (≤ h, w)
    __nv_bfloat16* out;   // [n][h][w][16]
};

struct LossArgs {
    const float* out;  // [n][h][w][16] network output: predicted log radiance over albedo, blend logit
    const float4* accum;
    const float4* albedo;
    const float4* target;  // per-pixel mean radiance of the converged render
    const float* samples;
    float samples_all;
    int n, h, w, src_h, src_w;
    float scale;   // 1 / (3 · pixels)
    float w_log;   // weight of |log radiance error| (over albedo)
    float w_rel;   // weight of the relative squared radiance error
    float rel_eps; // ε of the relative squared error's denominator (v̂² + ε)
    float tau;     // blend guard
    __nv_bfloat16* grad;  // [n][h][w][16]
    float* loss;
};

struct AdamArgs {
    float* param;
    __nv_bfloat16* param_bf16;
    const float* grad;
    float* m;
    float* v;
    size_t count;
    float beta1, beta2, step, eps_hat;
};

struct ComposeArgs {
    const float* out;  // network output [n][ph][pw][16]
    const float4* accum;
    const float4* albedo;
    const float* samples;  // per image, device; null uses samples_all
    float samples_all;
    int n, w, h, pw, ph;
    float tau;    // blend guard
    float4* dst;  // [n][h][w]
};

const char* check_conv(const ConvArgs& a, int mode);
cudaError_t launch_conv(ConvArgs a, int mode, int num_sms, cudaStream_t st);
bool conv_halo_fits(const ConvArgs& a, int mode);  // the halo kernel's weights fit in shared memory
cudaError_t launch_features(const FeatureArgs& f, cudaStream_t st);
cudaError_t launch_pool(const __nv_bfloat16* in, __nv_bfloat16* out, int n, int h, int w, int c, cudaStream_t st);
cudaError_t launch_split_up(const __nv_bfloat16* dcat, int cat_stride, __nv_bfloat16* g_coarse,
                            const __nv_bfloat16* coarse, int n, int h, int w, int cup, cudaStream_t st);
cudaError_t launch_merge(const __nv_bfloat16* skip, int skip_stride, const __nv_bfloat16* g_pool,
                         const __nv_bfloat16* act, __nv_bfloat16* out, int n, int h, int w, int c, cudaStream_t st);
cudaError_t launch_loss(const LossArgs& L, cudaStream_t st);
cudaError_t launch_adam(const AdamArgs& A, cudaStream_t st);
cudaError_t launch_compose(const ComposeArgs& C, cudaStream_t st);

}  // namespace net

void set_handleless_error(const char* msg);

}  // namespace rmd

// The network over one renderer's buffers (float4 per pixel), written to
// dst on the given stream.
int rmd_net_denoise(struct raymond_net* net, const float* accum, const float* albedo, const float* normal,
                    float samples, uint32_t w, uint32_t h, float* dst, void* stream, std::string* err);
