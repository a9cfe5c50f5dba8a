// Host side of the learned denoiser: the U-Net's layer table, its parameter,
// gradient, Adam and activation memory, and the forward, backward and
// training sequences behind the raymond_net_* and raymond_conv3x3_* entry
// points. The network only ever filters a displayed image; the renderer's
// running sums are inputs, never outputs.
//
// Network: five levels of widths 32, 64, 96, 128, 128; two 3×3 convolutions
// with a leaky ReLU per level on the way down (2×2 average pooling between
// levels) and on the way up (nearest-neighbour upsampling concatenated with
// the encoder's output at that level), and a last 3×3 convolution to the
// predicted log radiance over albedo and a blend weight: the display is the
// prediction blended with the running average (in FP32, per pixel). 19 convolutions: 1,649,664 weights and
// 1,696 biases.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/raymond.h"
#include "net.cuh"

using namespace rmd::net;
using bf16 = __nv_bfloat16;

namespace {

// Activation tensors of one forward pass.
enum Tensor {
    T_IN, T_E0A, T_E0, T_P1, T_E1A, T_E1, T_P2, T_E2A, T_E2, T_P3, T_E3A, T_E3, T_P4, T_E4A, T_E4,
    T_D3A, T_D3, T_D2A, T_D2, T_D1A, T_D1, T_D0A, T_D0,
    // gradients (training only)
    T_GOUT, T_DCAT0, T_DCAT1, T_DCAT2, T_DCAT3, T_GA0, T_GA1, T_GA2, T_GA3, T_GA4, T_GB0, T_GB1, T_GB2, T_GB3, T_GB4,
    T_COUNT
};
constexpr int kFirstGradient = T_GOUT;

struct TensorDef {
    int level, channels;
};
constexpr TensorDef kTensors[T_COUNT] = {
    {0, 16}, {0, 32}, {0, 32}, {1, 32}, {1, 64}, {1, 64}, {2, 64}, {2, 96}, {2, 96}, {3, 96}, {3, 128}, {3, 128},
    {4, 128}, {4, 128}, {4, 128}, {3, 128}, {3, 128}, {2, 96}, {2, 96}, {1, 64}, {1, 64}, {0, 32}, {0, 32},
    {0, 16}, {0, 96}, {1, 160}, {2, 224}, {3, 256}, {0, 32}, {1, 64}, {2, 96}, {3, 128}, {4, 128}, {0, 32},
    {1, 64}, {2, 96}, {3, 128}, {4, 128},
};

struct LayerDef {
    int src0, src1;  // tensors; src1 = -1 for one input. src0 is upsampled when src1 is set.
    int out;         // tensor, or -1 for the FP32 network output
    int cout, level, act;
};
constexpr int kLayers = 19;
constexpr LayerDef kLayerDefs[kLayers] = {
    {T_IN, -1, T_E0A, 32, 0, 1},   {T_E0A, -1, T_E0, 32, 0, 1},   {T_P1, -1, T_E1A, 64, 1, 1},
    {T_E1A, -1, T_E1, 64, 1, 1},   {T_P2, -1, T_E2A, 96, 2, 1},   {T_E2A, -1, T_E2, 96, 2, 1},
    {T_P3, -1, T_E3A, 128, 3, 1},  {T_E3A, -1, T_E3, 128, 3, 1},  {T_P4, -1, T_E4A, 128, 4, 1},
    {T_E4A, -1, T_E4, 128, 4, 1},  {T_E4, T_E3, T_D3A, 128, 3, 1}, {T_D3A, -1, T_D3, 128, 3, 1},
    {T_D3, T_E2, T_D2A, 96, 2, 1}, {T_D2A, -1, T_D2, 96, 2, 1},   {T_D2, T_E1, T_D1A, 64, 1, 1},
    {T_D1A, -1, T_D1, 64, 1, 1},   {T_D1, T_E0, T_D0A, 32, 0, 1}, {T_D0A, -1, T_D0, 32, 0, 1},
    {T_D0, -1, -1, 16, 0, 0},
};

inline int layer_cin(int l) {
    const LayerDef& d = kLayerDefs[l];
    return kTensors[d.src0].channels + (d.src1 >= 0 ? kTensors[d.src1].channels : 0);
}

struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    cudaError_t reserve(size_t need) {
        if (need <= bytes && ptr) return cudaSuccess;
        release();
        cudaError_t e = cudaMalloc(&ptr, need > 0 ? need : 16);
        if (e == cudaSuccess) bytes = need > 0 ? need : 16;
        return e;
    }
};

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Round-to-nearest-even FP32 → BF16 (finite inputs).
inline uint16_t to_bf16(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return uint16_t(u >> 16);
}

uint32_t mix32(uint32_t& s) {  // mulberry32
    s += 0x6D2B79F5u;
    uint32_t t = s;
    t = (t ^ (t >> 15)) * (t | 1u);
    t ^= t + (t ^ (t >> 7)) * (t | 61u);
    return t ^ (t >> 14);
}

}  // namespace

struct raymond_net {
    int device = 0;
    int num_sms = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;  // where the network's work is enqueued: its own, or the caller's
    cudaEvent_t ready = nullptr;
    std::string error;

    size_t w_off[kLayers] = {}, b_off[kLayers] = {};
    size_t param_count = 0;
    DevBuf params, params_bf16, grads, adam_m, adam_v, status, loss;
    uint32_t adam_t = 0;
    float w_log = 1.0f, w_rel = 0.0f;  // loss weights
    float rel_eps = kRelEps;           // the relative term's ε
    float tau = kBlendTau;             // the display blend's guard

    DevBuf work;
    int wn = 0, wh = 0, ww = 0;
    bool wtrain = false;
    void* tensor[T_COUNT] = {};
    float* out = nullptr;  // FP32 network output [n][h][w][16]

    int fail(int code, const char* fmt, ...) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        error = buf;
        return code;
    }
    int cuda_fail(cudaError_t e, const char* what) {
        return fail(e == cudaErrorMemoryAllocation ? RAYMOND_ENOMEM : RAYMOND_ECUDA, "%s: %s", what,
                    cudaGetErrorString(e));
    }
    bf16* t(int id) const { return static_cast<bf16*>(tensor[id]); }
    const bf16* weight(int l) const { return static_cast<const bf16*>(params_bf16.ptr) + w_off[l]; }
    const float* bias(int l) const { return static_cast<const float*>(params.ptr) + b_off[l]; }
    float* dweight(int l) const { return static_cast<float*>(grads.ptr) + w_off[l]; }
    float* dbias(int l) const { return static_cast<float*>(grads.ptr) + b_off[l]; }
    unsigned* status_word() const { return static_cast<unsigned*>(status.ptr); }

    cudaError_t reserve_work(int n, int h, int w, bool train) {
        if (work.ptr && n == wn && h == wh && w == ww && (wtrain || !train)) return cudaSuccess;
        size_t off[T_COUNT + 1];
        size_t total = 0;
        const int count = train ? T_COUNT : kFirstGradient;
        for (int i = 0; i < T_COUNT; ++i) {
            off[i] = total;
            if (i >= count) continue;
            const size_t px = size_t(n) * (h >> kTensors[i].level) * (w >> kTensors[i].level);
            total += align_up(px * kTensors[i].channels * sizeof(bf16), 256);
        }
        const size_t out_off = total;
        total += align_up(size_t(n) * h * w * 16 * sizeof(float), 256);
        cudaError_t e = work.reserve(total);
        if (e != cudaSuccess) return e;
        for (int i = 0; i < T_COUNT; ++i)
            tensor[i] = i < count ? static_cast<char*>(work.ptr) + off[i] : nullptr;
        out = reinterpret_cast<float*>(static_cast<char*>(work.ptr) + out_off);
        wn = n;
        wh = h;
        ww = w;
        wtrain = train;
        return cudaSuccess;
    }

    ConvArgs conv_args(int l) const {
        const LayerDef& d = kLayerDefs[l];
        ConvArgs a{};
        a.n = wn;
        a.h = wh >> d.level;
        a.w = ww >> d.level;
        a.cin = layer_cin(l);
        a.cout = d.cout;
        a.src[0] = ConvSrc{t(d.src0), kTensors[d.src0].channels, kTensors[d.src0].channels, d.src1 >= 0 ? 1 : 0};
        if (d.src1 >= 0) a.src[1] = ConvSrc{t(d.src1), kTensors[d.src1].channels, kTensors[d.src1].channels, 0};
        a.wt = weight(l);
        a.bias = bias(l);
        a.act = d.act;
        a.status = status_word();
        return a;
    }

    cudaError_t forward(cudaStream_t st) {
        cudaError_t e = cudaSuccess;
        auto conv = [&](int l) {
            if (e != cudaSuccess) return;
            ConvArgs a = conv_args(l);
            const LayerDef& d = kLayerDefs[l];
            if (d.out >= 0) {
                a.out = t(d.out);
                a.out_stride = d.cout;
            } else {
                a.out_f32 = out;
                a.out_stride = 16;
            }
            e = launch_conv(a, FWD, num_sms, st);
        };
        auto pool = [&](int from, int to, int level) {
            if (e != cudaSuccess) return;
            e = launch_pool(t(from), t(to), wn, wh >> level, ww >> level, kTensors[from].channels, st);
        };
        conv(0);
        conv(1);
        pool(T_E0, T_P1, 0);
        conv(2);
        conv(3);
        pool(T_E1, T_P2, 1);
        conv(4);
        conv(5);
        pool(T_E2, T_P3, 2);
        conv(6);
        conv(7);
        pool(T_E3, T_P4, 3);
        for (int l = 8; l < kLayers; ++l) conv(l);
        return e;
    }

    // Weight and bias gradients of layer l from dy; the input gradient into
    // dx (stride dx_stride) times the slope of `mask` when dx is set.
    cudaError_t backward_layer(int l, const bf16* dy, bf16* dx, int dx_stride, const bf16* mask, cudaStream_t st) {
        ConvArgs a = conv_args(l);
        a.dy = dy;
        a.dy_stride = a.cout;
        a.dw = dweight(l);
        a.db = dbias(l);
        cudaError_t e = launch_conv(a, BWD_WEIGHT, num_sms, st);
        if (e != cudaSuccess || !dx) return e;
        a.out = dx;
        a.out_stride = dx_stride;
        a.mask = mask;
        a.mask_stride = mask ? dx_stride : 0;
        return launch_conv(a, BWD_DATA, num_sms, st);
    }

    cudaError_t backward(cudaStream_t st) {
        cudaError_t e = cudaSuccess;
        auto bw = [&](int l, int dy, int dx, int mask) {
            if (e != cudaSuccess) return;
            const int cin = layer_cin(l);
            e = backward_layer(l, t(dy), dx >= 0 ? t(dx) : nullptr, cin, mask >= 0 ? t(mask) : nullptr, st);
        };
        auto split = [&](int dcat, int coarse_grad, int coarse, int level) {
            if (e != cudaSuccess) return;
            e = launch_split_up(t(dcat), kTensors[dcat].channels, t(coarse_grad), t(coarse), wn, wh >> level,
                                ww >> level, kTensors[coarse].channels, st);
        };
        auto merge = [&](int dcat, int skip_offset, int gpool, int act, int outg, int level) {
            if (e != cudaSuccess) return;
            e = launch_merge(t(dcat) + skip_offset, kTensors[dcat].channels, t(gpool), t(act), t(outg), wn,
                             wh >> level, ww >> level, kTensors[act].channels, st);
        };
        // decoder, top down
        bw(18, T_GOUT, T_GA0, T_D0);
        bw(17, T_GA0, T_GB0, T_D0A);
        bw(16, T_GB0, T_DCAT0, -1);
        split(T_DCAT0, T_GA1, T_D1, 0);
        bw(15, T_GA1, T_GB1, T_D1A);
        bw(14, T_GB1, T_DCAT1, -1);
        split(T_DCAT1, T_GA2, T_D2, 1);
        bw(13, T_GA2, T_GB2, T_D2A);
        bw(12, T_GB2, T_DCAT2, -1);
        split(T_DCAT2, T_GA3, T_D3, 2);
        bw(11, T_GA3, T_GB3, T_D3A);
        bw(10, T_GB3, T_DCAT3, -1);
        split(T_DCAT3, T_GA4, T_E4, 3);
        // encoder, bottom up
        bw(9, T_GA4, T_GB4, T_E4A);
        bw(8, T_GB4, T_GA4, -1);  // gradient of the pooled P4
        merge(T_DCAT3, 128, T_GA4, T_E3, T_GA3, 3);
        bw(7, T_GA3, T_GB3, T_E3A);
        bw(6, T_GB3, T_GA3, -1);  // P3
        merge(T_DCAT2, 128, T_GA3, T_E2, T_GA2, 2);
        bw(5, T_GA2, T_GB2, T_E2A);
        bw(4, T_GB2, T_GA2, -1);  // P2
        merge(T_DCAT1, 96, T_GA2, T_E1, T_GA1, 1);
        bw(3, T_GA1, T_GB1, T_E1A);
        bw(2, T_GB1, T_GA1, -1);  // P1
        merge(T_DCAT0, 64, T_GA1, T_E0, T_GA0, 0);
        bw(1, T_GA0, T_GB0, T_E0A);
        bw(0, T_GB0, -1, -1);
        return e;
    }
};

// ---------------------------------------------------------------- shared validation

static int check_batch(raymond_net* net, const raymond_net_batch* b, bool need_target, bool multiple_of_16) {
    if (!b) return net->fail(RAYMOND_EINVAL, "No batch.");
    if (b->n == 0 || b->width == 0 || b->height == 0) return net->fail(RAYMOND_EINVAL, "Empty batch.");
    if (!b->accum || !b->albedo || !b->normal) return net->fail(RAYMOND_EINVAL, "The batch needs accum, albedo and normal.");
    if (need_target && !b->target) return net->fail(RAYMOND_EINVAL, "Training needs a target.");
    if (multiple_of_16 && (b->width % 16 || b->height % 16))
        return net->fail(RAYMOND_EINVAL, "Training crops must be multiples of 16 pixels wide and high.");
    if (!b->samples && !(b->samples_all >= 1.0f)) return net->fail(RAYMOND_EINVAL, "Sample counts must be at least 1.");
    const uint64_t px = uint64_t(b->n) * ((b->height + 15) / 16 * 16) * ((b->width + 15) / 16 * 16);
    if (px >= (uint64_t(1) << 31) / 16) return net->fail(RAYMOND_EINVAL, "Batch too large.");
    return RAYMOND_OK;
}

static cudaError_t run_features(raymond_net* net, const raymond_net_batch* b, cudaStream_t st) {
    FeatureArgs f{};
    f.accum = reinterpret_cast<const float4*>(b->accum);
    f.albedo = reinterpret_cast<const float4*>(b->albedo);
    f.normal = reinterpret_cast<const float4*>(b->normal);
    f.samples = b->samples;
    f.samples_all = b->samples_all;
    f.n = net->wn;
    f.h = net->wh;
    f.w = net->ww;
    f.src_h = int(b->height);
    f.src_w = int(b->width);
    f.out = net->t(T_IN);
    return launch_features(f, st);
}

static cudaError_t run_loss(raymond_net* net, const raymond_net_batch* b, cudaStream_t st) {
    LossArgs L{};
    L.out = net->out;
    L.accum = reinterpret_cast<const float4*>(b->accum);
    L.albedo = reinterpret_cast<const float4*>(b->albedo);
    L.target = reinterpret_cast<const float4*>(b->target);
    L.samples = b->samples;
    L.samples_all = b->samples_all;
    L.n = net->wn;
    L.h = net->wh;
    L.w = net->ww;
    L.src_h = int(b->height);
    L.src_w = int(b->width);
    L.scale = 1.0f / (3.0f * float(b->n) * float(b->width) * float(b->height));
    L.w_log = net->w_log;
    L.w_rel = net->w_rel;
    L.rel_eps = net->rel_eps;
    L.tau = net->tau;
    L.grad = net->t(T_GOUT);
    L.loss = static_cast<float*>(net->loss.ptr);
    return launch_loss(L, st);
}

// Forward, loss and backward into net->grads (zeroed first).
static int run_gradients(raymond_net* net, const raymond_net_batch* b) {
    cudaError_t e = net->reserve_work(int(b->n), int(b->height), int(b->width), true);
    if (e != cudaSuccess) return net->cuda_fail(e, "network memory");
    cudaStream_t st = net->stream;
    e = cudaMemsetAsync(net->grads.ptr, 0, net->param_count * sizeof(float), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(net->loss.ptr, 0, sizeof(float), st);
    if (e == cudaSuccess) e = run_features(net, b, st);
    if (e == cudaSuccess) e = net->forward(st);
    if (e == cudaSuccess) e = run_loss(net, b, st);
    if (e == cudaSuccess) e = net->backward(st);
    return e == cudaSuccess ? RAYMOND_OK : net->cuda_fail(e, "training step");
}

static int finish(raymond_net* net, float* loss_out) {
    unsigned status = 0;
    cudaError_t e = cudaMemcpyAsync(&status, net->status.ptr, sizeof status, cudaMemcpyDeviceToHost, net->stream);
    if (e == cudaSuccess && loss_out)
        e = cudaMemcpyAsync(loss_out, net->loss.ptr, sizeof(float), cudaMemcpyDeviceToHost, net->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(net->stream);
    if (e != cudaSuccess) return net->cuda_fail(e, "network read-back");
    if (status) {
        cudaMemsetAsync(net->status.ptr, 0, sizeof(unsigned), net->stream);
        return net->fail(RAYMOND_ETIMEOUT, "A tensor-core wait ran out of time (status %u).", status);
    }
    return RAYMOND_OK;
}

// ---------------------------------------------------------------- C ABI

extern "C" {

int raymond_net_create(raymond_net** out, const raymond_net_config* cfg) {
    if (!out) return RAYMOND_EINVAL;
    *out = nullptr;
    const int device = cfg ? cfg->device : 0;
    const uint32_t seed = cfg ? cfg->seed : 1u;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
        rmd::set_handleless_error("No CUDA device with that index.");
        return RAYMOND_ECUDA;
    }
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, device);
    if (prop.major != 10 || prop.minor != 3) {
        rmd::set_handleless_error("The denoiser's tensor-core kernels are built for sm_103a only.");
        return RAYMOND_ECUDA;
    }
    raymond_net* net = new raymond_net;
    net->device = device;
    net->num_sms = prop.multiProcessorCount;
    cudaSetDevice(device);
    cudaError_t e = cudaStreamCreateWithFlags(&net->own_stream, cudaStreamNonBlocking);
    net->stream = net->own_stream;
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&net->ready, cudaEventDisableTiming);
    size_t off = 0;
    for (int l = 0; l < kLayers; ++l) {
        net->w_off[l] = off;
        off += align_up(size_t(kLayerDefs[l].cout) * 9 * layer_cin(l), 64);
        net->b_off[l] = off;
        off += align_up(size_t(kLayerDefs[l].cout), 64);
    }
    net->param_count = off;
    const size_t fb = off * sizeof(float);
    if (e == cudaSuccess) e = net->params.reserve(fb);
    if (e == cudaSuccess) e = net->params_bf16.reserve(off * sizeof(bf16));
    if (e == cudaSuccess) e = net->grads.reserve(fb);
    if (e == cudaSuccess) e = net->adam_m.reserve(fb);
    if (e == cudaSuccess) e = net->adam_v.reserve(fb);
    if (e == cudaSuccess) e = net->status.reserve(sizeof(unsigned));
    if (e == cudaSuccess) e = net->loss.reserve(sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(net->status.ptr, 0, sizeof(unsigned));
    if (e != cudaSuccess) {
        rmd::set_handleless_error(cudaGetErrorString(e));
        raymond_net_destroy(net);
        return e == cudaErrorMemoryAllocation ? RAYMOND_ENOMEM : RAYMOND_ECUDA;
    }
    // He-uniform weights for the leaky ReLU; the last layer starts small.
    std::vector<float> p(off, 0.0f);
    uint32_t s = seed;
    for (int l = 0; l < kLayers; ++l) {
        const int fan_in = 9 * layer_cin(l);
        float bound = std::sqrt(6.0f / ((1.0f + kLeak * kLeak) * float(fan_in)));
        if (kLayerDefs[l].out < 0) bound *= 0.1f;
        const size_t nw = size_t(kLayerDefs[l].cout) * fan_in;
        for (size_t i = 0; i < nw; ++i)
            p[net->w_off[l] + i] = (float(mix32(s)) * (1.0f / 4294967296.0f) * 2.0f - 1.0f) * bound;
    }
    int rc = raymond_net_set_params(net, p.data(), off);
    if (rc) {
        rmd::set_handleless_error(net->error.c_str());
        raymond_net_destroy(net);
        return rc;
    }
    *out = net;
    return RAYMOND_OK;
}

void raymond_net_destroy(raymond_net* net) {
    if (!net) return;
    cudaSetDevice(net->device);
    if (net->stream) cudaStreamSynchronize(net->stream);
    for (DevBuf* b : {&net->params, &net->params_bf16, &net->grads, &net->adam_m, &net->adam_v, &net->status,
                      &net->loss, &net->work})
        b->release();
    if (net->ready) cudaEventDestroy(net->ready);
    if (net->own_stream) cudaStreamDestroy(net->own_stream);
    delete net;
}

const char* raymond_net_last_error(const raymond_net* net) { return net ? net->error.c_str() : ""; }

uint64_t raymond_net_param_count(const raymond_net* net) { return net ? net->param_count : 0; }

int raymond_net_layout(const raymond_net* net, uint64_t* weight_offsets, uint64_t* bias_offsets, uint32_t* cin,
                       uint32_t* cout, uint32_t layers) {
    if (!net || layers < uint32_t(kLayers)) return RAYMOND_EINVAL;
    for (int l = 0; l < kLayers; ++l) {
        if (weight_offsets) weight_offsets[l] = net->w_off[l];
        if (bias_offsets) bias_offsets[l] = net->b_off[l];
        if (cin) cin[l] = uint32_t(layer_cin(l));
        if (cout) cout[l] = uint32_t(kLayerDefs[l].cout);
    }
    return RAYMOND_OK;
}

int raymond_net_set_params(raymond_net* net, const float* params, uint64_t count) {
    if (!net) return RAYMOND_EINVAL;
    if (!params || count != net->param_count)
        return net->fail(RAYMOND_EINVAL, "Expected %llu parameters.", (unsigned long long)net->param_count);
    std::vector<uint16_t> h(count);
    for (uint64_t i = 0; i < count; ++i) {
        if (!std::isfinite(params[i])) return net->fail(RAYMOND_EINVAL, "Parameter %llu is not finite.", (unsigned long long)i);
        h[i] = to_bf16(params[i]);
    }
    cudaSetDevice(net->device);
    cudaError_t e = cudaMemcpyAsync(net->params.ptr, params, count * 4, cudaMemcpyHostToDevice, net->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(net->params_bf16.ptr, h.data(), count * 2, cudaMemcpyHostToDevice, net->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(net->adam_m.ptr, 0, count * 4, net->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(net->adam_v.ptr, 0, count * 4, net->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(net->stream);
    net->adam_t = 0;
    return e == cudaSuccess ? RAYMOND_OK : net->cuda_fail(e, "set parameters");
}

int raymond_net_get_params(raymond_net* net, float* params, uint64_t count) {
    if (!net) return RAYMOND_EINVAL;
    if (!params || count != net->param_count)
        return net->fail(RAYMOND_EINVAL, "Expected %llu parameters.", (unsigned long long)net->param_count);
    cudaSetDevice(net->device);
    cudaError_t e = cudaMemcpyAsync(params, net->params.ptr, count * 4, cudaMemcpyDeviceToHost, net->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(net->stream);
    return e == cudaSuccess ? RAYMOND_OK : net->cuda_fail(e, "get parameters");
}

int raymond_net_gradients(raymond_net* net, const raymond_net_batch* batch, float* grads, uint64_t count, float* loss) {
    if (!net) return RAYMOND_EINVAL;
    int rc = check_batch(net, batch, true, true);
    if (rc) return rc;
    if (grads && count != net->param_count)
        return net->fail(RAYMOND_EINVAL, "Expected %llu gradients.", (unsigned long long)net->param_count);
    cudaSetDevice(net->device);
    if ((rc = run_gradients(net, batch))) return rc;
    if (grads) {
        cudaError_t e = cudaMemcpyAsync(grads, net->grads.ptr, count * 4, cudaMemcpyDeviceToHost, net->stream);
        if (e != cudaSuccess) return net->cuda_fail(e, "gradient read-back");
    }
    return finish(net, loss);
}

int raymond_net_train_step(raymond_net* net, const raymond_net_batch* batch, float learning_rate, float* loss) {
    if (!net) return RAYMOND_EINVAL;
    int rc = check_batch(net, batch, true, true);
    if (rc) return rc;
    if (!(learning_rate > 0.0f)) return net->fail(RAYMOND_EINVAL, "The learning rate must be positive.");
    cudaSetDevice(net->device);
    if ((rc = run_gradients(net, batch))) return rc;
    net->adam_t += 1;
    const double b1 = 0.9, b2 = 0.999, eps = 1e-8;
    const double c1 = 1.0 - std::pow(b1, double(net->adam_t)), c2 = 1.0 - std::pow(b2, double(net->adam_t));
    AdamArgs A{};
    A.param = static_cast<float*>(net->params.ptr);
    A.param_bf16 = static_cast<bf16*>(net->params_bf16.ptr);
    A.grad = static_cast<const float*>(net->grads.ptr);
    A.m = static_cast<float*>(net->adam_m.ptr);
    A.v = static_cast<float*>(net->adam_v.ptr);
    A.count = net->param_count;
    A.beta1 = float(b1);
    A.beta2 = float(b2);
    A.step = float(learning_rate * std::sqrt(c2) / c1);
    A.eps_hat = float(eps * std::sqrt(c2));
    cudaError_t e = launch_adam(A, net->stream);
    if (e != cudaSuccess) return net->cuda_fail(e, "adam");
    return loss ? finish(net, loss) : RAYMOND_OK;
}

int raymond_net_set_loss(raymond_net* net, float w_log, float w_rel, float rel_eps) {
    if (!net) return RAYMOND_EINVAL;
    if (!(w_log >= 0.0f) || !(w_rel >= 0.0f) || !(w_log + w_rel > 0.0f) || !std::isfinite(w_log + w_rel))
        return net->fail(RAYMOND_EINVAL, "Loss weights must be finite, non-negative and not both zero.");
    if (!(rel_eps > 0.0f) || !std::isfinite(rel_eps))
        return net->fail(RAYMOND_EINVAL, "The relative error's epsilon must be finite and positive.");
    net->w_log = w_log;
    net->w_rel = w_rel;
    net->rel_eps = rel_eps;
    return RAYMOND_OK;
}

int raymond_net_set_blend(raymond_net* net, float tau) {
    if (!net) return RAYMOND_EINVAL;
    if (!(tau > 0.0f) || !std::isfinite(tau)) return net->fail(RAYMOND_EINVAL, "The blend guard must be finite and positive.");
    net->tau = tau;
    return RAYMOND_OK;
}

float raymond_net_get_blend(const raymond_net* net) { return net ? net->tau : 0.0f; }

int raymond_net_sync(raymond_net* net) {
    if (!net) return RAYMOND_EINVAL;
    cudaSetDevice(net->device);
    return finish(net, nullptr);
}

int raymond_net_infer(raymond_net* net, const raymond_net_batch* batch, float* out_rgba, void* stream) {
    if (!net) return RAYMOND_EINVAL;
    int rc = check_batch(net, batch, false, false);
    if (rc) return rc;
    if (!out_rgba) return net->fail(RAYMOND_EINVAL, "No output buffer.");
    cudaSetDevice(net->device);
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : net->stream;
    const int n = int(batch->n), h = int(batch->height), w = int(batch->width);
    const int ph = (h + 15) / 16 * 16, pw = (w + 15) / 16 * 16;
    if (st != net->stream) {
        // The workspace belongs to the network's stream: order against it.
        cudaEventRecord(net->ready, net->stream);
        cudaStreamWaitEvent(st, net->ready, 0);
    }
    cudaError_t e = net->reserve_work(n, ph, pw, false);
    if (e != cudaSuccess) return net->cuda_fail(e, "network memory");
    e = run_features(net, batch, st);
    if (e == cudaSuccess) e = net->forward(st);
    if (e == cudaSuccess) {
        ComposeArgs C{};
        C.out = net->out;
        C.accum = reinterpret_cast<const float4*>(batch->accum);
        C.albedo = reinterpret_cast<const float4*>(batch->albedo);
        C.samples = batch->samples;
        C.samples_all = batch->samples_all;
        C.n = n;
        C.w = w;
        C.h = h;
        C.pw = pw;
        C.ph = ph;
        C.tau = net->tau;
        C.dst = reinterpret_cast<float4*>(out_rgba);
        e = launch_compose(C, st);
    }
    if (e != cudaSuccess) return net->cuda_fail(e, "inference");
    if (st != net->stream) {
        cudaEventRecord(net->ready, st);
        cudaStreamWaitEvent(net->stream, net->ready, 0);
    }
    return RAYMOND_OK;
}

void* raymond_net_get_stream(raymond_net* net) { return net ? static_cast<void*>(net->stream) : nullptr; }

int raymond_net_set_stream(raymond_net* net, void* stream) {
    if (!net) return RAYMOND_EINVAL;
    cudaSetDevice(net->device);
    cudaStream_t next = stream ? static_cast<cudaStream_t>(stream) : net->own_stream;
    if (next != net->stream) {
        // Work already enqueued on the old stream comes first.
        cudaEventRecord(net->ready, net->stream);
        cudaStreamWaitEvent(next, net->ready, 0);
        net->stream = next;
    }
    return RAYMOND_OK;
}

// ---- single kernels, on caller memory

static int conv_entry(const raymond_conv* c, void* stream, int mode) {
    if (!c) {
        rmd::set_handleless_error("No convolution description.");
        return RAYMOND_EINVAL;
    }
    ConvArgs a{};
    a.n = int(c->n);
    a.h = int(c->height);
    a.w = int(c->width);
    a.cin = int(c->cin);
    a.cout = int(c->cout);
    a.src[0] = ConvSrc{static_cast<const bf16*>(c->src0), int(c->src0_channels), int(c->src0_stride), int(c->src0_shift)};
    a.src[1] = ConvSrc{static_cast<const bf16*>(c->src1), int(c->src1_channels), int(c->src1_stride), int(c->src1_shift)};
    a.wt = static_cast<const bf16*>(c->weight);
    a.bias = c->bias;
    a.dy = static_cast<const bf16*>(c->dy);
    a.dy_stride = int(c->dy_stride);
    a.out = static_cast<bf16*>(c->out);
    a.out_stride = int(c->out_stride);
    a.out_f32 = c->out_f32;
    a.mask = static_cast<const bf16*>(c->mask);
    a.mask_stride = int(c->mask_stride);
    a.dw = c->dweight;
    a.db = c->dbias;
    a.act = c->activation;
    a.pixels_per_cta = int(c->pixels_per_cta);
    a.status = c->status;
    a.kernel = int(c->kernel);
    if (mode == BWD_WEIGHT && a.pixels_per_cta == 0) a.pixels_per_cta = 64;  // replaced by the launcher
    if (const char* why = check_conv(a, mode)) {
        rmd::set_handleless_error(why);
        return RAYMOND_EINVAL;
    }
    if (mode == BWD_WEIGHT && c->pixels_per_cta == 0) a.pixels_per_cta = 0;
    if (a.kernel < CONV_AUTO || a.kernel > CONV_HALO) {
        rmd::set_handleless_error("conv: kernel must be 0 (choose), 1 (pixel rows) or 2 (halo tiles)");
        return RAYMOND_EINVAL;
    }
    if (a.kernel == CONV_HALO && !conv_halo_fits(a, mode)) {
        rmd::set_handleless_error("conv: the weights do not fit in shared memory for halo tiles");
        return RAYMOND_EINVAL;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = launch_conv(a, mode, sms, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) {
        rmd::set_handleless_error(cudaGetErrorString(e));
        return RAYMOND_ECUDA;
    }
    return RAYMOND_OK;
}

int raymond_conv3x3_forward(const raymond_conv* c, void* stream) { return conv_entry(c, stream, FWD); }
int raymond_conv3x3_backward_data(const raymond_conv* c, void* stream) { return conv_entry(c, stream, BWD_DATA); }
int raymond_conv3x3_backward_weight(const raymond_conv* c, void* stream) { return conv_entry(c, stream, BWD_WEIGHT); }

}  // extern "C"

// Used by the renderer's raymond_denoise_learned: the network over one
// renderer's buffers, on the renderer's stream.
int rmd_net_denoise(raymond_net* net, const float* accum, const float* albedo, const float* normal, float samples,
                    uint32_t w, uint32_t h, float* dst, void* stream, std::string* err) {
    int dev = -1;
    cudaGetDevice(&dev);
    if (dev != net->device) {
        if (err) *err = "The network lives on another GPU than the renderer.";
        return RAYMOND_EINVAL;
    }
    raymond_net_batch b{};
    b.accum = accum;
    b.albedo = albedo;
    b.normal = normal;
    b.samples_all = samples;
    b.n = 1;
    b.width = w;
    b.height = h;
    const int rc = raymond_net_infer(net, &b, dst, stream);
    if (rc && err) *err = net->error;
    return rc;
}
