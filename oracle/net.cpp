// Oracle of the learned denoiser — TEST INFRASTRUCTURE ONLY.
//
// A direct (no GEMM) double-precision restatement of the network that the
// product runs on the tensor cores: 3×3 convolutions with zero padding, the
// leaky ReLU (slope 0.1), 2×2 average pooling, nearest-neighbour upsampling
// concatenated ahead of the skip input, the 12 input features, the display
// (the network's predicted radiance blended with the running average by a
// predicted weight), the loss (weighted L1 on log radiance over albedo plus
// relative squared error of the display), and reverse-mode gradients over the graph in
// plain forward order reversed. With `bf16` set, weights and every stored
// activation and output-gradient tensor are rounded to BF16 as the GPU
// stores them, so the two can be compared closely; without it the oracle is
// smooth enough for finite-difference checks of its own gradients.
//
// The network has no counterpart in the reference (its only denoiser is the
// à-trous filter, src/shaders.mjs:1916-2098); the feature definitions follow
// that filter's demodulation (albedo clamped at 0.01, src/shaders.mjs:1987-2017).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "oracle.h"

namespace {

double round_bf16(double v) {
    float f = float(v);
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7F800000u) == 0x7F800000u) return v;
    u += 0x7FFFu + ((u >> 16) & 1u);
    u &= 0xFFFF0000u;
    std::memcpy(&f, &u, 4);
    return f;
}

struct T {
    int n = 0, h = 0, w = 0, c = 0;
    std::vector<double> v;
    void init(int n_, int h_, int w_, int c_) {
        n = n_;
        h = h_;
        w = w_;
        c = c_;
        v.assign(size_t(n) * h * w * c, 0.0);
    }
    double& at(int i, int y, int x, int ch) { return v[((size_t(i) * h + y) * w + x) * c + ch]; }
    double at(int i, int y, int x, int ch) const { return v[((size_t(i) * h + y) * w + x) * c + ch]; }
};

const double kLeak = 0.1;
const double kMaxLog = 8.0;    // the prediction's exponent is clamped to ±this
const double kMaxGrad = 64.0;  // and clips each element's gradient to ±this (before scaling)
const double kBlendTau = 0.1;   // the blend guard's relative error scale (off below 4 samples)

// Layer table: sources (tensor ids), output id, cout, activation.
enum { IN, E0A, E0, P1, E1A, E1, P2, E2A, E2, P3, E3A, E3, P4, E4A, E4, D3A, D3, D2A, D2, D1A, D1, D0A, D0, OUT, NT };
struct Layer {
    int s0, s1, out, cout, act;
};
const Layer kNet[19] = {
    {IN, -1, E0A, 32, 1},  {E0A, -1, E0, 32, 1},  {P1, -1, E1A, 64, 1},   {E1A, -1, E1, 64, 1},
    {P2, -1, E2A, 96, 1},  {E2A, -1, E2, 96, 1},  {P3, -1, E3A, 128, 1},  {E3A, -1, E3, 128, 1},
    {P4, -1, E4A, 128, 1}, {E4A, -1, E4, 128, 1}, {E4, E3, D3A, 128, 1},  {D3A, -1, D3, 128, 1},
    {D3, E2, D2A, 96, 1},  {D2A, -1, D2, 96, 1},  {D2, E1, D1A, 64, 1},   {D1A, -1, D1, 64, 1},
    {D1, E0, D0A, 32, 1},  {D0A, -1, D0, 32, 1},  {D0, -1, OUT, 16, 0},
};
const int kWidth[NT] = {16, 32, 32, 32, 64, 64, 64, 96, 96, 96, 128, 128, 128, 128, 128,
                        128, 128, 96, 96, 64, 64, 32, 32, 16};
const int kLevel[NT] = {0, 0, 0, 1, 1, 1, 2, 2, 2, 3, 3, 3, 4, 4, 4, 3, 3, 2, 2, 1, 1, 0, 0, 0};

int cin_of(int l) { return kWidth[kNet[l].s0] + (kNet[l].s1 >= 0 ? kWidth[kNet[l].s1] : 0); }

size_t up64(size_t v) { return (v + 63) / 64 * 64; }

void layout(uint64_t* w_off, uint64_t* b_off, uint64_t* total) {
    size_t off = 0;
    for (int l = 0; l < 19; ++l) {
        if (w_off) w_off[l] = off;
        off += up64(size_t(kNet[l].cout) * 9 * cin_of(l));
        if (b_off) b_off[l] = off;
        off += up64(size_t(kNet[l].cout));
    }
    if (total) *total = off;
}

// Input value of channel ch at (i, y, x) of a concatenation of s0
// (upsampled when `up`) and s1; zero outside the image.
double in_at(const T& s0, const T* s1, bool up, int i, int y, int x, int ch, int H, int W) {
    if (y < 0 || x < 0 || y >= H || x >= W) return 0.0;
    if (ch < s0.c) return up ? s0.at(i, y >> 1, x >> 1, ch) : s0.at(i, y, x, ch);
    return s1->at(i, y, x, ch - s0.c);
}

void conv_forward(const T& s0, const T* s1, bool up, int H, int W, const double* wt, const double* b, int cout, int act,
                  T& out) {
    const int cin = s0.c + (s1 ? s1->c : 0);
    out.init(s0.n, H, W, cout);
    std::vector<double> col(9 * cin);
    for (int i = 0; i < s0.n; ++i)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                for (int tap = 0; tap < 9; ++tap)
                    for (int ch = 0; ch < cin; ++ch)
                        col[tap * cin + ch] = in_at(s0, s1, up, i, y + tap / 3 - 1, x + tap % 3 - 1, ch, H, W);
                for (int co = 0; co < cout; ++co) {
                    const double* wr = wt + size_t(co) * 9 * cin;
                    double acc = b[co];
                    for (int k = 0; k < 9 * cin; ++k) acc += wr[k] * col[k];
                    if (act && acc <= 0.0) acc *= kLeak;
                    out.at(i, y, x, co) = acc;
                }
            }
}

// dy: gradient before the activation. Adds into dw, db; writes dx over the
// concatenated input channels (full resolution).
void conv_backward(const T& s0, const T* s1, bool up, int H, int W, const double* wt, const T& dy, double* dw,
                   double* db, T* dx) {
    const int cin = s0.c + (s1 ? s1->c : 0), cout = dy.c;
    if (dx) dx->init(s0.n, H, W, cin);
    std::vector<double> col(9 * cin);
    for (int i = 0; i < s0.n; ++i)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                for (int tap = 0; tap < 9; ++tap)
                    for (int ch = 0; ch < cin; ++ch)
                        col[tap * cin + ch] = in_at(s0, s1, up, i, y + tap / 3 - 1, x + tap % 3 - 1, ch, H, W);
                for (int co = 0; co < cout; ++co) {
                    const double g = dy.at(i, y, x, co);
                    if (g == 0.0) continue;
                    db[co] += g;
                    double* wr = dw + size_t(co) * 9 * cin;
                    for (int k = 0; k < 9 * cin; ++k) wr[k] += g * col[k];
                    if (dx) {
                        const double* wv = wt + size_t(co) * 9 * cin;
                        for (int tap = 0; tap < 9; ++tap) {
                            const int yy = y + tap / 3 - 1, xx = x + tap % 3 - 1;
                            if (yy < 0 || xx < 0 || yy >= H || xx >= W) continue;
                            for (int ch = 0; ch < cin; ++ch) dx->at(i, yy, xx, ch) += g * wv[tap * cin + ch];
                        }
                    }
                }
            }
}

void pool(const T& in, T& out) {
    out.init(in.n, in.h / 2, in.w / 2, in.c);
    for (int i = 0; i < in.n; ++i)
        for (int y = 0; y < out.h; ++y)
            for (int x = 0; x < out.w; ++x)
                for (int ch = 0; ch < in.c; ++ch)
                    out.at(i, y, x, ch) = 0.25 * (in.at(i, 2 * y, 2 * x, ch) + in.at(i, 2 * y, 2 * x + 1, ch) +
                                                  in.at(i, 2 * y + 1, 2 * x, ch) + in.at(i, 2 * y + 1, 2 * x + 1, ch));
}

void round_all(T& t) {
    for (double& v : t.v) v = round_bf16(v);
}

double lum(double r, double g, double b) { return r * 0.2126 + g * 0.7152 + b * 0.0722; }

void features(const float* accum, const float* albedo, const float* normal, const float* samples, int n, int h, int w,
              T& out) {
    out.init(n, h, w, 16);
    for (int i = 0; i < n; ++i)
        for (int y = 0; y < h; ++y)
            for (int x = 0; x < w; ++x) {
                const size_t p = (size_t(i) * h + y) * w + x;
                const double s = std::fmax(double(samples[i]), 1.0);
                const float* ac = accum + 4 * p;
                const float* al = albedo + 4 * p;
                const float* nr = normal + 4 * p;
                const double a[3] = {std::fmax(al[0] / s, 0.01), std::fmax(al[1] / s, 0.01), std::fmax(al[2] / s, 0.01)};
                const double m[3] = {ac[0] / s, ac[1] / s, ac[2] / s};
                double v[16] = {};
                for (int c = 0; c < 3; ++c) v[c] = std::log1p(std::fmax(m[c] / a[c], 0.0));
                for (int c = 0; c < 3; ++c) v[3 + c] = a[c];
                const double d2 = double(nr[0]) * nr[0] + double(nr[1]) * nr[1] + double(nr[2]) * nr[2];
                if (d2 > 0.0) {
                    const double il = 1.0 / std::sqrt(d2);
                    for (int c = 0; c < 3; ++c) v[6 + c] = nr[c] * il;
                }
                v[9] = std::log1p(std::fmax(nr[3] / s, 0.0));
                const double ml = lum(m[0], m[1], m[2]);
                const double var = std::fmax(ac[3] / s - ml * ml, 0.0) / s;
                v[10] = std::log1p(std::sqrt(var));
                v[11] = 1.0 / std::sqrt(s);
                for (int c = 0; c < 16; ++c) out.at(i, y, x, c) = v[c];
            }
}

}  // namespace

extern "C" {

uint64_t ro_net_param_count(void) {
    uint64_t total = 0;
    layout(nullptr, nullptr, &total);
    return total;
}

void ro_net_layout(uint64_t* w_off, uint64_t* b_off, uint32_t* cin, uint32_t* cout) {
    layout(w_off, b_off, nullptr);
    for (int l = 0; l < 19; ++l) {
        if (cin) cin[l] = uint32_t(cin_of(l));
        if (cout) cout[l] = uint32_t(kNet[l].cout);
    }
}

double ro_net_loss_grad(const double* params, const float* accum, const float* albedo, const float* normal,
                        const float* target, const float* samples, uint32_t n, uint32_t h, uint32_t w, int bf16,
                        double w_log, double w_rel, double rel_eps, double* grads, float* out16) {
    uint64_t w_off[19], b_off[19], total = 0;
    layout(w_off, b_off, &total);
    std::vector<double> p(params, params + total);
    if (bf16)
        for (int l = 0; l < 19; ++l) {
            const size_t nw = size_t(kNet[l].cout) * 9 * cin_of(l);
            for (size_t k = 0; k < nw; ++k) p[w_off[l] + k] = round_bf16(p[w_off[l] + k]);
        }
    T t[NT];
    features(accum, albedo, normal, samples, int(n), int(h), int(w), t[IN]);
    if (bf16) round_all(t[IN]);
    auto run = [&](int l) {
        const Layer& L = kNet[l];
        const int lev = kLevel[L.out];
        conv_forward(t[L.s0], L.s1 >= 0 ? &t[L.s1] : nullptr, L.s1 >= 0, int(h) >> lev, int(w) >> lev,
                     p.data() + w_off[l], p.data() + b_off[l], L.cout, L.act, t[L.out]);
        if (bf16 && L.out != OUT) round_all(t[L.out]);
    };
    auto do_pool = [&](int from, int to) {
        pool(t[from], t[to]);
        if (bf16) round_all(t[to]);
    };
    run(0);
    run(1);
    do_pool(E0, P1);
    run(2);
    run(3);
    do_pool(E1, P2);
    run(4);
    run(5);
    do_pool(E2, P3);
    run(6);
    run(7);
    do_pool(E3, P4);
    for (int l = 8; l < 19; ++l) run(l);
    if (out16)
        for (size_t k = 0; k < t[OUT].v.size(); ++k) out16[k] = float(t[OUT].v[k]);

    // The display f blends the prediction p = a·e^o with the running average
    // by alpha = sigmoid(out[3]) · guard; the loss is lg(f) + lg(p), lg(v) = w_log ·
    // |log(1 + v/a) − log(1 + t/a)| + w_rel · (v − t)² / (v² + rel_eps) with
    // the relative term's denominator held constant.
    const double scale = 1.0 / (3.0 * double(n) * h * w);
    double loss = 0.0;
    T g[NT];
    g[OUT].init(int(n), int(h), int(w), 16);
    auto lg = [&](double v, double tc, double a, double* l) {
        const double d = std::log1p(v / a) - std::log1p(std::fmax(tc / a, 0.0));
        const double e = v - tc;
        const double den = v * v + rel_eps;
        *l += w_log * std::fabs(d) + w_rel * e * e / den;
        return w_log * (d > 0 ? 1.0 : d < 0 ? -1.0 : 0.0) / (a + v) + w_rel * 2.0 * e / den;
    };
    for (uint32_t i = 0; i < n; ++i)
        for (uint32_t y = 0; y < h; ++y)
            for (uint32_t x = 0; x < w; ++x) {
                const size_t q = (size_t(i) * h + y) * w + x;
                const double s = std::fmax(double(samples[i]), 1.0);
                const double z = std::fmin(std::fmax(t[OUT].at(int(i), int(y), int(x), 3), -20.0), 20.0);
                const double gate = 1.0 / (1.0 + std::exp(-z));
                // guard: the average's relative variance of the mean luminance v, v/(v + tau²)
                const double mr = std::fmax(accum[4 * q] / s, 0.0), mg = std::fmax(accum[4 * q + 1] / s, 0.0),
                             mb = std::fmax(accum[4 * q + 2] / s, 0.0);
                const double ml = lum(mr, mg, mb);
                const double vm = std::fmax(accum[4 * q + 3] / s - ml * ml, 0.0) / s;
                const double v = vm / (ml * ml + 1e-4);
                const double guard = s < 4.0 ? 1.0 : v / (v + kBlendTau * kBlendTau);
                const double alpha = gate * guard;
                double g_alpha = 0.0;
                for (int c = 0; c < 3; ++c) {
                    const double a = std::fmax(albedo[4 * q + c] / s, 0.01);
                    const double m = std::fmax(accum[4 * q + c] / s, 0.0);
                    const double o = t[OUT].at(int(i), int(y), int(x), c);
                    const double pred = std::exp(std::fmin(std::fmax(o, -kMaxLog), kMaxLog)) * a;
                    const double fin = alpha * pred + (1.0 - alpha) * m;
                    const double tc = target[4 * q + c];
                    const double gf = lg(fin, tc, a, &loss);
                    const double gp = lg(pred, tc, a, &loss);
                    g_alpha += gf * (pred - m);
                    const double go = (gf * alpha + gp) * pred;  // through the clamp as if unclamped
                    g[OUT].at(int(i), int(y), int(x), c) = std::fmin(std::fmax(go, -kMaxGrad), kMaxGrad) * scale;
                }
                const double ga = g_alpha * guard * gate * (1.0 - gate);
                g[OUT].at(int(i), int(y), int(x), 3) = std::fmin(std::fmax(ga, -kMaxGrad), kMaxGrad) * scale;
            }
    loss *= scale;
    if (!grads) return loss;
    std::memset(grads, 0, total * sizeof(double));
    if (bf16) round_all(g[OUT]);

    for (int id = 0; id < NT; ++id)
        if (id != OUT) g[id].init(t[id].n, t[id].h, t[id].w, t[id].c);
    auto back = [&](int l) {
        const Layer& L = kNet[l];
        const int lev = kLevel[L.out];
        const int H = int(h) >> lev, W = int(w) >> lev;
        T dy = g[L.out];
        if (L.act)
            for (size_t k = 0; k < dy.v.size(); ++k)
                if (t[L.out].v[k] <= 0.0) dy.v[k] *= kLeak;
        if (bf16) round_all(dy);
        T dx;
        conv_backward(t[L.s0], L.s1 >= 0 ? &t[L.s1] : nullptr, L.s1 >= 0, H, W, p.data() + w_off[l], dy,
                      grads + w_off[l], grads + b_off[l], l > 0 ? &dx : nullptr);
        if (l == 0) return;
        const int c0 = t[L.s0].c;
        for (int i = 0; i < dx.n; ++i)
            for (int y = 0; y < H; ++y)
                for (int x = 0; x < W; ++x)
                    for (int ch = 0; ch < dx.c; ++ch) {
                        const double v = dx.at(i, y, x, ch);
                        if (ch < c0) {
                            if (L.s1 >= 0) g[L.s0].at(i, y >> 1, x >> 1, ch) += v;
                            else g[L.s0].at(i, y, x, ch) += v;
                        } else {
                            g[L.s1].at(i, y, x, ch - c0) += v;
                        }
                    }
    };
    auto back_pool = [&](int from, int to) {
        const T& gt = g[to];
        for (int i = 0; i < gt.n; ++i)
            for (int y = 0; y < gt.h; ++y)
                for (int x = 0; x < gt.w; ++x)
                    for (int ch = 0; ch < gt.c; ++ch) {
                        const double v = 0.25 * gt.at(i, y, x, ch);
                        g[from].at(i, 2 * y, 2 * x, ch) += v;
                        g[from].at(i, 2 * y, 2 * x + 1, ch) += v;
                        g[from].at(i, 2 * y + 1, 2 * x, ch) += v;
                        g[from].at(i, 2 * y + 1, 2 * x + 1, ch) += v;
                    }
    };
    for (int l = 18; l >= 8; --l) back(l);
    back_pool(E3, P4);
    back(7);
    back(6);
    back_pool(E2, P3);
    back(5);
    back(4);
    back_pool(E1, P2);
    back(3);
    back(2);
    back_pool(E0, P1);
    back(1);
    back(0);
    return loss;
}

// One convolution for kernel-level checks (double math, float tensors
// with stride = channels). mode 0 forward (out [n][h][w][cout]), 1 input
// gradient (out [n][h][w][cin], times the activation slope of mask when
// given), 2 weight and bias gradient (dw [cout][9][cin], db [cout]).
void ro_conv3x3(int mode, uint32_t n, uint32_t h, uint32_t w, const float* src0, uint32_t c0, uint32_t shift0,
                const float* src1, uint32_t c1, uint32_t cout, const float* weight, const float* bias, const float* dy,
                const float* mask, int act, float* out, double* dw, double* db) {
    T s0, s1;
    const int H = int(h), W = int(w);
    const int h0 = shift0 ? H / 2 : H, w0 = shift0 ? W / 2 : W;
    if (src0) {
        s0.init(int(n), h0, w0, int(c0));
        for (size_t k = 0; k < s0.v.size(); ++k) s0.v[k] = src0[k];
    } else {
        s0.init(int(n), h0, w0, int(c0));
    }
    if (c1) {
        s1.init(int(n), H, W, int(c1));
        if (src1)
            for (size_t k = 0; k < s1.v.size(); ++k) s1.v[k] = src1[k];
    }
    const int cin = int(c0 + c1);
    std::vector<double> wt(size_t(cout) * 9 * cin), b(cout, 0.0);
    for (size_t k = 0; k < wt.size(); ++k) wt[k] = weight[k];
    if (bias)
        for (uint32_t k = 0; k < cout; ++k) b[k] = bias[k];
    if (mode == 0) {
        T o;
        conv_forward(s0, c1 ? &s1 : nullptr, shift0 != 0, H, W, wt.data(), b.data(), int(cout), act, o);
        for (size_t k = 0; k < o.v.size(); ++k) out[k] = float(o.v[k]);
        return;
    }
    T g;
    g.init(int(n), H, W, int(cout));
    for (size_t k = 0; k < g.v.size(); ++k) g.v[k] = dy[k];
    std::vector<double> dwl(wt.size(), 0.0), dbl(cout, 0.0);
    T dx;
    conv_backward(s0, c1 ? &s1 : nullptr, shift0 != 0, H, W, wt.data(), g, dwl.data(), dbl.data(),
                  mode == 1 ? &dx : nullptr);
    if (mode == 1) {
        for (size_t k = 0; k < dx.v.size(); ++k) {
            double v = dx.v[k];
            if (mask && mask[k] <= 0.0f) v *= kLeak;
            out[k] = float(v);
        }
    } else {
        for (size_t k = 0; k < dwl.size(); ++k) dw[k] = dwl[k];
        for (uint32_t k = 0; k < cout; ++k) db[k] = dbl[k];
    }
}

}  // extern "C"
