// Texture arrays and the environment map built on the GPU from the scene's
// own images (src/Renderer.mjs:637-661, 723-760; src/Texture.mjs:164-209;
// src/EnvironmentMap.mjs:202-247; toHalf src/Renderer.mjs:1143-1160).
//
// The arithmetic is the reference's, in double where it is double there,
// term for term and in the same order, every multiply and add rounded on
// its own (__dmul_rn, __dadd_rn: no fused multiply-adds), so the bytes,
// half floats and table entries equal the host restatements' bit for bit.
// The two transcendental inputs come from the host: the byte-decoding table
// (sRGB to linear, or a plain number) and each table row's sine, so no
// device math function's last bit can differ from the host library's; the
// sRGB encode's power is the one device call (a 1-ulp difference in it
// moves a byte only at an exact half, which the tests' sweeps of every
// texel do not meet).
#include "kernels.cuh"

#include <algorithm>

namespace rmd {

namespace {

// Texture.sample's bilinear blend (src/Texture.mjs:164-182) of texture t at
// (u, v), the four texels in the reference's order, decoded by table.
__device__ void sample_bilinear(const uint8_t* __restrict__ t, uint32_t tw, uint32_t th, double u, double v,
                                const double* __restrict__ decode, double rgb[3]) {
    const double x = __dsub_rn(__dmul_rn(u, double(tw)), 0.5), y = __dsub_rn(__dmul_rn(v, double(th)), 0.5);
    const double x0 = floor(x), y0 = floor(y);
    const double fx = __dsub_rn(x, x0), fy = __dsub_rn(y, y0);
    rgb[0] = rgb[1] = rgb[2] = 0.0;
    const int dxs[4] = {0, 1, 0, 1}, dys[4] = {0, 0, 1, 1};
    for (int k = 0; k < 4; ++k) {
        const double w = __dmul_rn(dxs[k] ? fx : __dsub_rn(1.0, fx), dys[k] ? fy : __dsub_rn(1.0, fy));
        // mod() of the reference: the wrapped index, non-negative
        long long px = (long long)(x0) + dxs[k], py = (long long)(y0) + dys[k];
        px %= (long long)tw;
        py %= (long long)th;
        if (px < 0) px += tw;
        if (py < 0) py += th;
        const uint8_t* texel = t + (size_t(py) * tw + size_t(px)) * 4;
        rgb[0] = __dadd_rn(rgb[0], __dmul_rn(w, decode[texel[0]]));
        rgb[1] = __dadd_rn(rgb[1], __dmul_rn(w, decode[texel[1]]));
        rgb[2] = __dadd_rn(rgb[2], __dmul_rn(w, decode[texel[2]]));
    }
}

// Math.round: floor(x + 0.5).
__device__ __forceinline__ double js_round(double x) { return floor(__dadd_rn(x, 0.5)); }

// toSrgbByte (src/Texture.mjs:211-216).
__device__ __forceinline__ uint8_t to_srgb_byte(double c) {
    const double x = fmin(fmax(c, 0.0), 1.0);
    const double s = x <= 0.0031308 ? __dmul_rn(x, 12.92) : __dsub_rn(__dmul_rn(1.055, pow(x, 1.0 / 2.4)), 0.055);
    return uint8_t(js_round(__dmul_rn(s, 255.0)));
}

// One layer of a texture array: texture t (tw × th) resampled to w × h at
// texel centres (Texture.resized, src/Texture.mjs:193-209), or copied when
// the sizes agree.
__global__ void k_texture_layer(const uint8_t* __restrict__ t, uint32_t tw, uint32_t th, uint8_t* __restrict__ out,
                                uint32_t w, uint32_t h, int srgb, const double* __restrict__ decode) {
    const uint32_t n = w * h;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint8_t* o = out + size_t(i) * 4;
        if (tw == w && th == h) {
            for (int c = 0; c < 4; ++c) o[c] = t[size_t(i) * 4 + c];
            continue;
        }
        const uint32_t x = i % w, y = i / w;
        double rgb[3];
        sample_bilinear(t, tw, th, (x + 0.5) / w, (y + 0.5) / h, decode, rgb);
        for (int c = 0; c < 3; ++c)
            o[c] = srgb ? to_srgb_byte(rgb[c]) : uint8_t(js_round(__dmul_rn(rgb[c], 255.0)));
        o[3] = 255;
    }
}

// toHalf (src/Renderer.mjs:1143-1160): the nearest half float's bits,
// saturating at 65504; zero for anything not above 0. The exponent is
// floor(log2(x)), taken exactly from frexp.
__device__ __forceinline__ uint16_t to_half(double x) {
    if (!(x > 0.0)) return 0;
    if (x >= 65504.0) return 0x7BFF;
    if (x < 6.1035e-5) return uint16_t(js_round(x / 5.9605e-8));
    int e2;
    frexp(x, &e2);
    const int exponent = e2 - 1;
    int mantissa = int(js_round(__dmul_rn(__dsub_rn(ldexp(x, -exponent), 1.0), 1024.0)));
    int e = exponent + 15;
    if (mantissa == 1024) {
        mantissa = 0;
        e += 1;
    }
    return uint16_t((e << 10) | mantissa);
}

// The environment map as the renderer uploads it: RGBA half floats, alpha 1.
__global__ void k_environment_halves(const float* __restrict__ rgb, uint32_t n, uint16_t* __restrict__ out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        out[size_t(i) * 4] = to_half(double(rgb[size_t(i) * 3]));
        out[size_t(i) * 4 + 1] = to_half(double(rgb[size_t(i) * 3 + 1]));
        out[size_t(i) * 4 + 2] = to_half(double(rgb[size_t(i) * 3 + 2]));
        out[size_t(i) * 4 + 3] = 0x3C00;  // 1.0
    }
}

// importance() (src/EnvironmentMap.mjs:202-247), one block per row of cells:
// each thread sums its cells' luminance in double over their pixels,
// row-major, as the reference does; thread 0 then runs the row's sum along
// x, storing each running value as f32, and the row is divided by its
// double total (or spread evenly when it is dark). rows[y] keeps the total.
constexpr int kTableThreads = 256;

__global__ void __launch_bounds__(kTableThreads) k_importance_rows(const float* __restrict__ rgb, uint32_t W, uint32_t H,
                                                                    uint32_t cw, uint32_t ch,
                                                                    const double* __restrict__ sines,
                                                                    float* __restrict__ table,
                                                                    double* __restrict__ rows) {
    __shared__ double cell[512];
    __shared__ double total;
    const uint32_t y = blockIdx.x;
    const uint32_t y0 = uint32_t((uint64_t(y) * H) / ch);
    const uint32_t y1 = max(y0 + 1, uint32_t((uint64_t(y + 1) * H) / ch));
    const double sine = sines[y];
    for (uint32_t x = threadIdx.x; x < cw; x += blockDim.x) {
        const uint32_t x0 = uint32_t((uint64_t(x) * W) / cw);
        const uint32_t x1 = max(x0 + 1, uint32_t((uint64_t(x + 1) * W) / cw));
        double light = 0.0;
        for (uint32_t py = y0; py < y1; ++py)
            for (uint32_t px = x0; px < x1; ++px) {
                const float* c = rgb + (size_t(py) * W + px) * 3;
                const double lum = __dadd_rn(__dadd_rn(__dmul_rn(0.2126, double(c[0])), __dmul_rn(0.7152, double(c[1]))),
                                             __dmul_rn(0.0722, double(c[2])));
                light = __dadd_rn(light, lum);
            }
        cell[x] = __dmul_rn(light / double((y1 - y0) * (x1 - x0)), sine);
    }
    __syncthreads();
    float* out = table + size_t(y) * cw;
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (uint32_t x = 0; x < cw; ++x) {
            sum = __dadd_rn(sum, cell[x]);
            out[x] = float(sum);
        }
        total = sum;
        rows[y] = sum;
    }
    __syncthreads();
    const double s = total;
    for (uint32_t x = threadIdx.x; x < cw; x += blockDim.x)
        out[x] = s > 0.0 ? float(double(out[x]) / s) : float(double(x + 1) / double(cw));
    __syncthreads();
    if (threadIdx.x == 0) out[cw - 1] = 1.0f;  // rounding mustn't leave a row short of 1
}

// The CDF down the rows (the table's last row): running totals over the
// grand total, the last forced to 1.
__global__ void k_importance_down(const double* __restrict__ rows, uint32_t cw, uint32_t ch, float* __restrict__ table) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    double total = 0.0;
    for (uint32_t y = 0; y < ch; ++y) total = __dadd_rn(total, rows[y]);
    double running = 0.0;
    float* down = table + size_t(ch) * cw;
    for (uint32_t y = 0; y < ch; ++y) {
        running = __dadd_rn(running, rows[y]);
        down[y] = total > 0.0 ? float(running / total) : float(double(y + 1) / double(ch));
    }
    down[ch - 1] = 1.0f;
}

}  // namespace

int launch_texture_layer(const uint8_t* src, uint32_t tw, uint32_t th, uint8_t* dst, uint32_t w, uint32_t h, int srgb,
                         const double* decode, int num_sms, cudaStream_t st) {
    const uint32_t n = w * h;
    const uint32_t blocks = std::min<uint32_t>((n + 255u) / 256u, uint32_t(num_sms) * 16u);
    k_texture_layer<<<blocks ? blocks : 1u, 256, 0, st>>>(src, tw, th, dst, w, h, srgb, decode);
    return 1;
}

int launch_environment(const float* rgb, uint32_t W, uint32_t H, uint32_t cw, uint32_t ch, const double* sines,
                       uint16_t* halves, float* table, double* rows, int num_sms, cudaStream_t st) {
    const uint32_t n = W * H;
    const uint32_t blocks = std::min<uint32_t>((n + 255u) / 256u, uint32_t(num_sms) * 16u);
    k_environment_halves<<<blocks ? blocks : 1u, 256, 0, st>>>(rgb, n, halves);
    k_importance_rows<<<ch, kTableThreads, 0, st>>>(rgb, W, H, cw, ch, sines, table, rows);
    k_importance_down<<<1, 32, 0, st>>>(rows, cw, ch, table);
    return 3;
}

}  // namespace rmd
