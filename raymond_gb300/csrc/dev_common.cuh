// Device-side basics for the sm_103a render path: the packed scene records,
// the 208-byte uniform block, vector arithmetic and the sample hashes.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace rmd {

constexpr uint32_t NONE = 0xffffffffu;
constexpr float PI = 3.14159265358979f;
constexpr float T_MIN = 1e-4f;
constexpr float INF = 1e30f;

// Primitive kinds and material types (src/shaders.mjs:60-70; src/Scene.mjs:102-107;
// src/Material.mjs:53-60).
constexpr uint32_t SPHERE = 0, QUAD = 1, BOX = 2, TRIANGLE = 3;
constexpr uint32_t DIFFUSE = 0, METAL = 1, PLASTIC = 2, GLASS = 3, LIGHT = 4, VOLUME = 5;
constexpr uint32_t VIEW_COLOR = 0, VIEW_ALBEDO = 1, VIEW_NORMAL = 2, VIEW_DEPTH = 3;

// The uniform block, 13 rows of 16 bytes (src/shaders.mjs:9-24), written on
// the host exactly as Renderer.#writeParams lays it out.
struct Params {
    float cam_pos[3];
    float lens_radius;
    float cam_right[3];
    float tan_half_fov;
    float cam_up[3];
    float focus_distance;
    float cam_forward[3];
    float aspect;
    float sky_zenith[3];
    float sun_omc;
    float sky_horizon[3];
    uint32_t sun_on;
    float sky_ground[3];
    float firefly_clamp;
    float sun_dir[3];
    uint32_t light_count;
    float sun_radiance[3];
    uint32_t max_bounces;
    uint32_t view, volume_count;
    float env_strength, env_rotation;
    uint32_t width, height, sample_offset, samples_per_frame;
    uint32_t total_samples;
    float exposure;
    uint32_t denoise, caustics;
    float photon_radius, photon_cell;
    uint32_t pad5, pad6;
};
static_assert(sizeof(Params) == 208, "Params is 208 bytes");

// Device view of the uploaded scene. Records stay in the reference's packed
// formats; the pointers are float4-typed so each record is 16-byte loads.
struct Scene {
    const float4* prims;       // 4 float4 per primitive: header (as u32), p0, p1, p2
    const float4* nodes;       // 2 float4 per node: min|first, max|count
    const float4* wide;        // 8 float4 per node of the 4-wide traversal tree, or null (bvh_wide.h)
    const float4* materials;   // 6 float4 per material
    const float4* attributes;  // 4 float4 per attribute block
    const uint32_t* lights;    // lights ‖ volumes ‖ CDF bits
    const float4* emitters;    // light tracing's sources and targets
    // Textures: colour (sRGB-decoded on sampling) and normal-map arrays.
    const uchar4* textures;
    const uchar4* normal_maps;
    uint32_t tex_w, tex_h, tex_layers;
    uint32_t nrm_w, nrm_h, nrm_layers;
    // Environment map (half RGBA) and its importance table.
    const ushort4* env_map;
    const float* env_table;
    uint32_t env_w, env_h, env_cw, env_ch;
    uint32_t prim_count;
    uint32_t seed_hash;  // XORed into the sample hashes; 0 keeps the reference streams
};

// ---- float3 arithmetic ----
__host__ __device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__host__ __device__ __forceinline__ float3 f3(float s) { return make_float3(s, s, s); }
__host__ __device__ __forceinline__ float3 f3(const float* p) { return make_float3(p[0], p[1], p[2]); }
__device__ __forceinline__ float3 xyz(float4 v) { return make_float3(v.x, v.y, v.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float3 operator/(float3 a, float3 b) { return f3(a.x / b.x, a.y / b.y, a.z / b.z); }
__device__ __forceinline__ float3& operator+=(float3& a, float3 b) { a = a + b; return a; }
__device__ __forceinline__ float3& operator*=(float3& a, float3 b) { a = a * b; return a; }
__device__ __forceinline__ float3& operator*=(float3& a, float s) { a = a * s; return a; }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross(float3 a, float3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float length(float3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ float3 normalize(float3 a) { return a / sqrtf(dot(a, a)); }
__device__ __forceinline__ float3 fmin3(float3 a, float3 b) { return f3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
__device__ __forceinline__ float3 fmax3(float3 a, float3 b) { return f3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
__device__ __forceinline__ float maxc(float3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float signf(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
__device__ __forceinline__ float3 mix3(float3 a, float3 b, float t) { return a * (1.0f - t) + b * t; }
// 1 − x·x with the square rounded on its own, as the reference's shader
// arithmetic has it. Where x is near 1 (a small cone's cos, a pole's z) the
// subtraction cancels, and a fused multiply-add would round that result
// differently by up to 1e-4 relative; the sample directions follow it.
__device__ __forceinline__ float one_minus_sq(float x) { return 1.0f - __fmul_rn(x, x); }
__device__ __forceinline__ float3 reflect3(float3 i, float3 n) { return i - n * (2.0f * dot(n, i)); }
// WGSL refract(e1, e2, e3): the zero vector under total internal reflection.
__device__ __forceinline__ float3 refract3(float3 i, float3 n, float eta) {
    const float ni = dot(n, i);
    const float k = 1.0f - __fmul_rn(__fmul_rn(eta, eta), one_minus_sq(ni));
    if (k < 0.0f) return f3(0.0f);
    return i * eta - n * (eta * ni + sqrtf(k));
}
__device__ __forceinline__ float luminance(float3 c) { return dot(c, f3(0.2126f, 0.7152f, 0.0722f)); }
// finite() of src/shaders.mjs:1833-1836: no component has an all-ones exponent.
__device__ __forceinline__ bool finite3(float3 v) {
    return ((__float_as_uint(v.x) & 0x7f800000u) != 0x7f800000u) &&
           ((__float_as_uint(v.y) & 0x7f800000u) != 0x7f800000u) &&
           ((__float_as_uint(v.z) & 0x7f800000u) != 0x7f800000u);
}
__device__ __forceinline__ bool finite1(float v) { return (__float_as_uint(v) & 0x7f800000u) != 0x7f800000u; }

// ---- sample hashes (bit-exact with src/shaders.mjs:135-212) ----
// The PCG output permutation used as a hash (Jarzynski & Olano, 2020).
__host__ __device__ __forceinline__ uint32_t pcg(uint32_t v) {
    const uint32_t state = v * 747796405u + 2891336453u;
    const uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
__device__ __forceinline__ float unit_f(uint32_t x) { return float(x >> 8u) * (1.0f / 16777216.0f); }
// Hash-based Owen scrambling (Burley, 2020): the Laine–Karras hash on reversed bits.
__device__ __forceinline__ uint32_t owen(uint32_t x, uint32_t seed) {
    uint32_t v = __brev(x);
    v ^= v * 0x3d20adeau;
    v += seed;
    v *= (seed >> 16u) | 1u;
    v ^= v * 0x05526c56u;
    v ^= v * 0x53a22864u;
    return __brev(v);
}
// Sobol's second dimension by its direction-number recurrence.
__device__ __forceinline__ uint32_t sobol2(uint32_t i) {
    uint32_t r = 0u, v = 0x80000000u;
    while (i != 0u) {
        if (i & 1u) r ^= v;
        i >>= 1u;
        v ^= v >> 1u;
    }
    return r;
}

// A path's random numbers: scrambled Sobol per dimension when qmc is on
// (camera paths), a PCG chain otherwise (photons, photon gather).
struct Rng {
    uint32_t state;  // PCG chain
    uint32_t seed;   // the pixel's scramble key
    uint32_t index;  // which sample of the pixel
    uint32_t dim;    // next dimension
    bool qmc;

    __device__ __forceinline__ float rand() {
        if (qmc) {
            const uint32_t key = pcg(seed ^ pcg(dim));
            dim++;
            const uint32_t y = owen(index, key);
            return unit_f(owen(__brev(y), pcg(key)));
        }
        state = pcg(state);
        return unit_f(state);
    }
    __device__ __forceinline__ float2 rand2() {
        if (qmc) {
            const uint32_t key = pcg(seed ^ pcg(dim));
            dim++;
            const uint32_t y = owen(index, key);
            return make_float2(unit_f(owen(__brev(y), pcg(key))), unit_f(owen(sobol2(y), pcg(key + 1u))));
        }
        const float a = rand();
        return make_float2(a, rand());
    }
};

// The streams' seeds. A camera path: pixel `index`, sample `sample` (main(),
// src/shaders.mjs:1852-1859), scrambled Sobol from dimension 0, with its
// golden-ratio spectrum position. A light path `id` of the frame starting at
// sample_offset (light_trace(), :1638) and a pixel's photon gather (:1585):
// PCG chains. seed_hash is 0 for the reference's streams.
__device__ __forceinline__ Rng camera_rng(uint32_t index, uint32_t sample, uint32_t seed_hash) {
    Rng r;
    r.state = pcg(index ^ pcg(sample)) ^ seed_hash;
    r.qmc = true;
    r.seed = pcg(index + 0x9e3779b9u) ^ seed_hash;
    r.index = sample;
    r.dim = 0u;
    return r;
}
__device__ __forceinline__ float spectrum_position(uint32_t index, uint32_t sample) {
    return float((pcg(index * 7919u + 1u) + sample * 2654435769u) >> 8u) * (1.0f / 16777216.0f);
}
__device__ __forceinline__ Rng light_rng(uint32_t id, uint32_t sample_offset, uint32_t seed_hash) {
    Rng r{};
    r.qmc = false;
    r.state = pcg(id ^ pcg(sample_offset * 2654435769u + 977u)) ^ seed_hash;
    return r;
}
__device__ __forceinline__ Rng gather_rng(uint32_t index, uint32_t sample_offset, uint32_t seed_hash) {
    Rng r{};
    r.qmc = false;
    r.state = pcg(index ^ pcg(sample_offset * 2654435769u + 4099u)) ^ seed_hash;
    return r;
}

// ---- sampling (src/shaders.mjs:217-256) ----
// Orthonormal basis whose third axis is n (Duff et al., 2017); returns the
// world vector for local coordinates l.
__device__ __forceinline__ float3 from_frame(float3 n, float3 l) {
    const float s = n.z >= 0.0f ? 1.0f : -1.0f;
    const float a = -1.0f / (s + n.z);
    const float b = n.x * n.y * a;
    const float3 c0 = f3(1.0f + s * n.x * n.x * a, s * b, -s * n.x);
    const float3 c1 = f3(b, s + n.y * n.y * a, -n.y);
    return c0 * l.x + c1 * l.y + n * l.z;
}
__device__ __forceinline__ void frame_axes(float3 n, float3& c0, float3& c1) {
    const float s = n.z >= 0.0f ? 1.0f : -1.0f;
    const float a = -1.0f / (s + n.z);
    const float b = n.x * n.y * a;
    c0 = f3(1.0f + s * n.x * n.x * a, s * b, -s * n.x);
    c1 = f3(b, s + n.y * n.y * a, -n.y);
}
__device__ __forceinline__ float3 cosine_hemisphere(float3 n, Rng& rng) {
    const float2 u = rng.rand2();
    const float r = sqrtf(u.x);
    const float phi = 2.0f * PI * u.y;
    float s, c;
    sincosf(phi, &s, &c);
    return normalize(from_frame(n, f3(r * c, r * s, sqrtf(fmaxf(0.0f, one_minus_sq(r))))));
}
__device__ __forceinline__ float3 sample_cone(float3 axis, float omc, Rng& rng) {
    const float2 u = rng.rand2();
    const float cos_t = 1.0f - u.x * omc;
    const float sin_t = sqrtf(fmaxf(0.0f, one_minus_sq(cos_t)));
    const float phi = 2.0f * PI * u.y;
    float s, c;
    sincosf(phi, &s, &c);
    return normalize(from_frame(axis, f3(sin_t * c, sin_t * s, cos_t)));
}
// Shirley–Chiu concentric square-to-disk map.
__device__ __forceinline__ float2 concentric_disk(Rng& rng) {
    const float2 r = rng.rand2();
    const float ux = 2.0f * r.x - 1.0f, uy = 2.0f * r.y - 1.0f;
    if (ux == 0.0f && uy == 0.0f) return make_float2(0.0f, 0.0f);
    float s, c;
    if (fabsf(ux) > fabsf(uy)) {
        sincosf((PI / 4.0f) * (uy / ux), &s, &c);
        return make_float2(ux * c, ux * s);
    }
    sincosf(PI / 2.0f - (PI / 4.0f) * (ux / uy), &s, &c);
    return make_float2(uy * c, uy * s);
}

}  // namespace rmd
