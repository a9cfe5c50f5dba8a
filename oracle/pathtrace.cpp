// The trace shader's path tracer (src/shaders.mjs:131-1899), its light
// tracing with splats and its photon map (src/shaders.mjs:1425-1831), the
// denoiser (src/shaders.mjs:1916-2098) and the display math
// (src/shaders.mjs:2114-2152), restated as scalar f32 C++ on the CPU — TEST
// INFRASTRUCTURE ONLY. The integer sample hashes are bit-exact; the f32
// arithmetic follows the WGSL expression by expression (compiled without
// contraction), with
// the math library's sqrt/sin/cos/exp/log/pow/atan2/acos called, never
// re-implemented. Environment maps, textures and normal maps are read as
// the renderer uploads them (ro_render_scene).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "oracle.h"

namespace {

const float PI = 3.14159265358979f;
const uint32_t NONE = 0xffffffffu;
const float INF = 1e30f;

struct V {
    float x, y, z;
};
inline V v3(float x, float y, float z) { return {x, y, z}; }
inline V vs(float s) { return {s, s, s}; }
inline V vf(const float* p) { return {p[0], p[1], p[2]}; }
inline V operator+(V a, V b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V operator-(V a, V b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V operator-(V a) { return {-a.x, -a.y, -a.z}; }
inline V operator*(V a, V b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V operator*(V a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V operator/(V a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline float dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V cross(V a, V b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float len(V a) { return std::sqrt(dot(a, a)); }
inline V norm(V a) { return a / std::sqrt(dot(a, a)); }
inline float wmin(float a, float b) { return b < a ? b : a; }  // WGSL min(e1, e2)
inline float wmax(float a, float b) { return b > a ? b : a; }
inline float clampf(float x, float lo, float hi) { return wmin(wmax(x, lo), hi); }
inline float sgn(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
inline uint32_t fbits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
inline float bitsf(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
inline bool finite3(V v) {
    return (fbits(v.x) & 0x7f800000u) != 0x7f800000u && (fbits(v.y) & 0x7f800000u) != 0x7f800000u &&
           (fbits(v.z) & 0x7f800000u) != 0x7f800000u;
}
inline float lum(V c) { return dot(c, v3(0.2126f, 0.7152f, 0.0722f)); }

// ---- uniform block (src/shaders.mjs:9-24) ----
struct Params {
    float cam_pos[3], lens_radius, cam_right[3], tan_half_fov, cam_up[3], focus_distance, cam_forward[3], aspect;
    float sky_zenith[3], sun_omc, sky_horizon[3];
    uint32_t sun_on;
    float sky_ground[3], firefly_clamp, sun_dir[3];
    uint32_t light_count;
    float sun_radiance[3];
    uint32_t max_bounces, view, volume_count;
    float env_strength, env_rotation;
    uint32_t width, height, sample_offset, samples_per_frame, total_samples;
    float exposure;
    uint32_t denoise, caustics;
    float photon_radius, photon_cell;
    uint32_t pad5, pad6;
};
static_assert(sizeof(Params) == 208, "208-byte uniforms");

// ---- sample hashes (src/shaders.mjs:135-212) ----
inline uint32_t pcg(uint32_t v) {
    const uint32_t state = v * 747796405u + 2891336453u;
    const uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
inline float unit(uint32_t x) { return float(x >> 8u) * (1.0f / 16777216.0f); }
inline uint32_t reverse_bits(uint32_t x) {
    uint32_t r = 0;
    for (int i = 0; i < 32; ++i) {
        r = (r << 1) | (x & 1u);
        x >>= 1;
    }
    return r;
}
inline uint32_t owen(uint32_t x, uint32_t seed) {
    uint32_t v = reverse_bits(x);
    v ^= v * 0x3d20adeau;
    v += seed;
    v *= (seed >> 16u) | 1u;
    v ^= v * 0x05526c56u;
    v ^= v * 0x53a22864u;
    return reverse_bits(v);
}
inline uint32_t sobol2(uint32_t i) {
    uint32_t r = 0u, v = 0x80000000u, j = i;
    while (j != 0u) {
        if ((j & 1u) != 0u) r ^= v;
        j >>= 1u;
        v ^= v >> 1u;
    }
    return r;
}

struct Sampler {
    uint32_t rng_state = 0;
    bool qmc_on = false;
    uint32_t qmc_seed = 0, qmc_index = 0, qmc_dim = 0;

    void qmc_next(uint32_t& key, uint32_t& idx) {
        key = pcg(qmc_seed ^ pcg(qmc_dim));
        qmc_dim++;
        idx = owen(qmc_index, key);
    }
    float rand() {
        if (qmc_on) {
            uint32_t k, y;
            qmc_next(k, y);
            return unit(owen(reverse_bits(y), pcg(k)));
        }
        rng_state = pcg(rng_state);
        return unit(rng_state);
    }
    void rand2(float& a, float& b) {
        if (qmc_on) {
            uint32_t k, y;
            qmc_next(k, y);
            a = unit(owen(reverse_bits(y), pcg(k)));
            b = unit(owen(sobol2(y), pcg(k + 1u)));
            return;
        }
        a = rand();
        b = rand();
    }
};

// The streams' seeds: main()'s per sample (src/shaders.mjs:1852-1859),
// light_trace()'s per photon (:1638), photon_gather()'s per pixel (:1585).
Sampler camera_sampler(uint32_t index, uint32_t sample, uint32_t seed_hash) {
    Sampler sm;
    sm.rng_state = pcg(index ^ pcg(sample)) ^ seed_hash;
    sm.qmc_on = true;
    sm.qmc_seed = pcg(index + 0x9e3779b9u) ^ seed_hash;
    sm.qmc_index = sample;
    sm.qmc_dim = 0u;
    return sm;
}
float spectrum_at(uint32_t index, uint32_t sample) {
    return float((pcg(index * 7919u + 1u) + sample * 2654435769u) >> 8u) * (1.0f / 16777216.0f);
}
Sampler light_sampler(uint32_t id, uint32_t sample_offset, uint32_t seed_hash) {
    Sampler sm;
    sm.rng_state = pcg(id ^ pcg(sample_offset * 2654435769u + 977u)) ^ seed_hash;
    return sm;
}
Sampler gather_sampler(uint32_t index, uint32_t sample_offset, uint32_t seed_hash) {
    Sampler sm;
    sm.rng_state = pcg(index ^ pcg(sample_offset * 2654435769u + 4099u)) ^ seed_hash;
    return sm;
}

// frame (src/shaders.mjs:217-225): columns c0, c1, n.
inline V in_frame(V n, V l) {
    const float s = n.z >= 0.0f ? 1.0f : -1.0f;
    const float a = -1.0f / (s + n.z);
    const float b = n.x * n.y * a;
    const V c0 = v3(1.0f + s * n.x * n.x * a, s * b, -s * n.x);
    const V c1 = v3(b, s + n.y * n.y * a, -n.y);
    return c0 * l.x + c1 * l.y + n * l.z;
}

// An environment map as the renderer uploads it: RGBA half floats and the
// importance table (cw × (ch + 1) floats).
struct Env {
    const uint16_t* map;
    uint32_t w, h;
    const float* table;
    uint32_t cw, ch;
};

// A texture array as the renderer uploads it: layers of w × h RGBA bytes.
struct Tex {
    const uint8_t* data;
    uint32_t w, h;
};

struct Ctx {
    const uint8_t* prims;
    const uint8_t* nodes;
    const float* mats;
    const float* attrs;
    const uint32_t* lights;
    Params P;
    // counters: all algorithmic bytes, rays, surface hits; traversal bytes
    // and rays of closest-hit and of shadow (any-hit) traces apart
    uint64_t bytes = 0, rays = 0, hits = 0;
    uint64_t trav_closest = 0, trav_shadow = 0, rays_closest = 0, rays_shadow = 0;
    const Env* env = nullptr;
    const Tex* textures = nullptr;     // colour and emission textures (sRGB)
    const Tex* normal_maps = nullptr;  // normal maps (plain numbers)

    const float* pf(uint32_t i) const { return reinterpret_cast<const float*>(prims + size_t(i) * 64); }
    const uint32_t* pu(uint32_t i) const { return reinterpret_cast<const uint32_t*>(prims + size_t(i) * 64); }
    const float* mf(uint32_t i) const { return mats + size_t(i) * 24; }
    uint32_t mu(uint32_t i, int k) const { return fbits(mats[size_t(i) * 24 + k]); }
};

struct HitR {
    float t;
    uint32_t prim;
    float u, v;
};

// Perturbation runs, for classifying disagreements with the GPU (off unless
// ro_set_jitter set a size): every traced ray's origin and direction
// components are scaled by 1 ± size, the signs a hash of the ray's own bits
// and the run's seed, and an odd seed flipping them all, so a pair of runs
// (2k, 2k+1) nudges each ray both ways. Results that change under such runs
// hang on a decision within rounding of its threshold (an edge, a pixel
// boundary, a lobe or roulette choice), where f32 arithmetic that rounds
// differently may legitimately take the other branch.
float g_jitter_size = 0.0f;
uint32_t g_jitter_seed = 0u;

void nudge(V& o, V& d) {
    uint32_t h = pcg(g_jitter_seed >> 1u ^ pcg(fbits(o.x) ^ pcg(fbits(o.y) ^ pcg(fbits(o.z) ^ pcg(fbits(d.x) ^
                     pcg(fbits(d.y) ^ pcg(fbits(d.z))))))));
    const float s = (g_jitter_seed & 1u) ? -g_jitter_size : g_jitter_size;
    float* f[6] = {&o.x, &o.y, &o.z, &d.x, &d.y, &d.z};
    for (int k = 0; k < 6; ++k) *f[k] *= 1.0f + (((h >> k) & 1u) ? s : -s);
}

HitR trace(Ctx& c, V o, V d, float t_max, bool any_hit) {
    if (g_jitter_size != 0.0f) nudge(o, d);
    const float of[3] = {o.x, o.y, o.z}, df[3] = {d.x, d.y, d.z};
    uint32_t prim, inner, tested;
    float tuv[3];
    ro_trace32_one(c.prims, c.nodes, of, df, t_max, any_hit ? 1 : 0, &prim, tuv, &inner, &tested);
    c.rays++;
    const uint64_t tb = 32ull * (1 + 2ull * inner) + 64ull * tested;
    c.bytes += tb;
    if (any_hit) {
        c.trav_shadow += tb;
        c.rays_shadow++;
    } else {
        c.trav_closest += tb;
        c.rays_closest++;
    }
    return {tuv[0], prim, tuv[1], tuv[2]};
}

struct Surf {
    V p, n, ng;
    bool front;
    uint32_t material, light, kind;
    float u, v;
};

// sphere_uv (src/shaders.mjs:573-577).
void sphere_uv(V n, const float* p, float& u, float& v) {
    const V x = vf(p + 8), north = vf(p + 12);
    const V z = cross(x, north);
    const float uu = std::atan2(-dot(n, z), dot(n, x)) / (2.0f * PI);
    u = uu - std::floor(uu);
    v = std::acos(clampf(dot(n, north), -1.0f, 1.0f)) / PI;
}

// ---- textures: bilinear with repeat, as the reference's sampler does ----
float srgb_to_linear(uint8_t b) {
    static const struct Table {
        float v[256];
        Table() {
            for (int i = 0; i < 256; ++i) {
                const double x = i / 255.0;
                v[i] = float(x <= 0.04045 ? x / 12.92 : std::pow((x + 0.055) / 1.055, 2.4));
            }
        }
    } table;
    return table.v[b];
}
V texel(const Tex& t, uint32_t layer, int x, int y, bool srgb) {
    const int xi = ((x % int(t.w)) + int(t.w)) % int(t.w);
    const int yi = ((y % int(t.h)) + int(t.h)) % int(t.h);
    const uint8_t* q = t.data + ((size_t(layer) * t.h + yi) * t.w + xi) * 4;
    if (srgb) return v3(srgb_to_linear(q[0]), srgb_to_linear(q[1]), srgb_to_linear(q[2]));
    return v3(q[0] / 255.0f, q[1] / 255.0f, q[2] / 255.0f);
}
V sample_texture(const Tex& t, uint32_t layer, float u, float v, bool srgb) {
    const float x = u * float(t.w) - 0.5f, y = v * float(t.h) - 0.5f;
    const float fx0 = std::floor(x), fy0 = std::floor(y);
    const float fx = x - fx0, fy = y - fy0;
    const int x0 = int(fx0), y0 = int(fy0);
    return texel(t, layer, x0, y0, srgb) * ((1.0f - fx) * (1.0f - fy)) +
           texel(t, layer, x0 + 1, y0, srgb) * (fx * (1.0f - fy)) +
           texel(t, layer, x0, y0 + 1, srgb) * ((1.0f - fx) * fy) +
           texel(t, layer, x0 + 1, y0 + 1, srgb) * (fx * fy);
}

// bump (src/shaders.mjs:582-594): n tilted by a normal-map texel.
V bump(V n, V ng, V tangent, V up, V t, float strength) {
    V right = tangent - n * dot(n, tangent);
    if (len(right) < 1e-9f) return n;
    right = norm(right);
    V above = cross(n, right);
    if (dot(above, up) < 0.0f) above = -above;
    const V tilted =
        norm(right * ((t.x * 2.0f - 1.0f) * strength) + above * ((t.y * 2.0f - 1.0f) * strength) + n * (t.z * 2.0f - 1.0f));
    return dot(tilted, ng) > 0.0f ? tilted : n;
}

// surface (src/shaders.mjs:460-569), with the texture's tangent frame and
// normal maps.
Surf surface(Ctx& c, V o, V d, const HitR& hit) {
    const float* p = c.pf(hit.prim);
    const uint32_t* pu = c.pu(hit.prim);
    const V point = o + d * hit.t;
    V ng, ns, tangent = vs(0.0f), up = vs(0.0f);
    float u = 0, v = 0;
    c.hits++;
    c.bytes += 64 + 96;  // the primitive record and its material
    switch (pu[0]) {
        case 0:
            ng = norm(point - vf(p + 4));
            ns = ng;
            sphere_uv(ng, p, u, v);
            tangent = cross(vf(p + 12), ng);
            if (len(tangent) < 1e-6f) tangent = vf(p + 8);
            up = cross(ng, tangent);
            break;
        case 1:
            ng = norm(cross(vf(p + 8), vf(p + 12)));
            ns = ng;
            u = hit.u;
            v = 1.0f - hit.v;
            tangent = vf(p + 8);
            up = vf(p + 12);
            break;
        case 2: {
            const V r0 = vf(p + 4), r1 = vf(p + 8), r2 = vf(p + 12);
            const V lp = v3(dot(r0, point) + p[7], dot(r1, point) + p[11], dot(r2, point) + p[15]);
            const V a = v3(std::fabs(lp.x), std::fabs(lp.y), std::fabs(lp.z));
            const V half = v3(1.0f / len(r0), 1.0f / len(r1), 1.0f / len(r2));
            if (a.x >= a.y && a.x >= a.z) {
                ng = r0 * sgn(lp.x);
                u = (1.0f - sgn(lp.x) * lp.z) * half.z;
                v = (1.0f - lp.y) * half.y;
                tangent = r2 * -sgn(lp.x);
                up = r1;
            } else if (a.y >= a.z) {
                ng = r1 * sgn(lp.y);
                u = (1.0f + lp.x) * half.x;
                v = (1.0f + sgn(lp.y) * lp.z) * half.z;
                tangent = r0;
                up = r2 * -sgn(lp.y);
            } else {
                ng = r2 * sgn(lp.z);
                u = (1.0f + sgn(lp.z) * lp.x) * half.x;
                v = (1.0f - lp.y) * half.y;
                tangent = r0 * sgn(lp.z);
                up = r1;
            }
            ng = norm(ng);
            ns = ng;
            break;
        }
        default: {
            const V e1 = vf(p + 8) - vf(p + 4), e2 = vf(p + 12) - vf(p + 4);
            ng = norm(cross(e1, e2));
            ns = ng;
            u = hit.u;
            v = hit.v;
            float du1x = 1.0f, du1y = 0.0f, du2x = 0.0f, du2y = 1.0f;
            if (pu[3] != NONE) {
                c.bytes += 64;  // the attribute block
                const float* A = c.attrs + size_t(pu[3]) * 4;
                const float w = 1.0f - hit.u - hit.v;
                const uint32_t flags = uint32_t(A[15]);
                if (flags & 1u) {
                    ns = norm(vf(A) * w + vf(A + 4) * hit.u + vf(A + 8) * hit.v);
                    if (dot(ns, ng) < 0.0f) ns = -ns;
                }
                if (flags & 2u) {
                    u = A[3] * w + A[7] * hit.u + A[11] * hit.v;
                    v = A[12] * w + A[13] * hit.u + A[14] * hit.v;
                    const float t1x = A[7] - A[3], t1y = A[13] - A[12];
                    const float t2x = A[11] - A[3], t2y = A[14] - A[12];
                    if (std::fabs(t1x * t2y - t2x * t1y) > 1e-12f) {
                        du1x = t1x;
                        du1y = t1y;
                        du2x = t2x;
                        du2y = t2y;
                    }
                }
            }
            // How the position changes with u and v.
            const float det = du1x * du2y - du2x * du1y;
            tangent = (e1 * du2y - e2 * du1y) / det;
            up = -((e2 * du1x - e1 * du2x) / det);
        }
    }
    const float* mm = c.mf(pu[1]);
    const uint32_t nm = fbits(mm[16]);
    if (c.normal_maps && nm != NONE) {
        const V t = sample_texture(*c.normal_maps, nm, u * mm[14], v * mm[15], false);
        ns = bump(ns, ng, tangent, up, t, mm[17]);
    }
    const bool front = dot(ng, d) < 0.0f;
    const float flip = front ? 1.0f : -1.0f;
    return {point, ns * flip, ng * flip, front, pu[1], pu[2], pu[0], u, v};
}

V offset(const Surf& s, V wi) {
    const float eps = 1e-4f * wmax(1.0f, wmax(std::fabs(s.p.x), wmax(std::fabs(s.p.y), std::fabs(s.p.z))));
    return s.p + s.ng * (dot(wi, s.ng) > 0.0f ? eps : -eps);
}

V sky(const Params& P, V d) {
    const V hz = vf(P.sky_horizon), zn = vf(P.sky_zenith), gr = vf(P.sky_ground);
    if (d.y >= 0.0f) {
        const float t = std::sqrt(wmin(d.y, 1.0f));
        return hz * (1.0f - t) + zn * t;
    }
    const float t = std::sqrt(wmin(-d.y, 1.0f));
    return hz * (1.0f - t) + gr * t;
}
bool in_sun(const Params& P, V d) { return P.sun_on != 0u && dot(d, vf(P.sun_dir)) >= 1.0f - P.sun_omc; }

// ---- environment map (src/shaders.mjs:611-676) ----
// IEEE 754 binary16 to binary32, from the format's definition.
inline float half_to_float(uint16_t h) {
    const uint32_t sign = uint32_t(h >> 15) << 31, exp = (h >> 10) & 0x1fu, man = h & 0x3ffu;
    if (exp == 0u) {
        const float v = std::ldexp(float(man), -24);
        return sign ? -v : v;
    }
    if (exp == 31u) return bitsf(sign | 0x7f800000u | (man << 13));
    return bitsf(sign | ((exp + 112u) << 23) | (man << 13));
}
inline bool env_on(const Ctx& c) { return c.env != nullptr && c.P.env_strength > 0.0f; }
void env_uv(const Params& P, V d, float& u, float& v) {
    const float uu = 0.5f + std::atan2(d.x, -d.z) / (2.0f * PI) - P.env_rotation / (2.0f * PI);
    u = uu - std::floor(uu);
    v = std::acos(clampf(d.y, -1.0f, 1.0f)) / PI;
}
// Bilinear, repeating round the horizon and clamped at the poles (the
// reference's sampler: repeat in u, clamp-to-edge in v).
V env_texel(const Env& e, int x, int y) {
    const int w = int(e.w), h = int(e.h);
    const int xi = ((x % w) + w) % w;
    const int yi = y < 0 ? 0 : (y >= h ? h - 1 : y);
    const uint16_t* t = e.map + (size_t(yi) * w + xi) * 4;
    return v3(half_to_float(t[0]), half_to_float(t[1]), half_to_float(t[2]));
}
V env_radiance(const Ctx& c, V d) {
    const Env& e = *c.env;
    float u, v;
    env_uv(c.P, d, u, v);
    const float x = u * float(e.w) - 0.5f, y = v * float(e.h) - 0.5f;
    const float fx0 = std::floor(x), fy0 = std::floor(y);
    const float fx = x - fx0, fy = y - fy0;
    const int x0 = int(fx0), y0 = int(fy0);
    const V col = env_texel(e, x0, y0) * ((1.0f - fx) * (1.0f - fy)) + env_texel(e, x0 + 1, y0) * (fx * (1.0f - fy)) +
                  env_texel(e, x0, y0 + 1) * ((1.0f - fx) * fy) + env_texel(e, x0 + 1, y0 + 1) * (fx * fy);
    return col * c.P.env_strength;
}
inline float env_cdf(const Env& e, uint32_t x, uint32_t y) { return e.table[size_t(y) * e.cw + x]; }
uint32_t env_search(const Env& e, uint32_t y, uint32_t n, float xi) {
    uint32_t lo = 0u, hi = n - 1u;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) / 2u;
        if (env_cdf(e, mid, y) > xi) hi = mid;
        else lo = mid + 1u;
    }
    return lo;
}
float env_pdf(const Ctx& c, V d) {
    const Env& e = *c.env;
    const uint32_t cw = e.cw, ch = e.ch;
    float u, v;
    env_uv(c.P, d, u, v);
    const uint32_t x = std::min(uint32_t(u * float(cw)), cw - 1u);
    const uint32_t y = std::min(uint32_t(v * float(ch)), ch - 1u);
    const float row = env_cdf(e, y, ch) - (y > 0u ? env_cdf(e, y - 1u, ch) : 0.0f);
    const float cell = env_cdf(e, x, y) - (x > 0u ? env_cdf(e, x - 1u, y) : 0.0f);
    const float sn = std::sin(v * PI);
    return sn > 0.0f ? row * cell * float(cw * ch) / (2.0f * PI * PI * sn) : 0.0f;
}
V sample_env(const Ctx& c, Sampler& s) {
    const Env& e = *c.env;
    const uint32_t cw = e.cw, ch = e.ch;
    float cx, cy;
    s.rand2(cx, cy);
    const uint32_t y = env_search(e, ch, ch, cy);
    const uint32_t x = env_search(e, y, cw, cx);
    float wx, wy;
    s.rand2(wx, wy);
    const float u = (float(x) + wx) / float(cw) + c.P.env_rotation / (2.0f * PI);
    const float v = (float(y) + wy) / float(ch);
    const float phi = (u - 0.5f) * 2.0f * PI;
    const float theta = v * PI;
    return v3(std::sin(theta) * std::sin(phi), std::cos(theta), -std::sin(theta) * std::cos(phi));
}
// sky (src/shaders.mjs:678-686): the environment map when there is one.
V sky_at(const Ctx& c, V d) { return env_on(c) ? env_radiance(c, d) : sky(c.P, d); }

// ---- materials (src/shaders.mjs:693-871) ----
struct Mat {
    V color;
    uint32_t kind;
    V emission;
    float roughness;
    V checker;
    float checker_size, ior, dispersion, density, anisotropy;
    uint32_t texture, emission_texture;
    float scale_u, scale_v;
};
Mat material(const Ctx& c, uint32_t i) {
    const float* m = c.mf(i);
    return {vf(m),  c.mu(i, 3), vf(m + 4),   m[7],        vf(m + 8), m[11], m[12],
            m[19], m[20],      m[21], c.mu(i, 13), c.mu(i, 18), m[14], m[15]};
}
V albedo(const Mat& m, V p) {
    V col = m.color;
    if (m.checker_size > 0.0f) {
        const float cx = std::floor(p.x / m.checker_size + 1e-3f), cy = std::floor(p.y / m.checker_size + 1e-3f),
                    cz = std::floor(p.z / m.checker_size + 1e-3f);
        const int odd = (int(cx) + int(cy) + int(cz)) & 1;
        col = odd != 0 ? m.checker : m.color;
    }
    return col;
}
bool is_delta(const Mat& m) { return m.kind == 3 || (m.kind == 1 && m.roughness < 0.01f); }
// albedo and emitted (src/shaders.mjs:693-712) at texture coordinate (u, v).
V albedo_uv(const Ctx& c, const Mat& m, V p, float u, float v) {
    const V col = albedo(m, p);
    if (!c.textures || m.texture == NONE) return col;
    return col * sample_texture(*c.textures, m.texture, u * m.scale_u, v * m.scale_v, true);
}
V emitted(const Ctx& c, const Mat& m, float u, float v) {
    if (!c.textures || m.emission_texture == NONE) return m.emission;
    return m.emission * sample_texture(*c.textures, m.emission_texture, u * m.scale_u, v * m.scale_v, true);
}
float ggx_alpha2(float r) {
    const float a = wmax(r * r, 0.002f);
    return a * a;
}
float ggx_d(float nh, float a2) {
    const float k = nh * nh * (a2 - 1.0f) + 1.0f;
    return a2 / (PI * k * k);
}
float smith_g1(float nv, float a2) { return 2.0f * nv / (nv + std::sqrt(a2 + (1.0f - a2) * nv * nv)); }
float schlick_s(float f0, float c) { return f0 + (1.0f - f0) * std::pow(1.0f - clampf(c, 0.0f, 1.0f), 5.0f); }
V schlick_v(V f0, float c) {
    const float k = std::pow(1.0f - clampf(c, 0.0f, 1.0f), 5.0f);
    return f0 + (vs(1.0f) - f0) * k;
}
float dielectric_f0(float ior) {
    const float r = (ior - 1.0f) / (ior + 1.0f);
    return r * r;
}
float fresnel(float cos_i, float eta) {
    const float sin2_t = (1.0f - cos_i * cos_i) / (eta * eta);
    if (sin2_t >= 1.0f) return 1.0f;
    const float cos_t = std::sqrt(1.0f - sin2_t);
    const float rs = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
    const float rp = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
    return 0.5f * (rs * rs + rp * rp);
}
float spec_chance(const Mat& m, float nv) { return clampf(schlick_s(dielectric_f0(m.ior), nv) * 4.0f + 0.1f, 0.1f, 0.9f); }

void eval_bsdf(const Mat& m, V base, V n, V wo, V wi, V& f, float& pdf) {
    const float nl = dot(n, wi), nv = dot(n, wo);
    f = vs(0.0f);
    pdf = 0.0f;
    if (nl <= 0.0f || nv <= 0.0f) return;
    if (m.kind == 0) {
        f = base * (nl / PI);
        pdf = nl / PI;
        return;
    }
    const float a2 = ggx_alpha2(m.roughness);
    const V h = norm(wo + wi);
    const float nh = wmax(dot(n, h), 0.0f), vh = wmax(dot(wo, h), 1e-6f);
    const float d = ggx_d(nh, a2);
    const float g = smith_g1(nv, a2) * smith_g1(nl, a2);
    const float spec_pdf = d * nh / (4.0f * vh);
    if (m.kind == 1) {
        f = schlick_v(base, vh) * (d * g / (4.0f * nv));
        pdf = spec_pdf;
        return;
    }
    const float f0 = dielectric_f0(m.ior);
    const float coat = schlick_s(f0, vh) * d * g / (4.0f * nv);
    const float through = (1.0f - schlick_s(f0, nl)) * (1.0f - schlick_s(f0, nv));
    const V diffuse = base * (through * nl / PI);
    const float chance = spec_chance(m, nv);
    f = vs(coat) + diffuse;
    pdf = chance * spec_pdf + (1.0f - chance) * nl / PI;
}

V cosine_hemisphere(V n, Sampler& s) {
    float a, b;
    s.rand2(a, b);
    const float r = std::sqrt(a), phi = 2.0f * PI * b;
    return norm(in_frame(n, v3(r * std::cos(phi), r * std::sin(phi), std::sqrt(wmax(0.0f, 1.0f - r * r)))));
}
V sample_cone(V axis, float omc, Sampler& s) {
    float a, b;
    s.rand2(a, b);
    const float cos_t = 1.0f - a * omc;
    const float sin_t = std::sqrt(wmax(0.0f, 1.0f - cos_t * cos_t));
    const float phi = 2.0f * PI * b;
    return norm(in_frame(axis, v3(sin_t * std::cos(phi), sin_t * std::sin(phi), cos_t)));
}
V reflect(V i, V n) { return i - n * (2.0f * dot(n, i)); }
V refract(V i, V n, float eta) {
    const float ni = dot(n, i);
    const float k = 1.0f - eta * eta * (1.0f - ni * ni);
    if (k < 0.0f) return vs(0.0f);
    return i * eta - n * (eta * ni + std::sqrt(k));
}

struct Bs {
    V wi, weight;
    float pdf;
    bool delta, ok;
};
Bs sample_bsdf(const Mat& m, V base, const Surf& sf, V wo, Sampler& s) {
    const V n = sf.n;
    const float nv = dot(n, wo);
    if (m.kind == 3) {
        const float eta = sf.front ? m.ior : 1.0f / m.ior;
        const float f = fresnel(clampf(nv, 0.0f, 1.0f), eta);
        if (s.rand() < f) return {reflect(-wo, n), vs(1.0f), 0.0f, true, true};
        const V wi = refract(-wo, n, 1.0f / eta);
        if (dot(wi, wi) == 0.0f) return {reflect(-wo, n), vs(1.0f), 0.0f, true, true};
        return {norm(wi), sf.front ? base : vs(1.0f), 0.0f, true, true};
    }
    if (m.kind == 1 && m.roughness < 0.01f) return {reflect(-wo, n), schlick_v(base, nv), 0.0f, true, true};
    V wi;
    if (m.kind == 0) {
        wi = cosine_hemisphere(n, s);
    } else if (m.kind == 1 || s.rand() < spec_chance(m, nv)) {
        const float a2 = ggx_alpha2(m.roughness);
        float a, b;
        s.rand2(a, b);
        const float cos_t = std::sqrt((1.0f - a) / (1.0f + (a2 - 1.0f) * a));
        const float sin_t = std::sqrt(wmax(0.0f, 1.0f - cos_t * cos_t));
        const float phi = 2.0f * PI * b;
        const V h = norm(in_frame(n, v3(sin_t * std::cos(phi), sin_t * std::sin(phi), cos_t)));
        wi = reflect(-wo, h);
    } else {
        wi = cosine_hemisphere(n, s);
    }
    if (dot(wi, sf.ng) <= 0.0f) return {vs(0), vs(0), 0.0f, false, false};
    V f;
    float pdf;
    eval_bsdf(m, base, n, wo, wi, f, pdf);
    if (pdf <= 0.0f) return {vs(0), vs(0), 0.0f, false, false};
    return {wi, f / pdf, pdf, false, true};
}

// ---- lights (src/shaders.mjs:877-1018), the environment among them ----
// light_choices (src/shaders.mjs:877-879): the lights, the sun, then the environment.
uint32_t choices(const Ctx& c) { return c.P.light_count + (c.P.sun_on != 0u ? 1u : 0u) + (env_on(c) ? 1u : 0u); }
float light_cdf(const Ctx& c, uint32_t l) { return bitsf(c.lights[c.P.light_count + c.P.volume_count + l]); }
float light_chance(const Ctx& c, uint32_t l) {
    const float below = l > 0u ? light_cdf(c, l - 1u) : 0.0f;
    return (light_cdf(c, l) - below) * float(c.P.light_count) / float(choices(c));
}
float sphere_omc(float r, float d2) {
    const float x = wmin(r * r / d2, 1.0f);
    return x / (1.0f + std::sqrt(1.0f - x));
}
float power_heuristic(float a, float b) {
    const float a2 = a * a, b2 = b * b;
    if (a2 + b2 <= 0.0f) return 0.0f;
    return a2 / (a2 + b2);
}
struct Ls {
    V wi;
    float dist;
    V radiance;
    float pdf;
};
Ls sample_light(Ctx& c, V p, Sampler& s) {
    const Params& P = c.P;
    const uint32_t ch = choices(c);
    const float x = s.rand() * float(ch);
    uint32_t pick = std::min(uint32_t(x), ch - 1u);
    float chance = 1.0f / float(ch);
    if (env_on(c) && pick == P.light_count + (P.sun_on != 0u ? 1u : 0u)) {
        const V wi = sample_env(c, s);
        const float pdf = env_pdf(c, wi);
        if (pdf <= 0.0f) return {vs(0), 0.0f, vs(0), 0.0f};
        return {wi, INF, env_radiance(c, wi), chance * pdf};
    }
    if (P.sun_on != 0u && pick == P.light_count) {
        const V wi = sample_cone(vf(P.sun_dir), P.sun_omc, s);
        return {wi, INF, vf(P.sun_radiance), chance / (2.0f * PI * P.sun_omc)};
    }
    // pick_light: the first CDF entry above u.
    const float u = x / float(P.light_count);
    uint32_t lo = 0u, hi = P.light_count - 1u;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) / 2u;
        if (light_cdf(c, mid) > u) hi = mid;
        else lo = mid + 1u;
    }
    pick = lo;
    chance = light_chance(c, pick);
    const uint32_t pi = c.lights[pick];
    const float* pr = c.pf(pi);
    const Mat m = material(c, c.pu(pi)[1]);
    c.bytes += 64 + 96;
    if (c.pu(pi)[0] == 1) {
        float a, b;
        s.rand2(a, b);
        const V q = vf(pr + 4) + vf(pr + 8) * a + vf(pr + 12) * b;
        const V to = q - p;
        const float d2 = dot(to, to);
        const float dist = std::sqrt(d2);
        const V wi = to / dist;
        const V cr = cross(vf(pr + 8), vf(pr + 12));
        const float area = len(cr);
        const float cos_l = -dot(wi, cr / area);
        if (cos_l <= 0.0f) return {vs(0), 0.0f, vs(0), 0.0f};
        return {wi, dist, emitted(c, m, a, 1.0f - b), chance * d2 / (cos_l * area)};
    }
    const V to = vf(pr + 4) - p;
    const float d2 = dot(to, to);
    const float r = pr[7];
    if (d2 <= r * r) return {vs(0), 0.0f, vs(0), 0.0f};
    const float omc = sphere_omc(r, d2);
    const V wi = sample_cone(to / std::sqrt(d2), omc, s);
    const float b = dot(to, wi);
    const float dist = b - std::sqrt(wmax(b * b - (d2 - r * r), 0.0f));
    V e = m.emission;
    if (c.textures && m.emission_texture != NONE) {
        float u, v;
        sphere_uv(norm(p + wi * dist - vf(pr + 4)), pr, u, v);
        e = emitted(c, m, u, v);
    }
    return {wi, dist, e, chance / (2.0f * PI * omc)};
}
float light_pdf(const Ctx& c, uint32_t prim, V p, V wi, float t) {
    const float* pr = c.pf(prim);
    const float chance = light_chance(c, c.pu(prim)[2]);
    if (c.pu(prim)[0] == 1) {
        const V cr = cross(vf(pr + 8), vf(pr + 12));
        const float area = len(cr);
        const float cos_l = std::fabs(dot(wi, cr / area));
        return chance * t * t / wmax(cos_l * area, 1e-12f);
    }
    const V to = vf(pr + 4) - p;
    return chance / (2.0f * PI * sphere_omc(pr[7], dot(to, to)));
}

// ---- media (src/shaders.mjs:1024-1123) ----
inline float safe1(float d) { return std::fabs(d) < 1e-20f ? (d >= 0.0f ? 1e-20f : -1e-20f) : d; }
void volume_span(const Ctx& c, uint32_t i, V o, V d, float& x, float& y) {
    const float* p = c.pf(i);
    if (c.pu(i)[0] == 0) {
        const V oc = o - vf(p + 4);
        const float a = dot(d, d), hb = dot(oc, d);
        const float disc = hb * hb - a * (dot(oc, oc) - p[7] * p[7]);
        if (disc < 0.0f) {
            x = 1.0f;
            y = 0.0f;
            return;
        }
        const float sq = std::sqrt(disc);
        x = wmax((-hb - sq) / a, 0.0f);
        y = (-hb + sq) / a;
        return;
    }
    float tn = -INF, tf = INF, tminv[3], tmaxv[3];
    for (int r = 0; r < 3; ++r) {
        const V row = vf(p + 4 + r * 4);
        const float lo = dot(row, o) + p[7 + r * 4];
        const float inv = 1.0f / safe1(dot(row, d));
        const float t0 = (-1.0f - lo) * inv, t1 = (1.0f - lo) * inv;
        tminv[r] = wmin(t0, t1);
        tmaxv[r] = wmax(t0, t1);
    }
    (void)tn;
    (void)tf;
    x = wmax(wmax(wmax(tminv[0], tminv[1]), tminv[2]), 0.0f);
    y = wmin(wmin(tmaxv[0], tmaxv[1]), tmaxv[2]);
}
float hg(float cth, float g) {
    const float k = 1.0f + g * g - 2.0f * g * cth;
    return (1.0f - g * g) / (4.0f * PI * k * std::sqrt(k));
}
float transmittance(const Ctx& c, V o, V d, float dist) {
    float depth = 0.0f;
    for (uint32_t k = 0; k < c.P.volume_count; ++k) {
        const uint32_t i = c.lights[c.P.light_count + k];
        float x, y;
        volume_span(c, i, o, d, x, y);
        const float end = wmin(y, dist);
        if (x < end) depth += c.mf(c.pu(i)[1])[20] * (end - x);
    }
    return std::exp(-depth);
}

// ---- dispersion (src/shaders.mjs:1127-1144) ----
float lobe(float x, float mu, float below, float above) {
    const float t = (x - mu) / (x < mu ? below : above);
    return std::exp(-0.5f * t * t);
}
V wavelength_rgb(float l) {
    const float x = 1.056f * lobe(l, 599.8f, 37.9f, 31.0f) + 0.362f * lobe(l, 442.0f, 16.0f, 26.7f) -
                    0.065f * lobe(l, 501.1f, 20.4f, 26.2f);
    const float y = 0.821f * lobe(l, 568.8f, 46.9f, 40.5f) + 0.286f * lobe(l, 530.9f, 16.3f, 31.1f);
    const float z = 1.217f * lobe(l, 437.0f, 11.8f, 36.0f) + 0.681f * lobe(l, 459.0f, 26.0f, 13.8f);
    const V rgb = v3(3.2406f * x - 1.5372f * y - 0.4986f * z, -0.9689f * x + 1.8758f * y + 0.0415f * z,
                     0.0557f * x - 0.2040f * y + 1.0570f * z);
    return v3(wmax(rgb.x, 0.0f), wmax(rgb.y, 0.0f), wmax(rgb.z, 0.0f)) * v3(1.92985f, 2.94689f, 3.11081f);
}

bool roulette(V& tp, uint32_t depth, Sampler& s) {
    if (depth < 3u) return true;
    const float survive = wmin(wmax(tp.x, wmax(tp.y, tp.z)), 0.95f);
    if (s.rand() >= survive) return false;
    tp = tp / survive;
    return true;
}

// radiance() (src/shaders.mjs:1179-1359), for the color view.
V radiance(Ctx& c, float px, float py, Sampler& s, float spectrum_u, V& g_albedo, float g_normal[4]) {
    const Params& P = c.P;
    g_albedo = vs(1.0f);
    g_normal[0] = g_normal[1] = g_normal[2] = g_normal[3] = 0.0f;
    bool guided = false;
    float travelled = 0.0f;

    // camera_ray(px, true) (src/shaders.mjs:1148-1166)
    const float ndcx = 2.0f * px / float(P.width) - 1.0f, ndcy = 1.0f - 2.0f * py / float(P.height);
    const V fwd = vf(P.cam_forward), right = vf(P.cam_right), up = vf(P.cam_up), pos = vf(P.cam_pos);
    V dir = norm(fwd + right * (ndcx * P.tan_half_fov * P.aspect) + up * (ndcy * P.tan_half_fov));
    V o = pos, d = dir;
    if (P.lens_radius > 0.0f) {
        const V focus = pos + dir * (P.focus_distance / dot(dir, fwd));
        float a, b;
        s.rand2(a, b);
        const float ux = 2.0f * a - 1.0f, uy = 2.0f * b - 1.0f;
        float lx = 0.0f, ly = 0.0f;
        if (!(ux == 0.0f && uy == 0.0f)) {
            if (std::fabs(ux) > std::fabs(uy)) {
                const float phi = (PI / 4.0f) * (uy / ux);
                lx = ux * std::cos(phi);
                ly = ux * std::sin(phi);
            } else {
                const float phi = PI / 2.0f - (PI / 4.0f) * (ux / uy);
                lx = uy * std::cos(phi);
                ly = uy * std::sin(phi);
            }
        }
        o = pos + right * (lx * P.lens_radius) + up * (ly * P.lens_radius);
        d = norm(focus - o);
    }

    V throughput = vs(1.0f), result = vs(0.0f);
    float last_pdf = 0.0f;
    bool last_delta = true;
    V last_p = o;
    const uint32_t ch = choices(c);
    float wavelength = 0.0f;
    bool caustic = false, diffuse_seen = false;

    for (uint32_t depth = 0; depth <= P.max_bounces; ++depth) {
        s.qmc_dim = (depth + 1u) << 16u;
        const HitR hit = trace(c, o, d, INF, false);

        if (P.volume_count > 0) {
            float sc_t = hit.t;
            uint32_t sc_v = NONE;
            for (uint32_t k = 0; k < P.volume_count; ++k) {
                const uint32_t i = c.lights[P.light_count + k];
                float x, y;
                volume_span(c, i, o, d, x, y);
                const float end = wmin(y, sc_t);
                if (x < end) {
                    const float t = x - std::log(1.0f - s.rand()) / c.mf(c.pu(i)[1])[20];
                    if (t < end) {
                        sc_t = t;
                        sc_v = i;
                    }
                }
            }
            if (sc_v != NONE) {
                const Mat vm = material(c, c.pu(sc_v)[1]);
                const V p = o + d * sc_t;
                travelled += sc_t;
                if (!guided) {
                    guided = true;
                    g_albedo = throughput * vm.color;
                    g_normal[0] = -d.x;
                    g_normal[1] = -d.y;
                    g_normal[2] = -d.z;
                    g_normal[3] = travelled;
                }
                if (depth == P.max_bounces) break;
                throughput = throughput * vm.color;
                if (ch > 0u) {
                    const Ls ls = sample_light(c, p, s);
                    if (ls.pdf > 0.0f) {
                        const float phase = hg(dot(d, ls.wi), vm.anisotropy);
                        const float reach = ls.dist * (1.0f - 1e-3f);
                        if (trace(c, p, ls.wi, reach, true).prim == NONE)
                            result = result + throughput * ls.radiance *
                                                  (phase * transmittance(c, p, ls.wi, reach) *
                                                   power_heuristic(ls.pdf, phase) / ls.pdf);
                    }
                }
                float a, b;
                s.rand2(a, b);
                float cth = 1.0f - 2.0f * a;
                const float g = vm.anisotropy;
                if (std::fabs(g) >= 1e-3f) {
                    const float sq = (1.0f - g * g) / (1.0f + g - 2.0f * g * a);
                    cth = clampf((1.0f + g * g - sq * sq) / (2.0f * g), -1.0f, 1.0f);
                }
                const float sin_t = std::sqrt(wmax(0.0f, 1.0f - cth * cth));
                const float phi = 2.0f * PI * b;
                const V wi = norm(in_frame(d, v3(sin_t * std::cos(phi), sin_t * std::sin(phi), cth)));
                last_pdf = hg(dot(d, wi), g);
                last_delta = false;
                last_p = p;
                o = p;
                d = wi;
                caustic = false;
                diffuse_seen = true;
                if (!roulette(throughput, depth, s)) break;
                continue;
            }
        }

        if (hit.prim == NONE) {
            if (!guided) g_albedo = throughput;
            // An environment is sampled directly too: weigh it against that.
            float sky_weight = 1.0f;
            if (env_on(c) && !last_delta) sky_weight = power_heuristic(last_pdf, env_pdf(c, d) / float(ch));
            result = result + throughput * sky_at(c, d) * sky_weight;
            if (in_sun(P, d) && !(caustic && last_delta)) {
                float w = 1.0f;
                if (!last_delta) w = power_heuristic(last_pdf, 1.0f / (float(ch) * 2.0f * PI * P.sun_omc));
                result = result + throughput * vf(P.sun_radiance) * w;
            }
            break;
        }

        const Surf sf = surface(c, o, d, hit);
        const Mat m = material(c, sf.material);
        travelled += hit.t;
        if (!guided && (m.kind == 4 || !is_delta(m) || depth == P.max_bounces)) {
            guided = true;
            g_albedo = throughput * (m.kind == 4 ? vs(1.0f) : albedo_uv(c, m, sf.p, sf.u, sf.v));
            g_normal[0] = sf.n.x;
            g_normal[1] = sf.n.y;
            g_normal[2] = sf.n.z;
            g_normal[3] = travelled;
        }
        if (sf.front && (m.emission.x > 0.0f || m.emission.y > 0.0f || m.emission.z > 0.0f) &&
            !(caustic && last_delta && sf.light != NONE)) {
            float w = 1.0f;
            if (!last_delta && sf.light != NONE) w = power_heuristic(last_pdf, light_pdf(c, hit.prim, last_p, d, hit.t));
            result = result + throughput * emitted(c, m, sf.u, sf.v) * w;
        }
        if (m.kind == 4) break;
        if (!is_delta(m)) {
            caustic = P.caustics != 0u && !diffuse_seen;
            diffuse_seen = true;
        }
        if (depth == P.max_bounces) break;

        const V base = albedo_uv(c, m, sf.p, sf.u, sf.v);
        const V wo = -d;
        if (!is_delta(m) && ch > 0u) {
            const Ls ls = sample_light(c, sf.p, s);
            if (ls.pdf > 0.0f && dot(ls.wi, sf.ng) > 0.0f) {
                V f;
                float pdf;
                eval_bsdf(m, base, sf.n, wo, ls.wi, f, pdf);
                const V origin = offset(sf, ls.wi);
                const float reach = (ls.dist - dot(origin - sf.p, ls.wi)) * (1.0f - 1e-3f);
                if (pdf > 0.0f && trace(c, origin, ls.wi, reach, true).prim == NONE)
                    result = result + throughput * f * ls.radiance *
                                          (transmittance(c, origin, ls.wi, reach) * power_heuristic(ls.pdf, pdf) / ls.pdf);
            }
        }
        // dispersed (src/shaders.mjs:1412-1423)
        Mat sm = m;
        if (m.kind == 3 && m.dispersion > 0.0f) {
            if (wavelength == 0.0f) {
                wavelength = 380.0f + 340.0f * spectrum_u;
                throughput = throughput * wavelength_rgb(wavelength);
            }
            const float l = wavelength * 1e-3f;
            sm.ior = m.ior + m.dispersion * (1.0f / (l * l) - 1.0f / (0.5876f * 0.5876f));
        }
        const Bs bs = sample_bsdf(sm, base, sf, wo, s);
        if (!bs.ok) break;
        throughput = throughput * bs.weight;
        last_pdf = bs.pdf;
        last_delta = bs.delta;
        last_p = sf.p;
        o = offset(sf, bs.wi);
        d = bs.wi;
        if (!roulette(throughput, depth, s)) break;
    }
    return result;
}

// inspect() (src/shaders.mjs:1377-1407).
V inspect(Ctx& c, float px, float py) {
    const Params& P = c.P;
    const float ndcx = 2.0f * px / float(P.width) - 1.0f, ndcy = 1.0f - 2.0f * py / float(P.height);
    const V d = norm(vf(P.cam_forward) + vf(P.cam_right) * (ndcx * P.tan_half_fov * P.aspect) +
                     vf(P.cam_up) * (ndcy * P.tan_half_fov));
    const V o = vf(P.cam_pos);
    const HitR hit = trace(c, o, d, INF, false);
    if (hit.prim == NONE) return P.view == 1u ? sky_at(c, d) : vs(0.0f);
    const Surf sf = surface(c, o, d, hit);
    const Mat m = material(c, sf.material);
    if (P.view == 1u) {
        if (m.kind == 4) {
            const V e = emitted(c, m, sf.u, sf.v);
            return e / wmax(wmax(e.x, e.y), wmax(e.z, 1.0f));
        }
        return albedo_uv(c, m, sf.p, sf.u, sf.v);
    }
    if (P.view == 2u) return sf.n;
    return vs(hit.t);
}

// ---- light tracing and photon mapping (src/shaders.mjs:1425-1831) ----
const float SPLAT_SCALE = 65536.0f;
const uint32_t PHOTON_TABLE = 1048576u;

// frame (src/shaders.mjs:217-225): its first two columns.
inline void frame_cols(V n, V& c0, V& c1) {
    const float s = n.z >= 0.0f ? 1.0f : -1.0f;
    const float a = -1.0f / (s + n.z);
    const float b = n.x * n.y * a;
    c0 = v3(1.0f + s * n.x * n.x * a, s * b, -s * n.x);
    c1 = v3(b, s + n.y * n.y * a, -n.y);
}

// concentric_disk (src/shaders.mjs:245-256), from PCG numbers.
inline void concentric_disk(Sampler& sm, float& x, float& y) {
    float a, b;
    sm.rand2(a, b);
    const float ux = 2.0f * a - 1.0f, uy = 2.0f * b - 1.0f;
    x = y = 0.0f;
    if (ux == 0.0f && uy == 0.0f) return;
    if (std::fabs(ux) > std::fabs(uy)) {
        const float phi = (PI / 4.0f) * (uy / ux);
        x = ux * std::cos(phi);
        y = ux * std::sin(phi);
        return;
    }
    const float phi = PI / 2.0f - (PI / 4.0f) * (ux / uy);
    x = uy * std::cos(phi);
    y = uy * std::sin(phi);
}

// camera_ray(px, true) (src/shaders.mjs:1148-1166), as radiance() starts.
void camera_ray(const Params& P, float px, float py, Sampler& s, V& o, V& d) {
    const float ndcx = 2.0f * px / float(P.width) - 1.0f, ndcy = 1.0f - 2.0f * py / float(P.height);
    const V fwd = vf(P.cam_forward), right = vf(P.cam_right), up = vf(P.cam_up), pos = vf(P.cam_pos);
    const V dir = norm(fwd + right * (ndcx * P.tan_half_fov * P.aspect) + up * (ndcy * P.tan_half_fov));
    o = pos;
    d = dir;
    if (P.lens_radius > 0.0f) {
        const V focus = pos + dir * (P.focus_distance / dot(dir, fwd));
        float lx, ly;
        concentric_disk(s, lx, ly);
        o = pos + right * (lx * P.lens_radius) + up * (ly * P.lens_radius);
        d = norm(focus - o);
    }
}

struct Photon {
    uint32_t id;
    V p, beta, wi;  // where it landed, its power, and whence it came (-d)
    // Its splat: the pixel (NONE if the camera doesn't see it) and the
    // fixed-point amounts added; and the smallest edge margin (barycentric
    // distance to an edge) of the triangles and quads its path hit.
    uint32_t splat_pixel = NONE, splat_rgb[3] = {0u, 0u, 0u};
    float margin = INF;
};

// How close a closest hit came to its primitive's edge: a triangle's or a
// quad's barycentric distance to its nearest edge; for a box, the hit
// point's distance (in box space, where the box is [-1, 1]³) to the
// nearest edge of the face it lies on; for a sphere, the cosine between
// the ray and the surface (near 0 at the silhouette).
float edge_margin(const Ctx& c, V o, V d, const HitR& h) {
    if (h.prim == NONE) return 1.0f;
    const uint32_t kind = c.pu(h.prim)[0];
    if (kind == 3u) return wmin(wmin(h.u, h.v), 1.0f - h.u - h.v);
    if (kind == 1u) return wmin(wmin(h.u, 1.0f - h.u), wmin(h.v, 1.0f - h.v));
    const float* f = c.pf(h.prim);
    const V p = o + d * h.t;
    if (kind == 2u) {
        float gap[3];
        for (int k = 0; k < 3; ++k) {
            const float* row = f + 4 + 4 * k;
            gap[k] = 1.0f - std::fabs(row[0] * p.x + row[1] * p.y + row[2] * p.z + row[3]);
        }
        // the smallest gap is the face the point lies on; the next is its nearest edge
        const float lo = wmin(gap[0], wmin(gap[1], gap[2])), hi = wmax(gap[0], wmax(gap[1], gap[2]));
        return gap[0] + gap[1] + gap[2] - lo - hi;
    }
    if (kind == 0u) return std::fabs(dot(norm(p - vf(f + 4)), norm(d)));
    return 1.0f;
}

// splat (src/shaders.mjs:1443-1491): the photon's light added, in fixed
// point with random rounding, to the pixel that sees the surface.
void splat(Ctx& c, const Surf& s, const Mat& m, V base, V d, V beta, Sampler& sm, uint32_t* splats, Photon& rec) {
    const Params& P = c.P;
    const V to_camera = vf(P.cam_pos) - s.p;
    const float dist = len(to_camera);
    const V wo = to_camera / dist;
    const float cos_film = -dot(wo, vf(P.cam_forward));
    if (cos_film <= 1e-6f || dot(wo, s.ng) <= 0.0f) return;
    const float x = -dot(wo, vf(P.cam_right)) / (cos_film * P.tan_half_fov * P.aspect);
    const float y = -dot(wo, vf(P.cam_up)) / (cos_film * P.tan_half_fov);
    const float px = (x + 1.0f) * 0.5f * float(P.width);
    const float py = (1.0f - y) * 0.5f * float(P.height);
    if (px < 0.0f || py < 0.0f || px >= float(P.width) || py >= float(P.height)) return;
    const V wi = -d;
    V f;
    float pdf;
    eval_bsdf(m, base, s.n, wo, wi, f, pdf);
    const float cos_in = dot(s.n, wi);
    if (pdf <= 0.0f || cos_in <= 0.0f) return;
    const V origin = offset(s, wo);
    if (trace(c, origin, wo, dist - dot(origin - s.p, wo), true).prim != NONE) return;
    const float pixel_area = (4.0f * P.tan_half_fov * P.tan_half_fov * P.aspect) / float(P.width * P.height);
    const V value = beta * (f / cos_in) * dot(wo, s.ng) /
                    (dist * dist * pixel_area * cos_film * cos_film * cos_film);
    if (!finite3(value)) return;
    const uint32_t index = (uint32_t(py) * P.width + uint32_t(px)) * 4u;
    const float r0 = sm.rand(), r1 = sm.rand(), r2 = sm.rand();
    const V fixed = value * SPLAT_SCALE + v3(r0, r1, r2);
    rec.splat_pixel = index / 4u;
    rec.splat_rgb[0] = uint32_t(wmin(fixed.x, 4e9f));
    rec.splat_rgb[1] = uint32_t(wmin(fixed.y, 4e9f));
    rec.splat_rgb[2] = uint32_t(wmin(fixed.z, 4e9f));
    splats[index] += rec.splat_rgb[0];
    splats[index + 1] += rec.splat_rgb[1];
    splats[index + 2] += rec.splat_rgb[2];
}

// light_trace (src/shaders.mjs:1628-1814): photon `id` from a light
// chosen by power, through mirrors and glass, splatted and stored where it
// first lands on anything else. E is the emitters buffer's vec4s.
void light_trace(Ctx& c, const float* E, uint32_t photons, uint32_t id, uint32_t seed_hash, uint32_t* splats,
                 std::vector<Photon>& stored, float* margin_out = nullptr) {
    const Params& P = c.P;
    Sampler sm = light_sampler(id, P.sample_offset, seed_hash);
    const float* header = E;
    const uint32_t sources = fbits(header[0]), targets = fbits(header[1]);
    const float xi = sm.rand();
    uint32_t k = 0;
    while (!(k + 1u >= sources || E[(1 + k) * 4] > xi)) ++k;
    const float* entry = E + (1 + k) * 4;
    const float chance = entry[2];
    if (chance <= 0.0f) return;
    const uint32_t prim_index = fbits(entry[1]);
    const uint32_t first_target = 1u + sources;
    auto target = [&](uint32_t i) { return E + (first_target + i) * 4; };

    V o, d, beta;
    if (prim_index == NONE) {
        d = -sample_cone(vf(P.sun_dir), P.sun_omc, sm);
        float pick = sm.rand() * header[3] / PI;
        uint32_t j = 0;
        for (;;) {
            const float r = target(j)[3];
            if (j + 1u >= targets || pick < r * r) break;
            pick -= r * r;
            ++j;
        }
        const float* circle = target(j);
        V c0, c1;
        frame_cols(d, c0, c1);
        float dx, dy;
        concentric_disk(sm, dx, dy);
        dx *= circle[3];
        dy *= circle[3];
        o = vf(circle) - d * header[2] + c0 * dx + c1 * dy;
        if (g_jitter_size != 0.0f) nudge(o, d);  // the counts below decide on the ray before it is traced
        float through = 1.0f;
        for (uint32_t i = 0; i < targets; ++i) {
            const V q = o - vf(target(i));
            const V across = q - d * dot(q, d);
            through += (i != j && dot(across, across) < target(i)[3] * target(i)[3]) ? 1.0f : 0.0f;
        }
        const V irradiance = vf(P.sun_radiance) * (2.0f * PI * P.sun_omc);
        beta = irradiance * header[3] / (through * chance * float(photons));
    } else {
        const float* pf = c.pf(prim_index);
        const uint32_t* pu = c.pu(prim_index);
        const Mat m = material(c, pu[1]);
        V n;
        float area, eu = 0.0f, ev = 0.0f;
        if (pu[0] == 1u) {  // QUAD
            const float a = sm.rand();
            const float b = sm.rand();
            o = vf(pf + 4) + vf(pf + 8) * a + vf(pf + 12) * b;
            const V cr = cross(vf(pf + 8), vf(pf + 12));
            area = len(cr);
            n = cr / area;
            eu = a;
            ev = 1.0f - b;
        } else {
            const float z = 1.0f - 2.0f * sm.rand();
            const float r = std::sqrt(wmax(0.0f, 1.0f - z * z));
            const float phi = 2.0f * PI * sm.rand();
            n = v3(r * std::cos(phi), z, r * std::sin(phi));
            o = vf(pf + 4) + n * pf[7];
            area = 4.0f * PI * pf[7] * pf[7];
            sphere_uv(n, pf, eu, ev);
        }
        if (g_jitter_size != 0.0f) {  // the aim below decides on the emission point before any ray is traced
            V normal = n;
            nudge(o, normal);
        }
        float cones = 0.0f;
        bool inside = false;
        for (uint32_t i = 0; i < targets; ++i) {
            const float* aim = target(i);
            const V to = vf(aim) - o;
            const float d2 = dot(to, to);
            inside = inside || d2 <= aim[3] * aim[3];
            cones += sphere_omc(aim[3], wmax(d2, aim[3] * aim[3]));
        }
        if (!inside) {
            float pick = sm.rand() * cones;
            uint32_t j = 0;
            for (;;) {
                const float* aim = target(j);
                const V to = vf(aim) - o;
                const float omc = sphere_omc(aim[3], dot(to, to));
                if (j + 1u >= targets || pick < omc) {
                    d = sample_cone(to / len(to), omc, sm);
                    break;
                }
                pick -= omc;
                ++j;
            }
            if (g_jitter_size != 0.0f) nudge(o, d);
            float within = 1.0f;
            for (uint32_t i = 0; i < targets; ++i) {
                const float* aim = target(i);
                const V to = vf(aim) - o;
                const float omc = sphere_omc(aim[3], dot(to, to));
                within += (i != j && 1.0f - dot(d, to / len(to)) <= omc) ? 1.0f : 0.0f;
            }
            const float cos_out = dot(d, n);
            if (cos_out <= 0.0f) return;
            beta = emitted(c, m, eu, ev) * (cos_out * area * 2.0f * PI * cones) / (within * chance * float(photons));
        } else {
            d = cosine_hemisphere(n, sm);
            beta = emitted(c, m, eu, ev) * (PI * area) / (chance * float(photons));
        }
        o = o + n * (1e-4f * wmax(1.0f, wmax(std::fabs(o.x), wmax(std::fabs(o.y), std::fabs(o.z)))));
    }

    float wavelength = 0.0f;
    uint32_t bounces = 0;
    V carried = vs(1.0f);
    float margin = INF;
    for (uint32_t depth = 0; depth < P.max_bounces; ++depth) {
        const HitR hit = trace(c, o, d, INF, false);
        if (hit.prim == NONE) return;
        if (margin_out) {  // tracked only when asked for: it costs a second traversal per hit
            margin = wmin(margin, edge_margin(c, o, d, hit));
            const float of[3] = {o.x, o.y, o.z}, df[3] = {d.x, d.y, d.z};
            if (ro_tie32(c.prims, c.nodes, of, df, hit.t, 1e-5f, hit.prim)) margin = 0.0f;
            *margin_out = margin;
        }
        const Surf s = surface(c, o, d, hit);
        const Mat m = material(c, s.material);
        if (m.kind == 4) return;
        const V base = albedo_uv(c, m, s.p, s.u, s.v);
        if (!is_delta(m)) {
            if (bounces > 0u) {
                Photon rec{id, s.p, beta * carried, -d};
                rec.margin = margin;
                splat(c, s, m, base, d, beta * carried, sm, splats, rec);
                stored.push_back(rec);
            }
            return;
        }
        // dispersed (src/shaders.mjs:1412-1423), its random number drawn
        // whether or not the glass splits colours.
        const float u = sm.rand();
        Mat dm = m;
        if (m.kind == 3 && m.dispersion > 0.0f) {
            if (wavelength == 0.0f) {
                wavelength = 380.0f + 340.0f * u;
                carried = carried * wavelength_rgb(wavelength);
            }
            const float l = wavelength * 1e-3f;
            dm.ior = m.ior + m.dispersion * (1.0f / (l * l) - 1.0f / (0.5876f * 0.5876f));
        }
        const Bs bs = sample_bsdf(dm, base, s, -d, sm);
        if (!bs.ok) return;
        carried = carried * bs.weight;
        ++bounces;
        o = offset(s, bs.wi);
        d = bs.wi;
        if (!roulette(carried, depth, sm)) return;
    }
}

inline uint32_t photon_cell_hash(int32_t x, int32_t y, int32_t z) {
    return ((uint32_t(x) * 73856093u) ^ (uint32_t(y) * 19349663u) ^ (uint32_t(z) * 83492791u)) & (PHOTON_TABLE - 1u);
}

struct PhotonMap {
    const float* ph;                 // 9 floats a photon: p, beta, wi
    std::vector<uint32_t> heads, next;  // lists through the photons, index + 1, 0 ends
};

// gather (src/shaders.mjs:1533-1572).
V gather(const Params& P, const PhotonMap& map, const Surf& s, const Mat& m, V base, V wo, uint32_t* visits = nullptr) {
    const float r = P.photon_radius;
    const float r2 = r * r;
    const float cell_size = P.photon_cell;
    const V here = s.p / cell_size;
    const int32_t cx = int32_t(std::floor(here.x)), cy = int32_t(std::floor(here.y)), cz = int32_t(std::floor(here.z));
    const int32_t sx = here.x - std::floor(here.x) >= 0.5f ? 1 : -1;
    const int32_t sy = here.y - std::floor(here.y) >= 0.5f ? 1 : -1;
    const int32_t sz = here.z - std::floor(here.z) >= 0.5f ? 1 : -1;
    V sum = vs(0.0f);
    uint32_t visited = 0;
    for (uint32_t k = 0; k < 8u; ++k) {
        uint32_t index = map.heads[photon_cell_hash(cx + int32_t(k & 1u) * sx, cy + int32_t((k >> 1u) & 1u) * sy,
                                                    cz + int32_t((k >> 2u) & 1u) * sz)];
        for (;;) {
            if (index == 0u || visited >= 4096u) break;
            ++visited;
            const float* at = map.ph + size_t(index - 1u) * 9;
            const V off = vf(at) - s.p;
            if (dot(off, off) < r2 && std::fabs(dot(off, s.ng)) < 0.25f * r) {
                const V wi = vf(at + 6);
                const float cos_in = dot(s.n, wi);
                if (cos_in > 0.0f && dot(s.ng, wi) > 0.0f) {
                    V f;
                    float pdf;
                    eval_bsdf(m, base, s.n, wo, wi, f, pdf);
                    sum = sum + vf(at + 3) * (f / cos_in);
                }
            }
            index = map.next[index - 1u];
        }
    }
    if (visits) *visits = visited;
    return sum / (PI * r2);
}

}  // namespace

namespace {
void render_impl(const void* prims, const void* nodes, const void* materials, const float* attributes,
                 const uint32_t* lights, const void* params208, uint32_t seed_hash, uint32_t x0, uint32_t y0,
                 uint32_t rw, uint32_t rh, float* accum_out, float* albedo_out, float* normal_out, uint64_t* counters,
                 int threads, const Env* env, const Tex* textures, const Tex* normal_maps) {
    Params P;
    std::memcpy(&P, params208, sizeof P);
    std::atomic<uint32_t> next{0};
    std::atomic<uint64_t> tot_bytes{0}, tot_rays{0}, tot_hits{0}, tot_tc{0}, tot_ts{0}, tot_rc{0}, tot_rs{0};
    const uint32_t n = rw * rh;
    auto worker = [&] {
        Ctx c{static_cast<const uint8_t*>(prims), static_cast<const uint8_t*>(nodes),
              static_cast<const float*>(materials), attributes, lights, P};
        c.env = env;
        c.textures = textures;
        c.normal_maps = normal_maps;
        for (;;) {
            const uint32_t k0 = next.fetch_add(64);
            if (k0 >= n) break;
            for (uint32_t k = k0; k < std::min(n, k0 + 64); ++k) {
                const uint32_t x = x0 + k % rw, y = y0 + k / rw;
                const uint32_t index = y * P.width + x;
                float sum[4] = {0, 0, 0, 0}, sa[3] = {0, 0, 0}, sn[4] = {0, 0, 0, 0};
                for (uint32_t s = 0; s < P.samples_per_frame; ++s) {
                    // main()'s seeding (src/shaders.mjs:1852-1859)
                    Sampler sm = camera_sampler(index, P.sample_offset + s, seed_hash);
                    const float spectrum_u = spectrum_at(index, P.sample_offset + s);
                    V col, ga = vs(0.0f);
                    float gn[4] = {0, 0, 0, 0};
                    if (P.view == 0u) {
                        float jx, jy;
                        sm.rand2(jx, jy);
                        col = radiance(c, float(x) + jx, float(y) + jy, sm, spectrum_u, ga, gn);
                        const float peak = wmax(col.x, wmax(col.y, col.z));
                        if (P.firefly_clamp > 0.0f && peak > P.firefly_clamp) col = col * (P.firefly_clamp / peak);
                    } else {
                        col = inspect(c, float(x) + 0.5f, float(y) + 0.5f);
                    }
                    if (finite3(col) && finite3(ga) && finite3(v3(gn[0], gn[1], gn[2])) && finite3(vs(gn[3]))) {
                        const float l = lum(col);
                        sum[0] += col.x;
                        sum[1] += col.y;
                        sum[2] += col.z;
                        sum[3] += l * l;
                        sa[0] += ga.x;
                        sa[1] += ga.y;
                        sa[2] += ga.z;
                        for (int q = 0; q < 4; ++q) sn[q] += gn[q];
                    }
                }
                for (int q = 0; q < 4; ++q) accum_out[size_t(k) * 4 + q] = sum[q];
                if (albedo_out) {
                    for (int q = 0; q < 3; ++q) albedo_out[size_t(k) * 4 + q] = sa[q];
                    albedo_out[size_t(k) * 4 + 3] = 0.0f;
                }
                if (normal_out)
                    for (int q = 0; q < 4; ++q) normal_out[size_t(k) * 4 + q] = sn[q];
            }
        }
        tot_bytes += c.bytes;
        tot_rays += c.rays;
        tot_hits += c.hits;
        tot_tc += c.trav_closest;
        tot_ts += c.trav_shadow;
        tot_rc += c.rays_closest;
        tot_rs += c.rays_shadow;
    };
    const int nt = std::max(1, threads);
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; ++t) pool.emplace_back(worker);
    worker();
    for (auto& t : pool) t.join();
    if (counters) {
        counters[0] = tot_bytes;
        counters[1] = tot_rays;
        counters[2] = tot_hits;
        counters[3] = uint64_t(n) * P.samples_per_frame;
        counters[4] = tot_tc;
        counters[5] = tot_ts;
        counters[6] = tot_rc;
        counters[7] = tot_rs;
    }
}
}  // namespace

extern "C" void ro_render(const void* prims, const void* nodes, const void* materials, const float* attributes,
                          const uint32_t* lights, const void* params208, uint32_t seed_hash, uint32_t x0, uint32_t y0,
                          uint32_t rw, uint32_t rh, float* accum_out, float* albedo_out, float* normal_out,
                          uint64_t* counters, int threads) {
    render_impl(prims, nodes, materials, attributes, lights, params208, seed_hash, x0, y0, rw, rh, accum_out,
                albedo_out, normal_out, counters, threads, nullptr, nullptr, nullptr);
}

extern "C" void ro_render_scene(const void* prims, const void* nodes, const void* materials, const float* attributes,
                                const uint32_t* lights, const void* params208, uint32_t seed_hash, uint32_t x0,
                                uint32_t y0, uint32_t rw, uint32_t rh, float* accum_out, float* albedo_out,
                                float* normal_out, uint64_t* counters, int threads, const uint16_t* env_rgba16f,
                                uint32_t env_w, uint32_t env_h, const float* table, uint32_t cw, uint32_t ch,
                                const uint8_t* tex, uint32_t tex_w, uint32_t tex_h, const uint8_t* nrm,
                                uint32_t nrm_w, uint32_t nrm_h) {
    const Env env{env_rgba16f, env_w, env_h, table, cw, ch};
    const Tex t{tex, tex_w, tex_h}, n{nrm, nrm_w, nrm_h};
    render_impl(prims, nodes, materials, attributes, lights, params208, seed_hash, x0, y0, rw, rh, accum_out,
                albedo_out, normal_out, counters, threads, env_rgba16f ? &env : nullptr, tex ? &t : nullptr,
                nrm ? &n : nullptr);
}

// light_trace for photons id0..id0+count-1 of a frame of `photons`
// (src/shaders.mjs:1628-1814): splats (W·H·4 u32, added to, wrapping as the
// GPU's atomics do) and the stored photons (9 floats each: p, beta, -d) in
// photon order. Returns how many were stored.
extern "C" uint32_t ro_light_trace(const void* prims, const void* nodes, const void* materials, const float* attributes,
                                   const uint32_t* lights, const void* params208, const float* emitters,
                                   uint32_t photons, uint32_t id0, uint32_t count, uint32_t seed_hash,
                                   uint32_t* splats, float* photons_out, uint32_t* ids_out, uint32_t* splat_out,
                                   float* margin_out, float* path_margin_out, int threads) {
    Params P;
    std::memcpy(&P, params208, sizeof P);
    const uint32_t cells = P.width * P.height * 4u;
    const int nt = std::max(1, threads);
    std::vector<std::vector<uint32_t>> part_splats(nt, std::vector<uint32_t>(cells, 0u));
    std::vector<std::vector<Photon>> part_photons(nt);
    std::atomic<uint32_t> next{0};
    auto worker = [&](int t) {
        Ctx c{static_cast<const uint8_t*>(prims), static_cast<const uint8_t*>(nodes),
              static_cast<const float*>(materials), attributes, lights, P};
        for (;;) {
            const uint32_t k0 = next.fetch_add(256);
            if (k0 >= count) break;
            for (uint32_t k = k0; k < std::min(count, k0 + 256); ++k)
                light_trace(c, emitters, photons, id0 + k, seed_hash, part_splats[t].data(), part_photons[t],
                            path_margin_out ? path_margin_out + k : nullptr);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; ++t) pool.emplace_back(worker, t);
    worker(0);
    for (auto& t : pool) t.join();
    for (int t = 0; t < nt; ++t)
        for (uint32_t i = 0; i < cells; ++i) splats[i] += part_splats[t][i];
    std::vector<Photon> all;
    for (auto& v : part_photons) all.insert(all.end(), v.begin(), v.end());
    std::sort(all.begin(), all.end(), [](const Photon& a, const Photon& b) { return a.id < b.id; });
    for (size_t i = 0; i < all.size(); ++i) {
        float* q = photons_out + i * 9;
        if (ids_out) ids_out[i] = all[i].id;
        if (splat_out) {
            splat_out[i * 4] = all[i].splat_pixel;
            for (int k = 0; k < 3; ++k) splat_out[i * 4 + 1 + k] = all[i].splat_rgb[k];
        }
        if (margin_out) margin_out[i] = all[i].margin;
        const V* v[3] = {&all[i].p, &all[i].beta, &all[i].wi};
        for (int j = 0; j < 3; ++j) {
            q[j * 3] = v[j]->x;
            q[j * 3 + 1] = v[j]->y;
            q[j * 3 + 2] = v[j]->z;
        }
    }
    return uint32_t(all.size());
}

// photon_gather (src/shaders.mjs:1585-1626) on rows y0..y0+rows-1: per
// pixel, from the camera through mirrors and glass to the first other
// surface, the photons near it; added to accum (W·H·4) once for each of the
// frame's samples.
extern "C" void ro_photon_gather(const void* prims, const void* nodes, const void* materials, const float* attributes,
                                 const uint32_t* lights, const void* params208, const float* photons, uint32_t count,
                                 uint32_t y0, uint32_t rows, uint32_t seed_hash, float* accum, uint32_t* visits_out,
                                 int threads) {
    Params P;
    std::memcpy(&P, params208, sizeof P);
    PhotonMap map{photons, std::vector<uint32_t>(PHOTON_TABLE, 0u), std::vector<uint32_t>(count, 0u)};
    for (uint32_t i = 0; i < count; ++i) {
        const float* p = photons + size_t(i) * 9;
        const uint32_t h = photon_cell_hash(int32_t(std::floor(p[0] / P.photon_cell)),
                                            int32_t(std::floor(p[1] / P.photon_cell)),
                                            int32_t(std::floor(p[2] / P.photon_cell)));
        map.next[i] = map.heads[h];
        map.heads[h] = i + 1u;
    }
    const uint32_t first = std::min(y0, P.height) * P.width;
    const uint32_t n = std::min(y0 + rows, P.height) * P.width;
    std::atomic<uint32_t> next{first};
    auto worker = [&] {
        Ctx c{static_cast<const uint8_t*>(prims), static_cast<const uint8_t*>(nodes),
              static_cast<const float*>(materials), attributes, lights, P};
        for (;;) {
            const uint32_t k0 = next.fetch_add(64);
            if (k0 >= n) break;
            for (uint32_t index = k0; index < std::min(n, k0 + 64); ++index) {
                Sampler sm = gather_sampler(index, P.sample_offset, seed_hash);
                const float jx = sm.rand();
                const float jy = sm.rand();
                V o, d;
                camera_ray(P, float(index % P.width) + jx, float(index / P.width) + jy, sm, o, d);
                V throughput = vs(1.0f);
                for (uint32_t depth = 0; depth < P.max_bounces; ++depth) {
                    const HitR hit = trace(c, o, d, INF, false);
                    if (hit.prim == NONE) break;
                    const Surf s = surface(c, o, d, hit);
                    const Mat m = material(c, s.material);
                    if (m.kind == 4) break;
                    const V base = albedo_uv(c, m, s.p, s.u, s.v);
                    if (!is_delta(m)) {
                        if (depth > 0u) {
                            uint32_t visits = 0;
                            const V light = throughput * gather(P, map, s, m, base, -d, &visits);
                            if (visits_out) visits_out[index] = visits;
                            if (finite3(light)) {
                                const float l = lum(light);
                                const float spf = float(P.samples_per_frame);
                                accum[size_t(index) * 4] += light.x * spf;
                                accum[size_t(index) * 4 + 1] += light.y * spf;
                                accum[size_t(index) * 4 + 2] += light.z * spf;
                                accum[size_t(index) * 4 + 3] += l * l * spf;
                            }
                        }
                        break;
                    }
                    const Bs bs = sample_bsdf(m, base, s, -d, sm);
                    if (!bs.ok) break;
                    throughput = throughput * bs.weight;
                    o = offset(s, bs.wi);
                    d = bs.wi;
                }
            }
        }
    };
    const int nt = std::max(1, threads);
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; ++t) pool.emplace_back(worker);
    worker();
    for (auto& t : pool) t.join();
}

// ---- denoiser (src/shaders.mjs:1930-2097) ----
namespace {
struct Den {
    const float *accum, *ga, *gn;
    uint32_t w, h;
    float n;
    V albedo_at(uint32_t i) const {
        return v3(wmax(ga[i * 4] / n, 0.01f), wmax(ga[i * 4 + 1] / n, 0.01f), wmax(ga[i * 4 + 2] / n, 0.01f));
    }
    void normal_at(uint32_t i, float* out) const {
        const V g = vf(gn + size_t(i) * 4);
        const V nn = dot(g, g) > 0.0f ? norm(g) : vs(0.0f);
        out[0] = nn.x;
        out[1] = nn.y;
        out[2] = nn.z;
        out[3] = gn[size_t(i) * 4 + 3] / n;
    }
    V light_at(uint32_t i) const {
        const V a = albedo_at(i);
        return v3(accum[i * 4] / n / a.x, accum[i * 4 + 1] / n / a.y, accum[i * 4 + 2] / n / a.z);
    }
};
float similarity(const float* p, const float* q, float step) {
    if (p[3] <= 0.0f || q[3] <= 0.0f) return (p[3] <= 0.0f && q[3] <= 0.0f) ? 1.0f : 0.0f;
    if (p[0] * p[0] + p[1] * p[1] + p[2] * p[2] == 0.0f) return 0.0f;
    const float wn = std::pow(wmax(p[0] * q[0] + p[1] * q[1] + p[2] * q[2], 0.0f), 64.0f);
    const float wz = std::exp(-std::fabs(p[3] - q[3]) / (p[3] * 0.02f * step + 1e-6f));
    return wn * wz;
}
const float KERNEL[3] = {0.375f, 0.25f, 0.0625f};

template <typename F>
void rows(uint32_t h, int threads, F fn) {
    std::atomic<uint32_t> next{0};
    auto worker = [&] {
        for (;;) {
            const uint32_t y = next.fetch_add(1);
            if (y >= h) return;
            fn(y);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < std::max(1, threads); ++t) pool.emplace_back(worker);
    worker();
    for (auto& t : pool) t.join();
}
}  // namespace

extern "C" void ro_denoise(const float* accum, const float* guide_albedo, const float* guide_normal, uint32_t w,
                           uint32_t h, uint32_t total_samples, float* out, int threads) {
    Den D{accum, guide_albedo, guide_normal, w, h, float(std::max(total_samples, 1u))};
    std::vector<float> a(size_t(w) * h * 4), b(size_t(w) * h * 4);
    // prepare
    rows(h, threads, [&](uint32_t y) {
        for (uint32_t x = 0; x < w; ++x) {
            const uint32_t i = y * w + x;
            const V light = D.light_at(i);
            float gp[4];
            D.normal_at(i, gp);
            const float al = lum(D.albedo_at(i));
            float variance;
            if (D.n >= 4.0f) {
                const float mean = lum(vf(accum + size_t(i) * 4)) / D.n;
                const float spread = wmax(accum[i * 4 + 3] / D.n - mean * mean, 0.0f) * D.n / (D.n - 1.0f);
                variance = spread / D.n / (al * al);
            } else {
                float sum = 0, sum2 = 0, weight = 0;
                for (int dy = -2; dy <= 2; ++dy)
                    for (int dx = -2; dx <= 2; ++dx) {
                        const int xx = int(x) + dx, yy = int(y) + dy;
                        if (xx < 0 || yy < 0 || xx >= int(w) || yy >= int(h)) continue;
                        const uint32_t j = uint32_t(yy) * w + uint32_t(xx);
                        float gq[4];
                        D.normal_at(j, gq);
                        const float wt = similarity(gp, gq, 1.0f);
                        const float l = lum(D.light_at(j));
                        sum += wt * l;
                        sum2 += wt * l * l;
                        weight += wt;
                    }
                const float mean = sum / wmax(weight, 1e-6f);
                variance = wmax(sum2 / wmax(weight, 1e-6f) - mean * mean, 0.0f) + 0.01f * mean * mean;
            }
            a[i * 4] = light.x;
            a[i * 4 + 1] = light.y;
            a[i * 4 + 2] = light.z;
            a[i * 4 + 3] = variance;
        }
    });
    std::vector<float>* from = &a;
    std::vector<float>* to = &b;
    for (int step : {1, 2, 4, 8, 16}) {
        const std::vector<float>& in = *from;
        std::vector<float>& o = *to;
        rows(h, threads, [&](uint32_t y) {
            for (uint32_t x = 0; x < w; ++x) {
                const uint32_t i = y * w + x;
                float gp[4];
                D.normal_at(i, gp);
                const float lp = lum(vf(&in[size_t(i) * 4]));
                float variance = 0, vw = 0;
                for (int dy = -1; dy <= 1; ++dy)
                    for (int dx = -1; dx <= 1; ++dx) {
                        const int xx = int(x) + dx, yy = int(y) + dy;
                        if (xx >= 0 && yy >= 0 && xx < int(w) && yy < int(h)) {
                            const float wt = KERNEL[std::abs(dx)] * KERNEL[std::abs(dy)];
                            variance += wt * in[(size_t(yy) * w + xx) * 4 + 3];
                            vw += wt;
                        }
                    }
                const float sigma = 4.0f * std::sqrt(variance / vw) + 1e-4f;
                V sum = vs(0);
                float sv = 0, weight = 0;
                for (int dy = -2; dy <= 2; ++dy)
                    for (int dx = -2; dx <= 2; ++dx) {
                        const int xx = int(x) + dx * step, yy = int(y) + dy * step;
                        if (xx < 0 || yy < 0 || xx >= int(w) || yy >= int(h)) continue;
                        const uint32_t j = uint32_t(yy) * w + uint32_t(xx);
                        const V q = vf(&in[size_t(j) * 4]);
                        float gq[4];
                        D.normal_at(j, gq);
                        const float wt = KERNEL[std::abs(dx)] * KERNEL[std::abs(dy)] * similarity(gp, gq, float(step)) *
                                         std::exp(-std::fabs(lp - lum(q)) / sigma);
                        sum = sum + q * wt;
                        sv += wt * wt * in[size_t(j) * 4 + 3];
                        weight += wt;
                    }
                if (weight > 0.0f) {
                    o[i * 4] = sum.x / weight;
                    o[i * 4 + 1] = sum.y / weight;
                    o[i * 4 + 2] = sum.z / weight;
                    o[i * 4 + 3] = sv / (weight * weight);
                } else {
                    for (int q = 0; q < 4; ++q) o[i * 4 + q] = in[i * 4 + q];
                }
            }
        });
        std::swap(from, to);
    }
    for (uint32_t i = 0; i < w * h; ++i) {
        const V al = D.albedo_at(i);
        out[i * 4] = (*from)[i * 4] * al.x;
        out[i * 4 + 1] = (*from)[i * 4 + 1] * al.y;
        out[i * 4 + 2] = (*from)[i * 4 + 2] * al.z;
        out[i * 4 + 3] = 0.0f;
    }
}

extern "C" void ro_display(const float* accum, const float* denoised, const void* params208, uint8_t* out) {
    Params P;
    std::memcpy(&P, params208, sizeof P);
    auto aces = [](float x) {
        return clampf((x * (2.51f * x + 0.03f)) / (x * (2.43f * x + 0.59f) + 0.14f), 0.0f, 1.0f);
    };
    auto srgb = [](float c) {
        const float x = clampf(c, 0.0f, 1.0f);
        return x <= 0.0031308f ? x * 12.92f : 1.055f * std::pow(x, 1.0f / 2.4f) - 0.055f;
    };
    auto byte = [](float v) { return uint8_t(std::lrint(clampf(v, 0.0f, 1.0f) * 255.0f)); };
    for (uint32_t i = 0; i < P.width * P.height; ++i) {
        float o[3] = {0, 0, 0};
        if (P.total_samples != 0u) {
            const float n = float(P.total_samples);
            const V c = v3(accum[i * 4] / n, accum[i * 4 + 1] / n, accum[i * 4 + 2] / n);
            if (P.view == 0u) {
                const V sh = P.denoise != 0u ? vf(denoised + size_t(i) * 4) : c;
                o[0] = srgb(aces(sh.x * P.exposure));
                o[1] = srgb(aces(sh.y * P.exposure));
                o[2] = srgb(aces(sh.z * P.exposure));
            } else if (P.view == 1u) {
                o[0] = srgb(c.x);
                o[1] = srgb(c.y);
                o[2] = srgb(c.z);
            } else if (P.view == 2u) {
                o[0] = c.x * 0.5f + 0.5f;
                o[1] = c.y * 0.5f + 0.5f;
                o[2] = c.z * 0.5f + 0.5f;
            } else {
                const float g = c.x <= 0.0f ? 0.0f : 1.0f / (1.0f + c.x / P.focus_distance);
                o[0] = o[1] = o[2] = g;
            }
        }
        out[i * 4] = byte(o[0]);
        out[i * 4 + 1] = byte(o[1]);
        out[i * 4 + 2] = byte(o[2]);
        out[i * 4 + 3] = 255;
    }
}

// The streams as the product's raymond_sample_streams lays them out: per
// (pixel index, sample index) pair, rand2() then rand() at each dimension id
// of the camera path's stream, its spectrum position, then `chain` draws of
// the light path's and of the gather's PCG chains.
extern "C" void ro_sample_streams(const uint32_t* pairs, uint32_t n, const uint32_t* dim_ids, uint32_t dims,
                                  uint32_t chain, uint32_t seed_hash, float* out) {
    const size_t per = 3u * dims + 1u + 2u * chain;
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t index = pairs[2 * i], sample = pairs[2 * i + 1];
        float* o = out + size_t(i) * per;
        for (uint32_t k = 0; k < dims; ++k) {
            Sampler s = camera_sampler(index, sample, seed_hash);
            s.qmc_dim = dim_ids[k];
            s.rand2(o[3 * k], o[3 * k + 1]);
            s.qmc_dim = dim_ids[k];
            o[3 * k + 2] = s.rand();
        }
        o += 3u * dims;
        *o++ = spectrum_at(index, sample);
        Sampler light = light_sampler(index, sample, seed_hash);
        for (uint32_t k = 0; k < chain; ++k) *o++ = light.rand();
        Sampler gather = gather_sampler(index, sample, seed_hash);
        for (uint32_t k = 0; k < chain; ++k) *o++ = gather.rand();
    }
}

// Sets the perturbation runs' size (0: off, the reference's arithmetic) and seed.
extern "C" void ro_set_jitter(uint32_t seed, float size) {
    g_jitter_seed = seed;
    g_jitter_size = size;
}
