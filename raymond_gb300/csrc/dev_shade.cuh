// Surfaces, materials, lights, sky, media and dispersion for the render
// path, in the f32 arithmetic of the trace shader (src/shaders.mjs:449-1423),
// and the path tracer's bounce as a resumable step: one call consumes one
// closest hit and produces at most one shadow ray and one extension ray, so
// a megakernel loop and the wavefront's shade kernel run the same code with
// the same random-number dimensions per bounce.
#pragma once
#include "dev_trace.cuh"
#include <cuda_fp16.h>

namespace rmd {

constexpr uint32_t F_VOLUMES = 1u, F_TEXTURES = 2u, F_ENVIRONMENT = 4u, F_DISPERSION = 8u;

// sRGB-encoded byte to linear. Without relocatable device code every
// translation unit that includes this header has its own copy, so each one
// fills its own through upload_srgb_table_here() (called by the host at
// start-up, once per device, through that unit's exported uploader).
static __constant__ float c_srgb_to_linear[256];

static inline cudaError_t upload_srgb_table_here() {
    float table[256];
    for (int i = 0; i < 256; ++i) {
        const double c = i / 255.0;
        table[i] = float(c <= 0.04045 ? c / 12.92 : pow((c + 0.055) / 1.055, 2.4));
    }
    return cudaMemcpyToSymbol(c_srgb_to_linear, table, sizeof table);
}

struct Material {
    float3 color;
    uint32_t kind;
    float3 emission;
    float roughness;
    float3 checker;
    float checker_size;
    float ior;
    uint32_t texture;
    float2 texture_scale;
    uint32_t normal_map;
    float normal_scale;
    uint32_t emission_texture;
    float dispersion;
    float density, anisotropy;
};

// Material record (src/shaders.mjs:82-89; offsets src/Scene.mjs:501-521).
__device__ __forceinline__ Material load_material(const Scene& s, uint32_t i) {
    const float4* r = s.materials + size_t(i) * 6;
    const float4 a = ldg4(r), b = ldg4(r + 1), c = ldg4(r + 2), d = ldg4(r + 3), e = ldg4(r + 4), f = ldg4(r + 5);
    Material m;
    m.color = xyz(a);
    m.kind = __float_as_uint(a.w);
    m.emission = xyz(b);
    m.roughness = b.w;
    m.checker = xyz(c);
    m.checker_size = c.w;
    m.ior = d.x;
    m.texture = __float_as_uint(d.y);
    m.texture_scale = make_float2(d.z, d.w);
    m.normal_map = __float_as_uint(e.x);
    m.normal_scale = e.y;
    m.emission_texture = __float_as_uint(e.z);
    m.dispersion = e.w;
    m.density = f.x;
    m.anisotropy = f.y;
    return m;
}
__device__ __forceinline__ uint32_t material_kind(const Scene& s, uint32_t i) {
    return __float_as_uint(__ldg(&s.materials[size_t(i) * 6].w));
}

// ---- textures: bilinear with repeat, as the WebGPU sampler and Texture.sample do ----
__device__ __forceinline__ float3 texel(const uchar4* data, uint32_t w, uint32_t h, uint32_t layer, int x, int y,
                                        bool srgb) {
    const int xi = ((x % int(w)) + int(w)) % int(w);
    const int yi = ((y % int(h)) + int(h)) % int(h);
    const uchar4 t = data[(size_t(layer) * h + yi) * w + xi];
    if (srgb) return f3(c_srgb_to_linear[t.x], c_srgb_to_linear[t.y], c_srgb_to_linear[t.z]);
    return f3(t.x / 255.0f, t.y / 255.0f, t.z / 255.0f);
}
__device__ __forceinline__ float3 sample_texture(const uchar4* data, uint32_t w, uint32_t h, uint32_t layer, float2 uv,
                                                 bool srgb) {
    const float x = uv.x * float(w) - 0.5f, y = uv.y * float(h) - 0.5f;
    const float fx0 = floorf(x), fy0 = floorf(y);
    const float fx = x - fx0, fy = y - fy0;
    const int x0 = int(fx0), y0 = int(fy0);
    return texel(data, w, h, layer, x0, y0, srgb) * ((1.0f - fx) * (1.0f - fy)) +
           texel(data, w, h, layer, x0 + 1, y0, srgb) * (fx * (1.0f - fy)) +
           texel(data, w, h, layer, x0, y0 + 1, srgb) * ((1.0f - fx) * fy) +
           texel(data, w, h, layer, x0 + 1, y0 + 1, srgb) * (fx * fy);
}

// ---- surfaces (src/shaders.mjs:449-605) ----
struct Surface {
    float3 p, n, ng;
    bool front;
    uint32_t material, light, kind;
    float2 uv;
};

// sphere_uv (src/shaders.mjs:573-577).
__device__ __forceinline__ float2 sphere_uv(float3 n, float3 x_axis, float3 north) {
    const float3 z = cross(x_axis, north);
    const float u = atan2f(-dot(n, z), dot(n, x_axis)) / (2.0f * PI);
    return make_float2(u - floorf(u), acosf(clampf(dot(n, north), -1.0f, 1.0f)) / PI);
}

// bump (src/shaders.mjs:582-594).
__device__ __forceinline__ float3 bump(float3 n, float3 ng, float3 tangent, float3 up, float3 t, float strength) {
    float3 right = tangent - n * dot(n, tangent);
    if (length(right) < 1e-9f) return n;
    right = normalize(right);
    float3 above = cross(n, right);
    if (dot(above, up) < 0.0f) above = -above;
    const float3 tilted = normalize(right * ((t.x * 2.0f - 1.0f) * strength) + above * ((t.y * 2.0f - 1.0f) * strength) +
                                    n * (t.z * 2.0f - 1.0f));
    return dot(tilted, ng) > 0.0f ? tilted : n;
}

template <uint32_t FEAT>
__device__ Surface surface_at(const Scene& s, float3 o, float3 d, const Hit& hit) {
    const float4* rec = s.prims + size_t(hit.prim) * 4;
    const float4 hdr = ldg4(rec), p0 = ldg4(rec + 1), p1 = ldg4(rec + 2), p2 = ldg4(rec + 3);
    const uint32_t kind = __float_as_uint(hdr.x);
    const uint32_t material = __float_as_uint(hdr.y);
    const uint32_t light = __float_as_uint(hdr.z);
    const uint32_t attrs = __float_as_uint(hdr.w);
    const float3 point = o + d * hit.t;
    float3 ng, ns, tangent = f3(1.0f, 0.0f, 0.0f), up = f3(0.0f, 1.0f, 0.0f);
    float2 uv;
    if (kind == SPHERE) {
        ng = normalize(point - xyz(p0));
        ns = ng;
        uv = sphere_uv(ng, xyz(p1), xyz(p2));
        if (FEAT & F_TEXTURES) {
            tangent = cross(xyz(p2), ng);
            if (length(tangent) < 1e-6f) tangent = xyz(p1);
            up = cross(ng, tangent);
        }
    } else if (kind == QUAD) {
        ng = normalize(cross(xyz(p1), xyz(p2)));
        ns = ng;
        uv = make_float2(hit.u, 1.0f - hit.v);
        tangent = xyz(p1);
        up = xyz(p2);
    } else if (kind == BOX) {
        const float3 lp = f3(dot(xyz(p0), point) + p0.w, dot(xyz(p1), point) + p1.w, dot(xyz(p2), point) + p2.w);
        const float3 a = f3(fabsf(lp.x), fabsf(lp.y), fabsf(lp.z));
        const float3 half = f3(1.0f / length(xyz(p0)), 1.0f / length(xyz(p1)), 1.0f / length(xyz(p2)));
        if (a.x >= a.y && a.x >= a.z) {
            ng = xyz(p0) * signf(lp.x);
            uv = make_float2((1.0f - signf(lp.x) * lp.z) * half.z, (1.0f - lp.y) * half.y);
            tangent = xyz(p2) * -signf(lp.x);
            up = xyz(p1);
        } else if (a.y >= a.z) {
            ng = xyz(p1) * signf(lp.y);
            uv = make_float2((1.0f + lp.x) * half.x, (1.0f + signf(lp.y) * lp.z) * half.z);
            tangent = xyz(p0);
            up = xyz(p2) * -signf(lp.y);
        } else {
            ng = xyz(p2) * signf(lp.z);
            uv = make_float2((1.0f + signf(lp.z) * lp.x) * half.x, (1.0f - lp.y) * half.y);
            tangent = xyz(p0) * signf(lp.z);
            up = xyz(p1);
        }
        ng = normalize(ng);
        ns = ng;
    } else {
        const float3 e1 = xyz(p1) - xyz(p0);
        const float3 e2 = xyz(p2) - xyz(p0);
        ng = normalize(cross(e1, e2));
        ns = ng;
        uv = make_float2(hit.u, hit.v);
        float2 du1 = make_float2(1.0f, 0.0f), du2 = make_float2(0.0f, 1.0f);
        if (attrs != NONE) {
            const float w = 1.0f - hit.u - hit.v;
            const float4* ab = s.attributes + size_t(attrs);
            const float4 a0 = ldg4(ab), a1 = ldg4(ab + 1), a2 = ldg4(ab + 2), vs = ldg4(ab + 3);
            const uint32_t flags = uint32_t(vs.w);
            if (flags & 1u) {
                ns = normalize(xyz(a0) * w + xyz(a1) * hit.u + xyz(a2) * hit.v);
                if (dot(ns, ng) < 0.0f) ns = -ns;
            }
            if (flags & 2u) {
                uv = make_float2(a0.w * w + a1.w * hit.u + a2.w * hit.v, vs.x * w + vs.y * hit.u + vs.z * hit.v);
                const float2 t1 = make_float2(a1.w - a0.w, vs.y - vs.x);
                const float2 t2 = make_float2(a2.w - a0.w, vs.z - vs.x);
                if (fabsf(t1.x * t2.y - t2.x * t1.y) > 1e-12f) {
                    du1 = t1;
                    du2 = t2;
                }
            }
        }
        if (FEAT & F_TEXTURES) {
            const float det = du1.x * du2.y - du2.x * du1.y;
            tangent = (e1 * du2.y - e2 * du1.y) / det;
            up = -(e2 * du1.x - e1 * du2.x) / det;
        }
    }
    if (FEAT & F_TEXTURES) {
        const float4 e = ldg4(s.materials + size_t(material) * 6 + 4);
        const uint32_t nm = __float_as_uint(e.x);
        if (nm != NONE) {
            const float4 dd = ldg4(s.materials + size_t(material) * 6 + 3);
            const float3 t = sample_texture(s.normal_maps, s.nrm_w, s.nrm_h, nm,
                                            make_float2(uv.x * dd.z, uv.y * dd.w), false);
            ns = bump(ns, ng, tangent, up, t, e.y);
        }
    }
    const bool front = dot(ng, d) < 0.0f;
    const float flip = front ? 1.0f : -1.0f;
    Surface sf;
    sf.p = point;
    sf.n = ns * flip;
    sf.ng = ng * flip;
    sf.front = front;
    sf.material = material;
    sf.light = light;
    sf.kind = kind;
    sf.uv = uv;
    return sf;
}

// offset (src/shaders.mjs:602-605).
__device__ __forceinline__ float3 offset_origin(const Surface& sf, float3 wi) {
    const float eps = 1e-4f * fmaxf(1.0f, fmaxf(fabsf(sf.p.x), fmaxf(fabsf(sf.p.y), fabsf(sf.p.z))));
    return sf.p + sf.ng * (dot(wi, sf.ng) > 0.0f ? eps : -eps);
}

// ---- sky and environment (src/shaders.mjs:611-687) ----
__device__ __forceinline__ float2 env_uv(const Params& P, float3 d) {
    const float u = 0.5f + atan2f(d.x, -d.z) / (2.0f * PI) - P.env_rotation / (2.0f * PI);
    return make_float2(u - floorf(u), acosf(clampf(d.y, -1.0f, 1.0f)) / PI);
}
// Bilinear, repeating round the horizon and clamped at the poles.
__device__ __forceinline__ float3 env_texel(const Scene& s, int x, int y) {
    const int w = int(s.env_w), h = int(s.env_h);
    const int xi = ((x % w) + w) % w;
    const int yi = y < 0 ? 0 : (y >= h ? h - 1 : y);
    const ushort4 t = s.env_map[size_t(yi) * w + xi];
    return f3(__half2float(__ushort_as_half(t.x)), __half2float(__ushort_as_half(t.y)),
              __half2float(__ushort_as_half(t.z)));
}
__device__ __forceinline__ float3 env_radiance(const Scene& s, const Params& P, float3 d) {
    const float2 uv = env_uv(P, d);
    const float x = uv.x * float(s.env_w) - 0.5f, y = uv.y * float(s.env_h) - 0.5f;
    const float fx0 = floorf(x), fy0 = floorf(y);
    const float fx = x - fx0, fy = y - fy0;
    const int x0 = int(fx0), y0 = int(fy0);
    const float3 c = env_texel(s, x0, y0) * ((1.0f - fx) * (1.0f - fy)) + env_texel(s, x0 + 1, y0) * (fx * (1.0f - fy)) +
                     env_texel(s, x0, y0 + 1) * ((1.0f - fx) * fy) + env_texel(s, x0 + 1, y0 + 1) * (fx * fy);
    return c * P.env_strength;
}
__device__ __forceinline__ float env_cdf(const Scene& s, uint32_t x, uint32_t y) { return s.env_table[size_t(y) * s.env_cw + x]; }
__device__ __forceinline__ uint32_t env_search(const Scene& s, uint32_t y, uint32_t n, float xi) {
    uint32_t lo = 0u, hi = n - 1u;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) / 2u;
        if (env_cdf(s, mid, y) > xi) hi = mid;
        else lo = mid + 1u;
    }
    return lo;
}
__device__ __forceinline__ float env_pdf(const Scene& s, const Params& P, float3 d) {
    const uint32_t cw = s.env_cw, ch = s.env_ch;
    const float2 uv = env_uv(P, d);
    const uint32_t x = min(uint32_t(uv.x * float(cw)), cw - 1u);
    const uint32_t y = min(uint32_t(uv.y * float(ch)), ch - 1u);
    const float row = env_cdf(s, y, ch) - (y > 0u ? env_cdf(s, y - 1u, ch) : 0.0f);
    const float cell = env_cdf(s, x, y) - (x > 0u ? env_cdf(s, x - 1u, y) : 0.0f);
    const float sn = sinf(uv.y * PI);
    return sn > 0.0f ? row * cell * float(cw * ch) / (2.0f * PI * PI * sn) : 0.0f;
}
__device__ __forceinline__ float3 sample_env(const Scene& s, const Params& P, Rng& rng) {
    const uint32_t cw = s.env_cw, ch = s.env_ch;
    const float2 cell = rng.rand2();
    const uint32_t y = env_search(s, ch, ch, cell.y);
    const uint32_t x = env_search(s, y, cw, cell.x);
    const float2 within = rng.rand2();
    const float u = (float(x) + within.x) / float(cw) + P.env_rotation / (2.0f * PI);
    const float v = (float(y) + within.y) / float(ch);
    const float phi = (u - 0.5f) * 2.0f * PI;
    const float theta = v * PI;
    return f3(sinf(theta) * sinf(phi), cosf(theta), -sinf(theta) * cosf(phi));
}
template <uint32_t FEAT>
__device__ __forceinline__ bool env_on(const Params& P) { return (FEAT & F_ENVIRONMENT) && P.env_strength > 0.0f; }

template <uint32_t FEAT>
__device__ __forceinline__ float3 sky(const Scene& s, const Params& P, float3 d) {
    if (env_on<FEAT>(P)) return env_radiance(s, P, d);
    if (d.y >= 0.0f) return mix3(f3(P.sky_horizon), f3(P.sky_zenith), sqrtf(fminf(d.y, 1.0f)));
    return mix3(f3(P.sky_horizon), f3(P.sky_ground), sqrtf(fminf(-d.y, 1.0f)));
}
__device__ __forceinline__ bool in_sun(const Params& P, float3 d) {
    return P.sun_on != 0u && dot(d, f3(P.sun_dir)) >= 1.0f - P.sun_omc;
}

// ---- materials (src/shaders.mjs:693-871) ----
template <uint32_t FEAT>
__device__ __forceinline__ float3 albedo(const Scene& s, const Material& m, float3 p, float2 uv) {
    float3 c = m.color;
    if (m.checker_size > 0.0f) {
        const float3 cell = f3(floorf(p.x / m.checker_size + 1e-3f), floorf(p.y / m.checker_size + 1e-3f),
                               floorf(p.z / m.checker_size + 1e-3f));
        const int odd = (int(cell.x) + int(cell.y) + int(cell.z)) & 1;
        c = odd != 0 ? m.checker : m.color;
    }
    if ((FEAT & F_TEXTURES) && m.texture != NONE)
        c *= sample_texture(s.textures, s.tex_w, s.tex_h, m.texture,
                            make_float2(uv.x * m.texture_scale.x, uv.y * m.texture_scale.y), true);
    return c;
}
template <uint32_t FEAT>
__device__ __forceinline__ float3 emitted(const Scene& s, const Material& m, float2 uv) {
    if (!(FEAT & F_TEXTURES) || m.emission_texture == NONE) return m.emission;
    return m.emission * sample_texture(s.textures, s.tex_w, s.tex_h, m.emission_texture,
                                       make_float2(uv.x * m.texture_scale.x, uv.y * m.texture_scale.y), true);
}
__device__ __forceinline__ bool is_delta(const Material& m) {
    return m.kind == GLASS || (m.kind == METAL && m.roughness < 0.01f);
}
__device__ __forceinline__ float ggx_alpha2(float roughness) {
    const float alpha = fmaxf(roughness * roughness, 0.002f);
    return alpha * alpha;
}
__device__ __forceinline__ float ggx_d(float nh, float a2) {
    const float k = nh * nh * (a2 - 1.0f) + 1.0f;
    return a2 / (PI * k * k);
}
__device__ __forceinline__ float smith_g1(float nv, float a2) {
    return 2.0f * nv / (nv + sqrtf(a2 + (1.0f - a2) * nv * nv));
}
__device__ __forceinline__ float3 sample_ggx(float3 n, float a2, Rng& rng) {
    const float2 u = rng.rand2();
    const float r = u.x;
    const float cos_t = sqrtf((1.0f - r) / (1.0f + (a2 - 1.0f) * r));
    const float sin_t = sqrtf(fmaxf(0.0f, one_minus_sq(cos_t)));
    const float phi = 2.0f * PI * u.y;
    float sn, cs;
    sincosf(phi, &sn, &cs);
    return normalize(from_frame(n, f3(sin_t * cs, sin_t * sn, cos_t)));
}
__device__ __forceinline__ float schlick1(float f0, float c) {
    return f0 + (1.0f - f0) * powf(1.0f - clampf(c, 0.0f, 1.0f), 5.0f);
}
__device__ __forceinline__ float3 schlick3(float3 f0, float c) {
    const float k = powf(1.0f - clampf(c, 0.0f, 1.0f), 5.0f);
    return f0 + (f3(1.0f) - f0) * k;
}
__device__ __forceinline__ float dielectric_f0(float ior) {
    const float r = (ior - 1.0f) / (ior + 1.0f);
    return r * r;
}
__device__ __forceinline__ float fresnel_dielectric(float cos_i, float eta) {
    const float sin2_t = one_minus_sq(cos_i) / (eta * eta);
    if (sin2_t >= 1.0f) return 1.0f;
    const float cos_t = sqrtf(1.0f - sin2_t);
    const float rs = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
    const float rp = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
    return 0.5f * (rs * rs + rp * rp);
}
__device__ __forceinline__ float plastic_spec_chance(const Material& m, float nv) {
    return clampf(schlick1(dielectric_f0(m.ior), nv) * 4.0f + 0.1f, 0.1f, 0.9f);
}

struct Eval {
    float3 f;  // BSDF × cos(n, wi)
    float pdf;
};
__device__ __forceinline__ Eval eval_bsdf(const Material& m, float3 base, float3 n, float3 wo, float3 wi) {
    const float nl = dot(n, wi), nv = dot(n, wo);
    if (nl <= 0.0f || nv <= 0.0f) return Eval{f3(0.0f), 0.0f};
    if (m.kind == DIFFUSE) return Eval{base * (nl / PI), nl / PI};
    const float a2 = ggx_alpha2(m.roughness);
    const float3 h = normalize(wo + wi);
    const float nh = fmaxf(dot(n, h), 0.0f);
    const float vh = fmaxf(dot(wo, h), 1e-6f);
    const float d = ggx_d(nh, a2);
    const float g = smith_g1(nv, a2) * smith_g1(nl, a2);
    const float spec_pdf = d * nh / (4.0f * vh);
    if (m.kind == METAL) return Eval{schlick3(base, vh) * (d * g / (4.0f * nv)), spec_pdf};
    const float f0 = dielectric_f0(m.ior);
    const float coat = schlick1(f0, vh) * d * g / (4.0f * nv);
    const float through = (1.0f - schlick1(f0, nl)) * (1.0f - schlick1(f0, nv));
    const float3 diffuse = base * (through * nl / PI);
    const float chance = plastic_spec_chance(m, nv);
    return Eval{f3(coat) + diffuse, chance * spec_pdf + (1.0f - chance) * nl / PI};
}

struct BsdfSample {
    float3 wi, weight;
    float pdf;
    bool delta, ok;
};
__device__ __forceinline__ BsdfSample sample_bsdf(const Material& m, float3 base, const Surface& sf, float3 wo, Rng& rng) {
    const BsdfSample fail{f3(0.0f), f3(0.0f), 0.0f, false, false};
    const float3 n = sf.n;
    const float nv = dot(n, wo);
    if (m.kind == GLASS) {
        const float eta = sf.front ? m.ior : 1.0f / m.ior;
        const float cos_i = clampf(nv, 0.0f, 1.0f);
        const float f = fresnel_dielectric(cos_i, eta);
        if (rng.rand() < f) return BsdfSample{reflect3(-wo, n), f3(1.0f), 0.0f, true, true};
        const float3 wi = refract3(-wo, n, 1.0f / eta);
        if (dot(wi, wi) == 0.0f) return BsdfSample{reflect3(-wo, n), f3(1.0f), 0.0f, true, true};
        return BsdfSample{normalize(wi), sf.front ? base : f3(1.0f), 0.0f, true, true};
    }
    if (m.kind == METAL && m.roughness < 0.01f) return BsdfSample{reflect3(-wo, n), schlick3(base, nv), 0.0f, true, true};
    float3 wi;
    if (m.kind == DIFFUSE) {
        wi = cosine_hemisphere(n, rng);
    } else if (m.kind == METAL || rng.rand() < plastic_spec_chance(m, nv)) {
        const float3 h = sample_ggx(n, ggx_alpha2(m.roughness), rng);
        wi = reflect3(-wo, h);
    } else {
        wi = cosine_hemisphere(n, rng);
    }
    if (dot(wi, sf.ng) <= 0.0f) return fail;
    const Eval e = eval_bsdf(m, base, n, wo, wi);
    if (e.pdf <= 0.0f) return fail;
    return BsdfSample{wi, e.f / e.pdf, e.pdf, false, true};
}

// ---- lights (src/shaders.mjs:877-1018) ----
template <uint32_t FEAT>
__device__ __forceinline__ uint32_t light_choices(const Params& P) {
    return P.light_count + (P.sun_on != 0u ? 1u : 0u) + (env_on<FEAT>(P) ? 1u : 0u);
}
__device__ __forceinline__ float light_cdf(const Scene& s, const Params& P, uint32_t l) {
    return __uint_as_float(s.lights[P.light_count + P.volume_count + l]);
}
template <uint32_t FEAT>
__device__ __forceinline__ float light_chance(const Scene& s, const Params& P, uint32_t l) {
    const float below = l > 0u ? light_cdf(s, P, l - 1u) : 0.0f;
    return (light_cdf(s, P, l) - below) * float(P.light_count) / float(light_choices<FEAT>(P));
}
__device__ __forceinline__ uint32_t pick_light(const Scene& s, const Params& P, float u) {
    uint32_t lo = 0u, hi = P.light_count - 1u;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) / 2u;
        if (light_cdf(s, P, mid) > u) hi = mid;
        else lo = mid + 1u;
    }
    return lo;
}
__device__ __forceinline__ float sphere_omc(float r, float d2) {
    const float x = fminf(r * r / d2, 1.0f);
    return x / (1.0f + sqrtf(1.0f - x));
}
__device__ __forceinline__ float power_heuristic(float a, float b) {
    const float a2 = a * a, b2 = b * b;
    if (a2 + b2 <= 0.0f) return 0.0f;
    return a2 / (a2 + b2);
}

struct LightSample {
    float3 wi;
    float dist;
    float3 radiance;
    float pdf;
};

template <uint32_t FEAT>
__device__ LightSample sample_light(const Scene& s, const Params& P, float3 p, Rng& rng) {
    const LightSample none{f3(0.0f), 0.0f, f3(0.0f), 0.0f};
    const uint32_t choices = light_choices<FEAT>(P);
    const float x = rng.rand() * float(choices);
    uint32_t pick = min(uint32_t(x), choices - 1u);
    float chance = 1.0f / float(choices);
    const uint32_t sun_choice = P.sun_on != 0u ? P.light_count : NONE;
    const uint32_t env_choice = env_on<FEAT>(P) ? P.light_count + (P.sun_on != 0u ? 1u : 0u) : NONE;

    if ((FEAT & F_ENVIRONMENT) && pick == env_choice) {
        const float3 wi = sample_env(s, P, rng);
        const float pdf = env_pdf(s, P, wi);
        if (pdf <= 0.0f) return none;
        return LightSample{wi, INF, env_radiance(s, P, wi), chance * pdf};
    }
    if (pick == sun_choice) {
        const float3 wi = sample_cone(f3(P.sun_dir), P.sun_omc, rng);
        return LightSample{wi, INF, f3(P.sun_radiance), chance / (2.0f * PI * P.sun_omc)};
    }
    pick = pick_light(s, P, x / float(P.light_count));
    chance = light_chance<FEAT>(s, P, pick);
    const uint32_t pi = s.lights[pick];
    const float4* rec = s.prims + size_t(pi) * 4;
    const float4 hdr = ldg4(rec), p0 = ldg4(rec + 1), p1 = ldg4(rec + 2), p2 = ldg4(rec + 3);
    const Material m = load_material(s, __float_as_uint(hdr.y));
    if (__float_as_uint(hdr.x) == QUAD) {
        const float2 ab = rng.rand2();
        const float3 q = xyz(p0) + xyz(p1) * ab.x + xyz(p2) * ab.y;
        const float3 to = q - p;
        const float d2 = dot(to, to);
        const float dist = sqrtf(d2);
        const float3 wi = to / dist;
        const float3 c = cross(xyz(p1), xyz(p2));
        const float area = length(c);
        const float cos_l = -dot(wi, c / area);
        if (cos_l <= 0.0f) return none;
        return LightSample{wi, dist, emitted<FEAT>(s, m, make_float2(ab.x, 1.0f - ab.y)), chance * d2 / (cos_l * area)};
    }
    const float3 to = xyz(p0) - p;
    const float d2 = dot(to, to);
    const float r = p0.w;
    if (d2 <= r * r) return none;
    const float omc = sphere_omc(r, d2);
    const float3 wi = sample_cone(to / sqrtf(d2), omc, rng);
    const float b = dot(to, wi);
    const float dist = b - sqrtf(fmaxf(b * b - (d2 - r * r), 0.0f));
    const float3 n = normalize(p + wi * dist - xyz(p0));
    return LightSample{wi, dist, emitted<FEAT>(s, m, sphere_uv(n, xyz(p1), xyz(p2))), chance / (2.0f * PI * omc)};
}

template <uint32_t FEAT>
__device__ __forceinline__ float light_pdf(const Scene& s, const Params& P, uint32_t prim_index, float3 p, float3 wi,
                                           float t) {
    const float4* rec = s.prims + size_t(prim_index) * 4;
    const float4 hdr = ldg4(rec), p0 = ldg4(rec + 1);
    const float chance = light_chance<FEAT>(s, P, __float_as_uint(hdr.z));
    if (__float_as_uint(hdr.x) == QUAD) {
        const float3 c = cross(xyz(ldg4(rec + 2)), xyz(ldg4(rec + 3)));
        const float area = length(c);
        const float cos_l = fabsf(dot(wi, c / area));
        return chance * t * t / fmaxf(cos_l * area, 1e-12f);
    }
    const float3 to = xyz(p0) - p;
    const float omc = sphere_omc(p0.w, dot(to, to));
    return chance / (2.0f * PI * omc);
}

// ---- participating media (src/shaders.mjs:1024-1123) ----
__device__ __forceinline__ float2 volume_span(const Scene& s, uint32_t i, float3 o, float3 d) {
    const float4* rec = s.prims + size_t(i) * 4;
    const float4 hdr = ldg4(rec), p0 = ldg4(rec + 1);
    if (__float_as_uint(hdr.x) == SPHERE) {
        const float3 oc = o - xyz(p0);
        const float a = dot(d, d);
        const float half_b = dot(oc, d);
        const float disc = half_b * half_b - a * (dot(oc, oc) - p0.w * p0.w);
        if (disc < 0.0f) return make_float2(1.0f, 0.0f);
        const float sq = sqrtf(disc);
        return make_float2(fmaxf((-half_b - sq) / a, 0.0f), (-half_b + sq) / a);
    }
    const float4 p1 = ldg4(rec + 2), p2 = ldg4(rec + 3);
    const float3 lo = f3(dot(xyz(p0), o) + p0.w, dot(xyz(p1), o) + p1.w, dot(xyz(p2), o) + p2.w);
    const float3 inv = f3(1.0f / safe1(dot(xyz(p0), d)), 1.0f / safe1(dot(xyz(p1), d)), 1.0f / safe1(dot(xyz(p2), d)));
    const float3 t0 = (f3(-1.0f) - lo) * inv, t1 = (f3(1.0f) - lo) * inv;
    const float3 tmn = fmin3(t0, t1), tmx = fmax3(t0, t1);
    return make_float2(fmaxf(fmaxf(fmaxf(tmn.x, tmn.y), tmn.z), 0.0f), fminf(fminf(tmx.x, tmx.y), tmx.z));
}
struct Scatter {
    float t;
    uint32_t volume;
};
template <uint32_t FEAT>
__device__ __forceinline__ Scatter scatter_in_volumes(const Scene& s, const Params& P, float3 o, float3 d, float t_max,
                                                      Rng& rng) {
    Scatter sc{t_max, NONE};
    if constexpr (!(FEAT & F_VOLUMES)) {
        return sc;
    } else {
        for (uint32_t k = 0; k < P.volume_count; ++k) {
            const uint32_t i = s.lights[P.light_count + k];
            const float2 span = volume_span(s, i, o, d);
            const float end = fminf(span.y, sc.t);
            if (span.x < end) {
                const uint32_t mat = __float_as_uint(ldg4(s.prims + size_t(i) * 4).y);
                const float density = __ldg(&s.materials[size_t(mat) * 6 + 5].x);
                const float t = span.x - logf(1.0f - rng.rand()) / density;
                if (t < end) sc = Scatter{t, i};
            }
        }
        return sc;
    }
}
template <uint32_t FEAT>
__device__ __forceinline__ float transmittance(const Scene& s, const Params& P, float3 o, float3 d, float dist) {
    if (!(FEAT & F_VOLUMES)) return 1.0f;
    float depth = 0.0f;
    for (uint32_t k = 0; k < P.volume_count; ++k) {
        const uint32_t i = s.lights[P.light_count + k];
        const float2 span = volume_span(s, i, o, d);
        const float end = fminf(span.y, dist);
        if (span.x < end) {
            const uint32_t mat = __float_as_uint(ldg4(s.prims + size_t(i) * 4).y);
            depth += __ldg(&s.materials[size_t(mat) * 6 + 5].x) * (end - span.x);
        }
    }
    return expf(-depth);
}
__device__ __forceinline__ float henyey_greenstein(float c, float g) {
    const float k = 1.0f + g * g - 2.0f * g * c;
    return (1.0f - g * g) / (4.0f * PI * k * sqrtf(k));
}
__device__ __forceinline__ float3 sample_henyey_greenstein(float3 d, float g, Rng& rng) {
    const float2 u = rng.rand2();
    float c = 1.0f - 2.0f * u.x;
    if (fabsf(g) >= 1e-3f) {
        const float sq = (1.0f - g * g) / (1.0f + g - 2.0f * g * u.x);
        c = clampf((1.0f + g * g - sq * sq) / (2.0f * g), -1.0f, 1.0f);
    }
    const float sin_t = sqrtf(fmaxf(0.0f, one_minus_sq(c)));
    const float phi = 2.0f * PI * u.y;
    float sn, cs;
    sincosf(phi, &sn, &cs);
    return normalize(from_frame(d, f3(sin_t * cs, sin_t * sn, c)));
}

// ---- dispersion (src/shaders.mjs:1127-1144, 1412-1423) ----
__device__ __forceinline__ float lobe(float x, float mu, float below, float above) {
    const float t = (x - mu) / (x < mu ? below : above);
    return expf(-0.5f * t * t);
}
// Wyman, Sloan and Shirley's analytic fit to the CIE 1931 matching
// functions, to linear sRGB, scaled so 380–720 nm averages to white.
__device__ __forceinline__ float3 wavelength_rgb(float l) {
    const float x = 1.056f * lobe(l, 599.8f, 37.9f, 31.0f) + 0.362f * lobe(l, 442.0f, 16.0f, 26.7f) -
                    0.065f * lobe(l, 501.1f, 20.4f, 26.2f);
    const float y = 0.821f * lobe(l, 568.8f, 46.9f, 40.5f) + 0.286f * lobe(l, 530.9f, 16.3f, 31.1f);
    const float z = 1.217f * lobe(l, 437.0f, 11.8f, 36.0f) + 0.681f * lobe(l, 459.0f, 26.0f, 13.8f);
    const float3 rgb = f3(3.2406f * x - 1.5372f * y - 0.4986f * z, -0.9689f * x + 1.8758f * y + 0.0415f * z,
                          0.0557f * x - 0.2040f * y + 1.0570f * z);
    return fmax3(rgb, f3(0.0f)) * f3(1.92985f, 2.94689f, 3.11081f);
}
template <uint32_t FEAT>
__device__ __forceinline__ Material dispersed(const Material& m, float& wavelength, float3& throughput, float u) {
    Material sm = m;
    if ((FEAT & F_DISPERSION) && m.kind == GLASS && m.dispersion > 0.0f) {
        if (wavelength == 0.0f) {
            wavelength = 380.0f + 340.0f * u;
            throughput *= wavelength_rgb(wavelength);
        }
        const float l = wavelength * 1e-3f;
        sm.ior = m.ior + m.dispersion * (1.0f / (l * l) - 1.0f / (0.5876f * 0.5876f));
    }
    return sm;
}

// camera_ray (src/shaders.mjs:1148-1166).
__device__ __forceinline__ void camera_ray(const Params& P, float2 px, bool jitter, Rng& rng, float3& o, float3& d) {
    const float ndcx = 2.0f * px.x / float(P.width) - 1.0f;
    const float ndcy = 1.0f - 2.0f * px.y / float(P.height);
    const float3 fwd = f3(P.cam_forward), right = f3(P.cam_right), up = f3(P.cam_up), pos = f3(P.cam_pos);
    const float3 dir = normalize(fwd + right * (ndcx * P.tan_half_fov * P.aspect) + up * (ndcy * P.tan_half_fov));
    if (!jitter || P.lens_radius <= 0.0f) {
        o = pos;
        d = dir;
        return;
    }
    const float3 focus = pos + dir * (P.focus_distance / dot(dir, fwd));
    const float2 lens = concentric_disk(rng);
    o = pos + right * (lens.x * P.lens_radius) + up * (lens.y * P.lens_radius);
    d = normalize(focus - o);
}

// ---- one camera path as a resumable state (radiance(), src/shaders.mjs:1179-1374) ----
enum : uint32_t { PF_LAST_DELTA = 1u, PF_CAUSTIC = 2u, PF_DIFFUSE_SEEN = 4u, PF_GUIDED = 8u };

struct PathState {
    float3 o, d;
    float3 throughput;
    float3 result;
    float3 last_p;
    float last_pdf;
    float wavelength;
    float travelled;
    float spectrum_u;
    float3 g_albedo;
    float4 g_normal;
    uint32_t depth;
    uint32_t flags;
    Rng rng;
};

struct ShadowRay {
    float3 o, d;
    float reach;
    float3 contribution;
    bool valid;
};

// Per-sample seeding of main() (src/shaders.mjs:1852-1859) and the first
// part of radiance(): the jittered camera ray. seed_hash is 0 for the
// reference's streams.
__device__ __forceinline__ void path_begin(const Params& P, uint32_t seed_hash, uint32_t x, uint32_t y, uint32_t k,
                                           PathState& ps) {
    const uint32_t index = y * P.width + x;
    const uint32_t sample = P.sample_offset + k;
    ps.rng = camera_rng(index, sample, seed_hash);
    ps.spectrum_u = spectrum_position(index, sample);
    const float2 j = ps.rng.rand2();
    ps.g_albedo = f3(1.0f);
    ps.g_normal = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    ps.travelled = 0.0f;
    camera_ray(P, make_float2(float(x) + j.x, float(y) + j.y), true, ps.rng, ps.o, ps.d);
    ps.throughput = f3(1.0f);
    ps.result = f3(0.0f);
    ps.last_pdf = 0.0f;
    ps.last_p = ps.o;
    ps.wavelength = 0.0f;
    ps.depth = 0u;
    ps.flags = PF_LAST_DELTA;
}

// roulette (src/shaders.mjs:1363-1374).
__device__ __forceinline__ bool roulette(float3& throughput, uint32_t depth, Rng& rng) {
    if (depth < 3u) return true;
    const float survive = fminf(maxc(throughput), 0.95f);
    if (rng.rand() >= survive) return false;
    throughput = throughput / survive;
    return true;
}

// One bounce of radiance()'s loop body, given the nearest hit along
// (ps.o, ps.d). Returns true when the path continues with the new ray in
// ps; a shadow ray, if any, is left in sh with the light it adds if
// unoccluded.
template <uint32_t FEAT>
__device__ bool path_step(const Scene& s, const Params& P, PathState& ps, const Hit& hit, ShadowRay& sh) {
    sh.valid = false;
    ps.rng.dim = (ps.depth + 1u) << 16u;
    const uint32_t choices = light_choices<FEAT>(P);
    const float3 d = ps.d;

    if (FEAT & F_VOLUMES) {
        const Scatter sc = scatter_in_volumes<FEAT>(s, P, ps.o, d, hit.t, ps.rng);
        if (sc.volume != NONE) {
            const Material vm = load_material(s, __float_as_uint(ldg4(s.prims + size_t(sc.volume) * 4).y));
            const float3 p = ps.o + d * sc.t;
            ps.travelled += sc.t;
            if (!(ps.flags & PF_GUIDED)) {
                ps.flags |= PF_GUIDED;
                ps.g_albedo = ps.throughput * vm.color;
                ps.g_normal = make_float4(-d.x, -d.y, -d.z, ps.travelled);
            }
            if (ps.depth == P.max_bounces) return false;
            ps.throughput *= vm.color;
            if (choices > 0u) {
                const LightSample ls = sample_light<FEAT>(s, P, p, ps.rng);
                if (ls.pdf > 0.0f) {
                    const float phase = henyey_greenstein(dot(d, ls.wi), vm.anisotropy);
                    const float reach = ls.dist * (1.0f - 1e-3f);
                    sh.o = p;
                    sh.d = ls.wi;
                    sh.reach = reach;
                    sh.contribution = ps.throughput * ls.radiance *
                                      (phase * transmittance<FEAT>(s, P, p, ls.wi, reach) *
                                       power_heuristic(ls.pdf, phase) / ls.pdf);
                    sh.valid = true;
                }
            }
            const float3 wi = sample_henyey_greenstein(d, vm.anisotropy, ps.rng);
            ps.last_pdf = henyey_greenstein(dot(d, wi), vm.anisotropy);
            ps.flags &= ~(PF_LAST_DELTA | PF_CAUSTIC);
            ps.flags |= PF_DIFFUSE_SEEN;
            ps.last_p = p;
            ps.o = p;
            ps.d = wi;
            if (!roulette(ps.throughput, ps.depth, ps.rng)) return false;
            ps.depth++;
            return true;
        }
    }

    const bool last_delta = (ps.flags & PF_LAST_DELTA) != 0u;
    const bool caustic = (ps.flags & PF_CAUSTIC) != 0u;

    if (hit.prim == NONE) {
        if (!(ps.flags & PF_GUIDED)) ps.g_albedo = ps.throughput;
        float sky_weight = 1.0f;
        if (env_on<FEAT>(P) && !last_delta) sky_weight = power_heuristic(ps.last_pdf, env_pdf(s, P, d) / float(choices));
        ps.result += ps.throughput * sky<FEAT>(s, P, d) * sky_weight;
        if (in_sun(P, d) && !(caustic && last_delta)) {
            float w = 1.0f;
            if (!last_delta) w = power_heuristic(ps.last_pdf, 1.0f / (float(choices) * 2.0f * PI * P.sun_omc));
            ps.result += ps.throughput * f3(P.sun_radiance) * w;
        }
        return false;
    }

    const Surface sf = surface_at<FEAT>(s, ps.o, d, hit);
    const Material m = load_material(s, sf.material);
    ps.travelled += hit.t;
    const bool delta = is_delta(m);

    if (!(ps.flags & PF_GUIDED) && (m.kind == LIGHT || !delta || ps.depth == P.max_bounces)) {
        ps.flags |= PF_GUIDED;
        ps.g_albedo = ps.throughput * (m.kind == LIGHT ? f3(1.0f) : albedo<FEAT>(s, m, sf.p, sf.uv));
        ps.g_normal = make_float4(sf.n.x, sf.n.y, sf.n.z, ps.travelled);
    }

    if (sf.front && (m.emission.x > 0.0f || m.emission.y > 0.0f || m.emission.z > 0.0f) &&
        !(caustic && last_delta && sf.light != NONE)) {
        float w = 1.0f;
        if (!last_delta && sf.light != NONE)
            w = power_heuristic(ps.last_pdf, light_pdf<FEAT>(s, P, hit.prim, ps.last_p, d, hit.t));
        ps.result += ps.throughput * emitted<FEAT>(s, m, sf.uv) * w;
    }

    if (m.kind == LIGHT) return false;

    if (!delta) {
        if (P.caustics != 0u && !(ps.flags & PF_DIFFUSE_SEEN)) ps.flags |= PF_CAUSTIC;
        else ps.flags &= ~PF_CAUSTIC;
        ps.flags |= PF_DIFFUSE_SEEN;
    }

    if (ps.depth == P.max_bounces) return false;

    const float3 base = albedo<FEAT>(s, m, sf.p, sf.uv);
    const float3 wo = -d;

    if (!delta && choices > 0u) {
        const LightSample ls = sample_light<FEAT>(s, P, sf.p, ps.rng);
        if (ls.pdf > 0.0f && dot(ls.wi, sf.ng) > 0.0f) {
            const Eval e = eval_bsdf(m, base, sf.n, wo, ls.wi);
            const float3 origin = offset_origin(sf, ls.wi);
            const float reach = (ls.dist - dot(origin - sf.p, ls.wi)) * (1.0f - 1e-3f);
            if (e.pdf > 0.0f) {
                sh.o = origin;
                sh.d = ls.wi;
                sh.reach = reach;
                sh.contribution = ps.throughput * e.f * ls.radiance *
                                  (transmittance<FEAT>(s, P, origin, ls.wi, reach) * power_heuristic(ls.pdf, e.pdf) /
                                   ls.pdf);
                sh.valid = true;
            }
        }
    }

    const Material sm = dispersed<FEAT>(m, ps.wavelength, ps.throughput, ps.spectrum_u);
    const BsdfSample bs = sample_bsdf(sm, base, sf, wo, ps.rng);
    if (!bs.ok) return false;

    ps.throughput *= bs.weight;
    ps.last_pdf = bs.pdf;
    if (bs.delta) ps.flags |= PF_LAST_DELTA;
    else ps.flags &= ~PF_LAST_DELTA;
    ps.last_p = sf.p;
    ps.o = offset_origin(sf, bs.wi);
    ps.d = bs.wi;
    if (!roulette(ps.throughput, ps.depth, ps.rng)) return false;
    ps.depth++;
    return true;
}

// inspect (src/shaders.mjs:1377-1407): albedo, normal or depth of the first hit.
template <uint32_t FEAT>
__device__ float3 inspect_hit(const Scene& s, const Params& P, float3 o, float3 d, const Hit& hit) {
    if (hit.prim == NONE) return P.view == VIEW_ALBEDO ? sky<FEAT>(s, P, d) : f3(0.0f);
    const Surface sf = surface_at<FEAT>(s, o, d, hit);
    const Material m = load_material(s, sf.material);
    if (P.view == VIEW_ALBEDO) {
        if (m.kind == LIGHT) {
            const float3 e = emitted<FEAT>(s, m, sf.uv);
            return e / fmaxf(fmaxf(e.x, e.y), fmaxf(e.z, 1.0f));
        }
        return albedo<FEAT>(s, m, sf.p, sf.uv);
    }
    if (P.view == VIEW_NORMAL) return sf.n;
    return f3(hit.t);
}

}  // namespace rmd
