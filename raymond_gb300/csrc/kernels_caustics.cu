// Caustics for the render path: light tracing connected to the camera with
// atomic splats, and a hashed-grid photon map gathered through mirrors and
// glass (src/shaders.mjs:1425-1831). One thread per photon and one per
// pixel; the grid is the reference's (2^20 heads, lists linked by
// atomicExch) so counts, weights and the radius schedule match it.
#include "dev_shade.cuh"
#include "kernels.cuh"

namespace rmd {

namespace {

constexpr float SPLAT_SCALE = 65536.0f;
constexpr int CAUSTIC_BLOCK = 128;

__device__ __forceinline__ uint32_t photon_cell_hash(int cx, int cy, int cz, uint32_t table) {
    return ((uint32_t(cx) * 73856093u) ^ (uint32_t(cy) * 19349663u) ^ (uint32_t(cz) * 83492791u)) & (table - 1u);
}

// splat (src/shaders.mjs:1444-1491): the photon's light at the pixel that
// sees sf. Returns that pixel, or NONE when nothing was added.
template <uint32_t FEAT>
__device__ uint32_t splat(const Scene& s, const Params& P, const CausticBuffers& cb, const Surface& sf,
                          const Material& m, float3 base, float3 d, float3 beta, Rng& rng, uint32_t* stack_col,
                          uint32_t stride) {
    const float3 cam = f3(P.cam_pos);
    const float3 to_camera = cam - sf.p;
    const float dist = length(to_camera);
    const float3 wo = to_camera / dist;
    const float cos_film = -dot(wo, f3(P.cam_forward));
    if (cos_film <= 1e-6f || dot(wo, sf.ng) <= 0.0f) return NONE;
    const float x = -dot(wo, f3(P.cam_right)) / (cos_film * P.tan_half_fov * P.aspect);
    const float y = -dot(wo, f3(P.cam_up)) / (cos_film * P.tan_half_fov);
    const float px = (x + 1.0f) * 0.5f * float(P.width);
    const float py = (1.0f - y) * 0.5f * float(P.height);
    if (px < 0.0f || py < 0.0f || px >= float(P.width) || py >= float(P.height)) return NONE;
    const float3 wi = -d;
    const Eval e = eval_bsdf(m, base, sf.n, wo, wi);
    const float cos_in = dot(sf.n, wi);
    if (e.pdf <= 0.0f || cos_in <= 0.0f) return NONE;
    const float3 origin = offset_origin(sf, wo);
    if (trace_ray<true>(s, origin, wo, dist - dot(origin - sf.p, wo), stack_col, stride).prim != NONE) return NONE;
    const float pixel_area = (4.0f * P.tan_half_fov * P.tan_half_fov * P.aspect) / float(P.width * P.height);
    const float3 value =
        beta * (e.f / cos_in) * (dot(wo, sf.ng) / (dist * dist * pixel_area * cos_film * cos_film * cos_film));
    if (!finite3(value)) return NONE;
    const uint32_t index = (uint32_t(py) * P.width + uint32_t(px)) * 4u;
    const float r0 = rng.rand(), r1 = rng.rand(), r2 = rng.rand();
    atomicAdd(&cb.splats[index], uint32_t(fminf(value.x * SPLAT_SCALE + r0, 4e9f)));
    atomicAdd(&cb.splats[index + 1], uint32_t(fminf(value.y * SPLAT_SCALE + r1, 4e9f)));
    atomicAdd(&cb.splats[index + 2], uint32_t(fminf(value.z * SPLAT_SCALE + r2, 4e9f)));
    return index / 4u;
}

// deposit (src/shaders.mjs:1518-1528): one photon into the hashed grid. The
// power record's fourth word keeps the light path's id and the direction
// record's the pixel its splat went to (NONE for none), so a photon and its
// splat can be told apart from the others whatever order the atomics
// stored them in.
__device__ void deposit(const Params& P, const CausticBuffers& cb, float3 p, float3 d, float3 beta, uint32_t id,
                        uint32_t splat_pixel) {
    const uint32_t i = atomicAdd(&cb.heads[cb.table], 1u);
    if (i >= cb.capacity) return;
    const int cx = int(floorf(p.x / P.photon_cell)), cy = int(floorf(p.y / P.photon_cell)),
              cz = int(floorf(p.z / P.photon_cell));
    const uint32_t next = atomicExch(&cb.heads[photon_cell_hash(cx, cy, cz, cb.table)], i + 1u);
    cb.photons[size_t(i) * 3] = make_float4(p.x, p.y, p.z, __uint_as_float(next));
    cb.photons[size_t(i) * 3 + 1] = make_float4(beta.x, beta.y, beta.z, __uint_as_float(id));
    cb.photons[size_t(i) * 3 + 2] = make_float4(-d.x, -d.y, -d.z, __uint_as_float(splat_pixel));
}

// light_trace (src/shaders.mjs:1630-1814).
template <uint32_t FEAT>
__global__ void __launch_bounds__(CAUSTIC_BLOCK) k_light_trace(Scene s, Params P, CausticBuffers cb) {
    __shared__ uint32_t stack[STACK_SHARED * CAUSTIC_BLOCK];
    uint32_t* col = stack + threadIdx.x;
    const uint32_t photons = cb.photons_per_frame;
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < photons; id += gridDim.x * blockDim.x) {
        Rng rng = light_rng(id, P.sample_offset, s.seed_hash);

        const float4 header = s.emitters[0];
        const uint32_t sources = __float_as_uint(header.x);
        const uint32_t targets = __float_as_uint(header.y);
        const float xi = rng.rand();
        uint32_t k = 0;
        while (!(k + 1u >= sources || s.emitters[1u + k].x > xi)) ++k;
        const float4 entry = s.emitters[1u + k];
        const float chance = entry.z;
        if (chance <= 0.0f) continue;
        const uint32_t prim_index = __float_as_uint(entry.y);
        const uint32_t first_target = 1u + sources;

        float3 o, d, beta;
        if (prim_index == NONE) {
            // The sun, through a target circle chosen by area.
            d = -sample_cone(f3(P.sun_dir), P.sun_omc, rng);
            float pick = rng.rand() * header.w / PI;
            uint32_t j = 0;
            for (;;) {
                const float r = s.emitters[first_target + j].w;
                if (j + 1u >= targets || pick < r * r) break;
                pick -= r * r;
                ++j;
            }
            const float4 circle = s.emitters[first_target + j];
            float3 f0, f1;
            frame_axes(d, f0, f1);
            const float2 disk = concentric_disk(rng);
            o = xyz(circle) - d * header.z + f0 * (disk.x * circle.w) + f1 * (disk.y * circle.w);
            float through = 1.0f;
            for (uint32_t i = 0; i < targets; ++i) {
                const float4 c = s.emitters[first_target + i];
                const float3 q = o - xyz(c);
                const float3 across = q - d * dot(q, d);
                through += (i != j && dot(across, across) < c.w * c.w) ? 1.0f : 0.0f;
            }
            const float3 irradiance = f3(P.sun_radiance) * (2.0f * PI * P.sun_omc);
            beta = irradiance * (header.w / (through * chance * float(photons)));
        } else {
            const float4* rec = s.prims + size_t(prim_index) * 4;
            const float4 hdr = ldg4(rec), p0 = ldg4(rec + 1), p1 = ldg4(rec + 2), p2 = ldg4(rec + 3);
            const Material m = load_material(s, __float_as_uint(hdr.y));
            float3 n;
            float area;
            float2 uv;
            if (__float_as_uint(hdr.x) == QUAD) {
                const float a = rng.rand();
                const float b = rng.rand();
                o = xyz(p0) + xyz(p1) * a + xyz(p2) * b;
                const float3 c = cross(xyz(p1), xyz(p2));
                area = length(c);
                n = c / area;
                uv = make_float2(a, 1.0f - b);
            } else {
                const float z = 1.0f - 2.0f * rng.rand();
                const float r = sqrtf(fmaxf(0.0f, one_minus_sq(z)));
                const float phi = 2.0f * PI * rng.rand();
                n = f3(r * cosf(phi), z, r * sinf(phi));
                o = xyz(p0) + n * p0.w;
                area = 4.0f * PI * p0.w * p0.w;
                uv = sphere_uv(n, xyz(p1), xyz(p2));
            }
            // Aim at the targets' spheres by solid angle; shared where cones overlap.
            float cones = 0.0f;
            bool inside = false;
            for (uint32_t i = 0; i < targets; ++i) {
                const float4 aim = s.emitters[first_target + i];
                const float3 to = xyz(aim) - o;
                const float d2 = dot(to, to);
                inside = inside || d2 <= aim.w * aim.w;
                cones += sphere_omc(aim.w, fmaxf(d2, aim.w * aim.w));
            }
            if (!inside) {
                float pick = rng.rand() * cones;
                uint32_t j = 0;
                for (;;) {
                    const float4 aim = s.emitters[first_target + j];
                    const float3 to = xyz(aim) - o;
                    const float omc = sphere_omc(aim.w, dot(to, to));
                    if (j + 1u >= targets || pick < omc) {
                        d = sample_cone(to / length(to), omc, rng);
                        break;
                    }
                    pick -= omc;
                    ++j;
                }
                float within = 1.0f;
                for (uint32_t i = 0; i < targets; ++i) {
                    const float4 aim = s.emitters[first_target + i];
                    const float3 to = xyz(aim) - o;
                    const float omc = sphere_omc(aim.w, dot(to, to));
                    within += (i != j && 1.0f - dot(d, to / length(to)) <= omc) ? 1.0f : 0.0f;
                }
                const float cos_out = dot(d, n);
                if (cos_out <= 0.0f) continue;
                beta = emitted<FEAT>(s, m, uv) *
                       ((cos_out * area * 2.0f * PI * cones) / (within * chance * float(photons)));
            } else {
                d = cosine_hemisphere(n, rng);
                beta = emitted<FEAT>(s, m, uv) * ((PI * area) / (chance * float(photons)));
            }
            o = o + n * (1e-4f * fmaxf(1.0f, fmaxf(fabsf(o.x), fmaxf(fabsf(o.y), fabsf(o.z)))));
        }

        float wavelength = 0.0f;
        uint32_t bounces = 0;
        float3 carried = f3(1.0f);
        for (uint32_t depth = 0; depth < P.max_bounces; ++depth) {
            const Hit hit = trace_ray<false>(s, o, d, INF, col, CAUSTIC_BLOCK);
            if (hit.prim == NONE) break;
            const Surface sf = surface_at<FEAT>(s, o, d, hit);
            const Material m = load_material(s, sf.material);
            if (m.kind == LIGHT) break;
            const float3 base = albedo<FEAT>(s, m, sf.p, sf.uv);
            if (!is_delta(m)) {
                // Straight from the lamp is the path tracer's; after mirrors or glass, a caustic.
                if (bounces > 0u) {
                    const uint32_t pixel = splat<FEAT>(s, P, cb, sf, m, base, d, beta * carried, rng, col, CAUSTIC_BLOCK);
                    deposit(P, cb, sf.p, d, beta * carried, id, pixel);
                }
                break;
            }
            const float u = rng.rand();  // drawn for dispersion whether or not it is used
            const Material sm = dispersed<FEAT>(m, wavelength, carried, u);
            const BsdfSample bs = sample_bsdf(sm, base, sf, -d, rng);
            if (!bs.ok) break;
            carried *= bs.weight;
            ++bounces;
            o = offset_origin(sf, bs.wi);
            d = bs.wi;
            if (!roulette(carried, depth, rng)) break;
        }
    }
}

// resolve_splats (src/shaders.mjs:1819-1831), then the photon map's gather
// term of the pixel (k_photon_gather's output), added in that order as the
// reference's passes add them.
__global__ void k_resolve_splats(Params P, CausticBuffers cb, float4* __restrict__ accum) {
    const uint32_t n = P.width * P.height;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float r = float(atomicExch(&cb.splats[i * 4], 0u)) / SPLAT_SCALE;
        const float g = float(atomicExch(&cb.splats[i * 4 + 1], 0u)) / SPLAT_SCALE;
        const float b = float(atomicExch(&cb.splats[i * 4 + 2], 0u)) / SPLAT_SCALE;
        const float l = luminance(f3(r, g, b));
        const float k = float(P.samples_per_frame);
        const float4 a = accum[i];
        const float4 s = make_float4(a.x + r * k, a.y + g * k, a.z + b * k, a.w + l * l * k);
        const float4 t = cb.gathered[i];
        accum[i] = make_float4(s.x + t.x, s.y + t.y, s.z + t.z, s.w + t.w);
    }
}

// gather (src/shaders.mjs:1534-1570).
__device__ float3 gather(const Params& P, const CausticBuffers& cb, const Surface& sf, const Material& m, float3 base,
                         float3 wo) {
    const float r = P.photon_radius;
    const float r2 = r * r;
    const float cell = P.photon_cell;
    const float3 here = sf.p / cell;
    const float fx = floorf(here.x), fy = floorf(here.y), fz = floorf(here.z);
    const int cx = int(fx), cy = int(fy), cz = int(fz);
    const int sx = here.x - fx >= 0.5f ? 1 : -1, sy = here.y - fy >= 0.5f ? 1 : -1, sz = here.z - fz >= 0.5f ? 1 : -1;
    float3 sum = f3(0.0f);
    uint32_t visited = 0;
    for (uint32_t k = 0; k < 8u; ++k) {
        const int ccx = cx + int(k & 1u) * sx, ccy = cy + int((k >> 1) & 1u) * sy, ccz = cz + int((k >> 2) & 1u) * sz;
        uint32_t index = cb.heads[photon_cell_hash(ccx, ccy, ccz, cb.table)];
        while (index != 0u && visited < 4096u) {
            ++visited;
            const float4 at = cb.photons[size_t(index - 1u) * 3];
            const float3 off = xyz(at) - sf.p;
            if (dot(off, off) < r2 && fabsf(dot(off, sf.ng)) < 0.25f * r) {
                const float3 wi = xyz(cb.photons[size_t(index - 1u) * 3 + 2]);
                const float cos_in = dot(sf.n, wi);
                if (cos_in > 0.0f && dot(sf.ng, wi) > 0.0f) {
                    const Eval e = eval_bsdf(m, base, sf.n, wo, wi);
                    sum += xyz(cb.photons[size_t(index - 1u) * 3 + 1]) * (e.f / cos_in);
                }
            }
            index = __float_as_uint(at.w);
        }
    }
    return sum / (PI * r2);
}

// photon_gather (src/shaders.mjs:1577-1626): each pixel's term (its light
// times the frame's samples, and luminance² likewise; zero where the camera
// ray finds nothing to gather) written to out, for k_resolve_splats to add
// once the camera paths' sums are in.
template <uint32_t FEAT>
__global__ void __launch_bounds__(CAUSTIC_BLOCK) k_photon_gather(Scene s, Params P, CausticBuffers cb,
                                                                 float4* __restrict__ out) {
    __shared__ uint32_t stack[STACK_SHARED * CAUSTIC_BLOCK];
    uint32_t* col = stack + threadIdx.x;
    const uint32_t n = P.width * P.height;
    for (uint32_t index = blockIdx.x * blockDim.x + threadIdx.x; index < n; index += gridDim.x * blockDim.x) {
        Rng rng = gather_rng(index, P.sample_offset, s.seed_hash);
        const float jx = rng.rand();
        const float jy = rng.rand();
        float3 o, d;
        camera_ray(P, make_float2(float(index % P.width) + jx, float(index / P.width) + jy), true, rng, o, d);
        float3 throughput = f3(1.0f);
        float4 term = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        for (uint32_t depth = 0; depth < P.max_bounces; ++depth) {
            const Hit hit = trace_ray<false>(s, o, d, INF, col, CAUSTIC_BLOCK);
            if (hit.prim == NONE) break;
            const Surface sf = surface_at<FEAT>(s, o, d, hit);
            const Material m = load_material(s, sf.material);
            if (m.kind == LIGHT) break;
            const float3 base = albedo<FEAT>(s, m, sf.p, sf.uv);
            if (!is_delta(m)) {
                if (depth > 0u) {
                    const float3 light = throughput * gather(P, cb, sf, m, base, -d);
                    if (finite3(light)) {
                        const float l = luminance(light);
                        const float k = float(P.samples_per_frame);
                        term = make_float4(__fmul_rn(light.x, k), __fmul_rn(light.y, k), __fmul_rn(light.z, k),
                                           __fmul_rn(l * l, k));
                    }
                }
                break;
            }
            const BsdfSample bs = sample_bsdf(m, base, sf, -d, rng);
            if (!bs.ok) break;
            throughput *= bs.weight;
            o = offset_origin(sf, bs.wi);
            d = bs.wi;
        }
        out[index] = term;
    }
}

// Links a given photon list (cb.photons, 3 float4 each) into the hashed
// grid, as deposit does, for gathering a caller's photons.
__global__ void k_link_photons(Params P, CausticBuffers cb, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 at = cb.photons[size_t(i) * 3];
        const int cx = int(floorf(at.x / P.photon_cell)), cy = int(floorf(at.y / P.photon_cell)),
                  cz = int(floorf(at.z / P.photon_cell));
        const uint32_t next = atomicExch(&cb.heads[photon_cell_hash(cx, cy, cz, cb.table)], i + 1u);
        at.w = __uint_as_float(next);
        cb.photons[size_t(i) * 3] = at;
    }
}

template <uint32_t FEAT>
int light_trace_alone(const Scene& s, const Params& P, const CausticBuffers& cb, int num_sms, cudaStream_t st) {
    cudaMemsetAsync(cb.heads, 0, (size_t(cb.table) + 1) * sizeof(uint32_t), st);
    k_light_trace<FEAT><<<num_sms * 8, CAUSTIC_BLOCK, 0, st>>>(s, P, cb);
    return 1;
}

template <uint32_t FEAT>
int gather_alone(const Scene& s, const Params& P, const CausticBuffers& cb, uint32_t n, float4* out, int num_sms,
                 cudaStream_t st) {
    cudaMemsetAsync(cb.heads, 0, (size_t(cb.table) + 1) * sizeof(uint32_t), st);
    k_link_photons<<<num_sms * 8, 256, 0, st>>>(P, cb, n);
    k_photon_gather<FEAT><<<num_sms * 8, CAUSTIC_BLOCK, 0, st>>>(s, P, cb, out);
    return 2;
}

// A frame's light tracing and gathering need nothing of its camera paths,
// so they run on a stream of their own beside them; only the resolve waits
// for the camera paths' sums.
template <uint32_t FEAT>
int caustics_light(const Scene& s, const Params& P, const CausticBuffers& cb, int num_sms, cudaStream_t st) {
    cudaMemsetAsync(cb.heads, 0, (size_t(cb.table) + 1) * sizeof(uint32_t), st);
    const int grid = num_sms * 8;
    k_light_trace<FEAT><<<grid, CAUSTIC_BLOCK, 0, st>>>(s, P, cb);
    k_photon_gather<FEAT><<<grid, CAUSTIC_BLOCK, 0, st>>>(s, P, cb, cb.gathered);
    return 2;
}

}  // namespace

cudaError_t upload_srgb_table_caustics() { return upload_srgb_table_here(); }

int launch_light_trace_alone(const Scene& s, const Params& P, uint32_t features, const CausticBuffers& cb, int num_sms,
                             cudaStream_t st) {
    switch (features & 15u) {
        case 0: return light_trace_alone<0>(s, P, cb, num_sms, st);
        case F_DISPERSION: return light_trace_alone<F_DISPERSION>(s, P, cb, num_sms, st);
        default: return light_trace_alone<15u>(s, P, cb, num_sms, st);
    }
}

int launch_gather_alone(const Scene& s, const Params& P, uint32_t features, const CausticBuffers& cb, uint32_t n,
                        float4* out, int num_sms, cudaStream_t st) {
    switch (features & 15u) {
        case 0: return gather_alone<0>(s, P, cb, n, out, num_sms, st);
        case F_DISPERSION: return gather_alone<F_DISPERSION>(s, P, cb, n, out, num_sms, st);
        default: return gather_alone<15u>(s, P, cb, n, out, num_sms, st);
    }
}

int launch_caustic_light(const Scene& s, const Params& P, uint32_t features, const CausticBuffers& cb, int num_sms,
                         cudaStream_t st) {
    switch (features & 15u) {
        case 0: return caustics_light<0>(s, P, cb, num_sms, st);
        case F_DISPERSION: return caustics_light<F_DISPERSION>(s, P, cb, num_sms, st);
        default: return caustics_light<15u>(s, P, cb, num_sms, st);
    }
}

int launch_caustic_resolve(const Params& P, const CausticBuffers& cb, const PixelBuffers& px, int num_sms,
                           cudaStream_t st) {
    k_resolve_splats<<<num_sms * 8, 256, 0, st>>>(P, cb, px.accum);
    return 1;
}

}  // namespace rmd
