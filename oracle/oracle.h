// Raymond CPU oracle — TEST INFRASTRUCTURE ONLY.
//
// A plain CPU restatement of the reference renderer's algorithms (Raymond,
// JavaScript + WGSL), used by tests/, __graft_entry__.smoke() and the
// cpu_baseline leg of bench.py to check the product. The product library
// (libraymond_cuda.so) never links, loads or calls anything here.
//
// Parity status: the reference is JavaScript/WGSL and no JS engine exists on
// either machine, so no executed reference output is available. The oracle is
// pinned instead against every known answer the reference's own tests hold
// for this path: its unit tests (tests/unit/bvh.test.mjs, scene.test.mjs,
// camera.test.mjs, shaders.test.mjs, ...) restated in
// tests/test_reference_*.py, and its browser tests' exact answers and
// estimator agreements (tests/browser/app.test.mjs: furnaces, direct light,
// environment, textures, caustics, denoiser) run on this oracle in
// tests/test_oracle_*.py.
// Byte-level parity of the BVH build with BVH.mjs is therefore pinned by
// those invariants only ("parity unpinned" against executed reference code).
//
// Every function names the reference file:line it restates.
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RO_NONE 0xffffffffu

// ---- BVH.build (src/BVH.mjs:57-234) ----
// mins/maxs: 3 doubles per primitive. nodes_out must hold max(1, 2*count-1)
// 32-byte nodes; order_out `count` u32. Returns the node count.
uint32_t ro_bvh_build(const double* mins, const double* maxs, uint32_t count, uint32_t max_leaf,
                      void* nodes_out, uint32_t* order_out);

// ---- Scene.raycast (src/Scene.mjs:202-283, 549-674), in double ----
// Packed buffers exactly as Scene.#pack lays them out. rays: 6 floats per
// ray (origin xyz, direction xyz), read as doubles. Outputs per ray: the
// leaf-order primitive index (RO_NONE for a miss), t, u, v, and the facing
// shading normal and front flag of Scene.raycast's Hit (normal maps are
// not applied here).
void ro_raycast_batch(const void* prims, uint32_t prim_count, const void* nodes,
                      const float* attributes, const float* rays, uint32_t n, double t_max,
                      uint32_t* prim_out, double* t_out, double* uv_out, double* normal_out,
                      uint8_t* front_out, int threads);

// Intersection of one primitive in double (Scene.#intersect, src/Scene.mjs:579-674).
// Returns 1 and writes t,u,v on a hit nearer than t_max.
int ro_intersect_double(const void* prims, uint32_t p, const double* o, const double* d,
                        double t_max, double* tuv);

// The surface frame of a hit as Scene.raycast builds it, in double
// (src/Scene.mjs:687-879): geometric and shading normal (unflipped), uv,
// tangent and up — 14 doubles.
void ro_surface_double(const void* prims, const float* attributes, uint32_t p, const double* o, const double* d,
                       double t, double bu, double bv, double* out);

// ---- trace() of the trace shader (src/shaders.mjs:363-447), in f32 ----
// The GPU's own traversal order and arithmetic, restated on the CPU, with
// counters for the algorithmic byte figure: inner nodes whose two children
// were tested, and primitives tested. any_hit as the shader's shadow rays.
void ro_trace32_batch(const void* prims, const void* nodes, const float* rays, uint32_t n,
                      float t_max, int any_hit, uint32_t* prim_out, float* t_out,
                      uint32_t* inner_out, uint32_t* tested_out, int threads);

// One ray of the above, returning (t, u, v) too.
void ro_trace32_one(const void* prims, const void* nodes, const float* o, const float* d, float t_max, int any_hit,
                    uint32_t* prim_out, float* tuv_out, uint32_t* inner_out, uint32_t* tested_out);

// ---- the trace shader's path tracer (src/shaders.mjs:131-1899), in f32 ----
// Renders params.samples_per_frame samples for every pixel of the region
// [x0, x0+rw) × [y0, y0+rh) of the params' image, as main() does, and
// writes the region's per-pixel sums (accum rgb+lum², guide albedo, guide
// normal), 4 floats each, row-major over the region. seed_hash is XORed into
// the sample hashes (0: the reference's streams). counters (optional, 8
// u64): algorithmic bytes, rays traced, surface hits, paths; traversal bytes
// of closest-hit traces, of shadow traces; closest-hit rays, shadow rays.
void ro_render(const void* prims, const void* nodes, const void* materials, const float* attributes,
               const uint32_t* lights, const void* params208, uint32_t seed_hash, uint32_t x0, uint32_t y0,
               uint32_t rw, uint32_t rh, float* accum_out, float* albedo_out, float* normal_out,
               uint64_t* counters, int threads);
// ro_render with what the renderer uploads beside the packed scene, each
// optional (null): an environment map (RGBA half floats, env_w × env_h,
// and its importance table, cw × (ch + 1) floats), the colour and emission
// texture array and the normal-map array (layers of w × h RGBA bytes).
void ro_render_scene(const void* prims, const void* nodes, const void* materials, const float* attributes,
                     const uint32_t* lights, const void* params208, uint32_t seed_hash, uint32_t x0, uint32_t y0,
                     uint32_t rw, uint32_t rh, float* accum_out, float* albedo_out, float* normal_out,
                     uint64_t* counters, int threads, const uint16_t* env_rgba16f, uint32_t env_w, uint32_t env_h,
                     const float* table, uint32_t cw, uint32_t ch, const uint8_t* tex, uint32_t tex_w,
                     uint32_t tex_h, const uint8_t* nrm, uint32_t nrm_w, uint32_t nrm_h);

// ---- light tracing and photon mapping (src/shaders.mjs:1425-1831) ----
// Photons id0..id0+count-1 of a frame of `photons`: fixed-point splats
// added to `splats` (W·H·4 u32) and the stored photons (9 floats: p, power,
// -d) in photon order, with (each optional, NULL for none) their light
// paths' ids, their splats (4 u32: pixel or NONE, then the fixed-point
// amounts added) and their paths' smallest edge margins; and every path's
// smallest edge margin, whether or not it stored a photon (count floats,
// 1 for a path that hit nothing); returns how many were stored.
uint32_t ro_light_trace(const void* prims, const void* nodes, const void* materials, const float* attributes,
                        const uint32_t* lights, const void* params208, const float* emitters, uint32_t photons,
                        uint32_t id0, uint32_t count, uint32_t seed_hash, uint32_t* splats, float* photons_out,
                        uint32_t* ids_out, uint32_t* splat_out, float* margin_out, float* path_margin_out,
                        int threads);
// The photon map's caustic light through mirrors and glass on rows
// y0..y0+rows-1, added to accum (W·H·4); each gathering pixel's count of
// photons visited in visits_out (W·H, or NULL).
void ro_photon_gather(const void* prims, const void* nodes, const void* materials, const float* attributes,
                      const uint32_t* lights, const void* params208, const float* photons, uint32_t count,
                      uint32_t y0, uint32_t rows, uint32_t seed_hash, float* accum, uint32_t* visits_out,
                      int threads);

// ---- the denoiser (src/shaders.mjs:1916-2098) and display (2114-2152) ----
// Full-image à-trous from the accumulated buffers: prepare, steps 1..16,
// compose. out: w*h*4 floats.
void ro_denoise(const float* accum, const float* guide_albedo, const float* guide_normal, uint32_t w, uint32_t h,
                uint32_t total_samples, float* out, int threads);
// The display pass into RGBA8.
void ro_display(const float* accum, const float* denoised, const void* params208, uint8_t* out);

// Whether another primitive than `exclude` is crossed within rtol·t of t.
int ro_tie32(const void* prims, const void* nodes, const float* o3, const float* d3, float t, float rtol,
             uint32_t exclude);

// The sample streams in raymond_sample_streams's layout, and the
// perturbation runs' size (0: off) and seed.
void ro_sample_streams(const uint32_t* pairs, uint32_t n, const uint32_t* dim_ids, uint32_t dims, uint32_t chain,
                       uint32_t seed_hash, float* out);
void ro_set_jitter(uint32_t seed, float size);

/* The learned denoiser's network (net.cpp): parameter layout, loss and
 * gradients in double (bf16 != 0 rounds weights and stored tensors to BF16
 * as the GPU stores them; rel_eps is the relative term's ε, 0.01 on the
 * GPU), and single convolutions. */
uint64_t ro_net_param_count(void);
void ro_net_layout(uint64_t* w_off, uint64_t* b_off, uint32_t* cin, uint32_t* cout);
double ro_net_loss_grad(const double* params, const float* accum, const float* albedo, const float* normal,
                        const float* target, const float* samples, uint32_t n, uint32_t h, uint32_t w, int bf16,
                        double w_log, double w_rel, double rel_eps, double* grads, float* out16);
void ro_conv3x3(int mode, uint32_t n, uint32_t h, uint32_t w, const float* src0, uint32_t c0, uint32_t shift0,
                const float* src1, uint32_t c1, uint32_t cout, const float* weight, const float* bias, const float* dy,
                const float* mask, int act, float* out, double* dw, double* db);

#ifdef __cplusplus
}
#endif
