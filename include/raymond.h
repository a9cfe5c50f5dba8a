/*
 * raymond.h — the C ABI of libraymond_cuda.so, the GB300 (sm_103a) backend
 * for Raymond's GPU render path.
 *
 * These entry points replace what src/Renderer.mjs does through WebGPU. The
 * packed buffers they take are byte-for-byte the ones Scene.pack() makes
 * (src/Scene.mjs:15-60): 64-byte primitives, 32-byte BVH nodes
 * (src/BVH.mjs:1-16), 96-byte materials, 16-float triangle attribute blocks
 * and the u32 lights/volumes/CDF list (src/Renderer.mjs:598-607). The
 * 208-byte uniform block is Params (src/shaders.mjs:9-30) as
 * Renderer.#writeParams fills it (src/Renderer.mjs:925-991).
 *
 * Conventions: every call returns RAYMOND_OK (0) or a negative status; the
 * message is kept per handle (raymond_last_error). Host pointers are only
 * read during the call. A handle is used from one host thread at a time and
 * all its device work runs in order on the handle's CUDA stream.
 */
#ifndef RAYMOND_H
#define RAYMOND_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RAYMOND_OK 0
#define RAYMOND_EINVAL -1    /* bad argument or malformed packed data */
#define RAYMOND_ENOMEM -2    /* a device or host allocation failed */
#define RAYMOND_ECUDA -3     /* a CUDA call or kernel failed */
#define RAYMOND_ESTATE -4    /* call out of order (e.g. read before render) */
#define RAYMOND_ETIMEOUT -5  /* a device-side wait hit its iteration limit */
#define RAYMOND_ECAPACITY -6 /* a request exceeds a fixed capacity */

/* Optional trace-shader features (src/shaders.mjs:55-58; src/Renderer.mjs:434-439). */
#define RAYMOND_FEATURE_VOLUMES 1u
#define RAYMOND_FEATURE_TEXTURES 2u
#define RAYMOND_FEATURE_ENVIRONMENT 4u
#define RAYMOND_FEATURE_DISPERSION 8u

/* raymond_render flags. */
#define RAYMOND_FLAG_CAUSTICS 1u /* run light tracing + photon mapping this frame */
#define RAYMOND_FLAG_DENOISE 2u  /* run the à-trous passes this frame */
#define RAYMOND_FLAG_MEGAKERNEL 4u /* force the one-kernel path (else the tuned choice) */
#define RAYMOND_FLAG_WAVEFRONT 8u  /* force the wavefront path */

#define RAYMOND_PARAMS_BYTES 208
#define RAYMOND_IMAGE_KEY_BYTES 168

typedef struct raymond raymond_t;

typedef struct raymond_config {
    int device;              /* CUDA ordinal */
    uint32_t seed;           /* XORed into the sample hashes; 0 reproduces the reference streams */
    uint64_t path_capacity;  /* wavefront paths in flight; 0 = sized from free memory */
    uint32_t reserved[4];
} raymond_config;

/* Renderer.create (src/Renderer.mjs:247-279): picks the device, makes the stream. */
int raymond_create(raymond_t** out, const raymond_config* cfg);

/* Renderer.dispose (src/Renderer.mjs:531-547). */
void raymond_destroy(raymond_t* h);

/* The message of the handle's last failure ("" if none). With h NULL: the last
 * failure on this thread of a call that has no handle (create, denoise_static). */
const char* raymond_last_error(raymond_t* h);

/*
 * Renderer.#upload (src/Renderer.mjs:550-626). prims: prim_slots 64-byte
 * records, the first bvh_prim_count in BVH leaf order, then the volumes.
 * nodes: node_count 32-byte records. materials: mat_count 96-byte records.
 * attributes: attr_vec4s vec4s. lights: words u32 = light_count light
 * primitive indices, volume_count volume primitive indices, light_count CDF
 * entries as f32 bits. Validates every index before anything is uploaded;
 * restarts the average.
 */
int raymond_upload_scene(raymond_t* h, const void* prims, uint32_t prim_slots, uint32_t bvh_prim_count,
                         const void* nodes, uint32_t node_count, const void* materials, uint32_t mat_count,
                         const float* attributes, uint32_t attr_vec4s, const uint32_t* lights, uint32_t words,
                         uint32_t light_count, uint32_t volume_count);

/*
 * Renderer.#uploadTextures (src/Renderer.mjs:637-661). which: 0 = colour
 * textures (sRGB bytes, decoded on sampling), 1 = normal maps (plain bytes).
 * rgba: layers × h × w × 4 bytes, every layer already resized to w × h.
 */
int raymond_upload_textures(raymond_t* h, int which, const uint8_t* rgba, uint32_t w, uint32_t hgt,
                            uint32_t layers);

/*
 * Renderer.#uploadEnvironment (src/Renderer.mjs:723-760). rgba16f: w × h
 * half floats × 4; table: cw × (ch + 1) f32 as EnvironmentMap.importance()
 * lays it out (src/EnvironmentMap.mjs:202-247).
 */
int raymond_upload_environment(raymond_t* h, const uint16_t* rgba16f, uint32_t w, uint32_t hgt,
                               const float* table, uint32_t cw, uint32_t ch_plus_1);

/*
 * The texture array built on the GPU from the scene's own images, as
 * Renderer.#uploadTextures builds it on the host (src/Renderer.mjs:637-661):
 * `count` RGBA8 images (widths[k] × heights[k], host pointers) become the
 * layers of an array whose layers are the largest width and height (at most
 * 2048); an image of another size is resampled to it as Texture.resized
 * does (src/Texture.mjs:193-209): bilinear with wrap at texel centres, in
 * double, its bytes decoded by decode256 (the 256 values a byte stands for:
 * sRGB to linear light for colour, byte/255 for normal maps) and, with
 * srgb, re-encoded by toSrgbByte, else rounded as plain numbers. which: 0
 * colour and emission textures, 1 normal maps. Does what
 * raymond_upload_textures does with an array resized on the host; the
 * bytes are the same.
 */
int raymond_upload_texture_images(raymond_t* h, int which, const uint8_t* const* images, const uint32_t* widths,
                                  const uint32_t* heights, uint32_t count, int srgb, const double* decode256);

/*
 * The environment map built on the GPU from its float RGB pixels (w × h × 3,
 * host), as Renderer.#uploadEnvironment builds it on the host
 * (src/Renderer.mjs:723-760): RGBA half floats by toHalf's steps
 * (src/Renderer.mjs:1143-1160) and the importance table of
 * EnvironmentMap.importance (src/EnvironmentMap.mjs:202-247: min(w, 512) ×
 * min(h, 256, that) cells, each row's running sums, then the CDF over
 * rows). row_sines holds sin((y + 0.5) / rows · π) for each of the `rows`
 * rows of cells, computed by the caller as the reference computes it. Does
 * what raymond_upload_environment does with arrays made on the host; the
 * halves and the table are the same.
 */
int raymond_upload_environment_rgb(raymond_t* h, const float* rgb, uint32_t w, uint32_t hgt, const double* row_sines,
                                   uint32_t rows);

/* The uploaded texture array (which 0 or 1) and environment, copied back to host memory. */
int raymond_read_textures(raymond_t* h, int which, uint8_t* out, uint64_t bytes);
int raymond_read_environment(raymond_t* h, uint16_t* rgba16f, uint64_t map_bytes, float* table, uint64_t table_bytes);

/* Renderer.#writeEmitters' buffer (src/Renderer.mjs:670-717): vec4_count vec4s. */
int raymond_set_emitters(raymond_t* h, const float* data, uint32_t vec4_count);

/*
 * Light tracing and photon mapping beyond the reference's fixed sizes
 * (src/Renderer.mjs:37-39; src/shaders.mjs:1495-1510). photons_per_frame:
 * light paths traced per frame (0: min(w·h·spp, capacity), as the
 * reference). capacity: photons the map holds per frame (0: 524,288).
 * radius: a fixed gathering radius (0: the params' shrinking radius; the
 * grid cell is twice the radius either way). The hash table grows to at
 * least twice the capacity (power of two, at least 2^20).
 */
int raymond_set_photons(raymond_t* h, uint32_t photons_per_frame, uint32_t capacity, float radius);

/* Renderer.#resize (src/Renderer.mjs:766-799): keeps buffers that are big enough. */
int raymond_resize(raymond_t* h, uint32_t w, uint32_t hgt);

/*
 * Renderer.render's GPU work (src/Renderer.mjs:441-490): the trace, then
 * with RAYMOND_FLAG_CAUSTICS light tracing, splat resolve and photon gather,
 * then with RAYMOND_FLAG_DENOISE prepare, 5 à-trous passes and compose,
 * then the tone map into the headless display buffer. Enqueued only.
 */
int raymond_render(raymond_t* h, const void* params208, uint32_t features, uint32_t flags);

/*
 * One frame of many renderers in one pass (the batched workload): every
 * job's paths share the executor's wavefront path pool — generate, then per
 * bounce extend / shade / shadow over all jobs' paths at once, then finalize,
 * the à-trous passes and the tone map over all jobs' images — so small and
 * large images fill the GPU together. With RAYMOND_BATCH_GRAPH the frame's
 * launches are captured once as a CUDA graph and replayed while the jobs'
 * sizes, sample counts and bounces stay the same; each frame's uniforms
 * reach it through a device job table copied before the launch. Colour
 * frames only; light tracing does not run in a batch (each job's caustics
 * flag is taken as off). Work runs on the executor's stream: sync the
 * executor before reading the jobs' images. Limits: ≤ 2048 jobs, ≤ 2^21
 * pixels per job.
 */
typedef struct raymond_job {
    raymond_t* renderer;   /* the job's scene, image buffers and state */
    const void* params208; /* this frame's uniform block for it */
    uint32_t features;     /* RAYMOND_FEATURE_* of its scene */
} raymond_job;
#define RAYMOND_BATCH_GRAPH 1u
int raymond_render_batch(raymond_t* executor, const raymond_job* jobs, uint32_t n, uint32_t flags);

/* Waits for the handle's stream: backs device.queue.onSubmittedWorkDone(). */
int raymond_sync(raymond_t* h);

/*
 * Renderer.readPixels (src/Renderer.mjs:502-528): w × h × 4 floats, the
 * average (every float divided by samples) or, with denoised, the denoised
 * result as is. Synchronous.
 */
int raymond_read_pixels(raymond_t* h, float* out_rgba, uint64_t bytes, int denoised, uint32_t samples);

/*
 * The raw per-pixel sums behind readPixels: accum (rgb, luminance² in w),
 * guide albedo and guide normal (w: distance), w × h × 4 floats each, not
 * divided by the sample count. Any output may be NULL. Synchronous.
 */
int raymond_read_guides(raymond_t* h, float* accum, float* guide_albedo, float* guide_normal, uint64_t bytes_each);

/* The display pass's output (src/shaders.mjs:2124-2152) as w × h RGBA8. */
int raymond_read_display(raymond_t* h, uint8_t* out_rgba8, uint64_t bytes);

/*
 * Primary-ray closest hits on the uploaded scene: rays are 6 floats each
 * (origin, direction); out prim is the leaf-order primitive index
 * (0xffffffff for a miss), the index space of the shader's Hit.prim
 * (src/shaders.mjs:380-447) and of Scene.raycast's best (src/Scene.mjs:250).
 * Host pointers; copies in and out inside the call.
 */
int raymond_trace_primary(raymond_t* h, const float* rays, uint32_t n, uint32_t* prim, float* t);

/* The same on device pointers, enqueued on the handle's stream (no copies, no sync). */
int raymond_trace_primary_device(raymond_t* h, const float* d_rays, uint32_t n, uint32_t* d_prim,
                                 float* d_t);

/*
 * The sample streams the kernels draw from, for checking them bit for bit
 * against the reference's (src/shaders.mjs:135-212; seeding :1852-1859 for
 * camera paths, :1638 for light paths, :1585 for the photon gather). For
 * each of n (pixel index, sample index) pairs: for each dimension id in
 * dim_ids, the camera path's rand2() at that dimension (two values) then its
 * rand() (one); the path's spectrum position (:1857-1859); then `chain`
 * draws of light path `pixel index`'s PCG chain in a frame starting at
 * `sample index`, and `chain` draws of that pixel's gather chain. out holds
 * n × (3·dims + 1 + 2·chain) floats. At most 2^20 pairs, 64 dimensions and
 * 64 chain draws. Host pointers; synchronous. Test support: no counterpart
 * call in the reference, whose streams live inside its shader.
 */
int raymond_sample_streams(raymond_t* h, const uint32_t* pairs, uint32_t n, const uint32_t* dim_ids, uint32_t dims,
                           uint32_t chain, uint32_t seed_hash, float* out);

/*
 * One frame's light tracing alone, for checking it against the reference's
 * light_trace (src/shaders.mjs:1628-1814): runs the light-tracing kernel a
 * caustics frame runs, with params208 on the uploaded scene and emitters
 * (the photon count, capacity and radius of raymond_set_photons), and copies
 * out its fixed-point splat sums before they are resolved into the image
 * (width × height × 4 u32, 1/65536 units; splat_bytes ≥ width·height·16)
 * and the photons it deposited, 11 floats each: where it landed, its power,
 * the direction it came from, its light path's id and the pixel its splat
 * went to (both u32 bits; 0xffffffff for no splat). Photons come in the
 * order the GPU's atomics stored them; *photon_count is their number (at
 * most the map's capacity) and photon_floats must hold 11 per photon (NULL
 * photons: the count alone). The image is untouched. Host pointers;
 * synchronous.
 */
int raymond_light_trace(raymond_t* h, const void* params208, uint32_t features, uint32_t* splats, uint64_t splat_bytes,
                        float* photons, uint64_t photon_floats, uint32_t* photon_count);

/*
 * The photon map's gather alone, on a caller's photons (n × 9 floats:
 * position, power, direction it came from; n at most the map's capacity),
 * for checking it against the reference's photon_gather (src/shaders.mjs:
 * 1577-1626): links them into the hashed grid and runs the gather kernel a
 * caustics frame runs, writing the light it adds to each pixel (width ×
 * height × 4 floats: RGB × samples_per_frame and luminance² ×
 * samples_per_frame, as the frame accumulates it) into out. Host pointers;
 * synchronous.
 */
int raymond_photon_gather(raymond_t* h, const void* params208, uint32_t features, const float* photons, uint32_t n,
                          float* out, uint64_t out_bytes);

/*
 * Standalone BVH builder producing BVH.build's exact output (src/BVH.mjs:
 * 57-234): mins/maxs 3 doubles per primitive; nodes_out room for
 * max(1, 2*count - 1) 32-byte nodes; order_out count u32. Host only, no
 * handle. Returns the node count, or 0 on a bad argument.
 */
uint32_t raymond_bvh_build(const double* mins, const double* maxs, uint32_t count, uint32_t max_leaf,
                           void* nodes_out, uint32_t* order_out, int threads);

/* Device-side pointers of the handle's per-pixel buffers, for zero-copy callers (bench, tests). */
typedef struct raymond_buffers {
    float* accum;         /* w*h float4 */
    float* guide_albedo;  /* w*h float4 */
    float* guide_normal;  /* w*h float4 */
    float* denoised;      /* w*h float4 */
    uint8_t* display;     /* w*h RGBA8 */
    uint32_t width, height;
} raymond_buffers;
int raymond_get_buffers(raymond_t* h, raymond_buffers* out);

/* The handle's CUDA stream (a cudaStream_t), for callers that time or order work around it. */
void* raymond_get_stream(raymond_t* h);

/*
 * How frames are launched: the one-kernel path or the wavefront, and the
 * wavefront's launch shape. raymond_autotune picks it by timing; flags on a
 * raymond_render call can still force either path.
 */
#define RAYMOND_PATH_MEGAKERNEL 1u
#define RAYMOND_PATH_WAVEFRONT 2u
typedef struct raymond_tuning {
    uint32_t path;                    /* RAYMOND_PATH_* */
    uint32_t steps;                   /* traversal steps between lane refills, 1..256 */
    uint32_t traversal_blocks_per_sm; /* persistent extend/shadow blocks of 128 threads per SM, 1..16 */
    uint32_t shade_blocks_per_sm;     /* shade/generate/finalize blocks per SM, 1..64 */
    uint32_t bvh_width;               /* 2: walk the reference's binary nodes; 4: the 4-wide tree derived from
                                         them at upload (when it could be built); 0: 4 on the wavefront path,
                                         2 on the one-kernel path */
} raymond_tuning;
int raymond_set_tuning(raymond_t* h, const raymond_tuning* t);
int raymond_get_tuning(raymond_t* h, raymond_tuning* out);

/*
 * Times candidate tunings on whole frames of the uploaded scene with these
 * parameters and keeps the fastest (also written to best if not NULL). The
 * trial frames overwrite the accumulation, so call it before the first
 * frame of an image (the renderer does, when asked to tune). trials: frames
 * timed per candidate (>= 1).
 */
int raymond_autotune(raymond_t* h, const void* params208, uint32_t features, uint32_t trials, raymond_tuning* best);

/*
 * Counters of the last frame: kernel launches, paths, and the device time of
 * each stage from CUDA events recorded on the handle's stream around it
 * (valid once the frame has finished, e.g. after raymond_sync).
 */
typedef struct raymond_stats {
    uint64_t launches;
    uint64_t rays_primary, rays_extension, rays_shadow, rays_photon;
    uint64_t paths;
    float ms_trace, ms_caustics, ms_denoise, ms_display;
    /* wavefront frames: summed device time and launches of each stage kernel */
    float ms_extend, ms_shade, ms_shadow;
    uint32_t launches_extend, launches_shade, launches_shadow;
} raymond_stats;
int raymond_get_stats(raymond_t* h, raymond_stats* out);

/*
 * The à-trous denoiser (prepare, five passes, compose) on caller-owned device
 * buffers, allocating nothing. It has no counterpart in the reference: it is
 * for callers that cannot allocate device memory once they are running — a
 * host that hands this library a fixed memory budget up front, or a frame
 * loop that must not take cudaMalloc's device-wide synchronization — and so
 * cannot give a renderer its intermediate buffers. accum, guide_albedo and
 * guide_normal are w × h float4 device arrays as a renderer accumulates them
 * (raymond_get_buffers); out receives w × h float4; total_samples is the
 * frame's sample count; stream is a cudaStream_t (NULL: the default stream);
 * the kernels are only enqueued. The two intermediate light buffers live in
 * one static device array sized for RAYMOND_DENOISE_STATIC_MAX_PIXELS pixels
 * (8 MiB, held by every GPU that loads the library until exit); larger
 * images return RAYMOND_ECAPACITY. The first call on a device resolves the
 * array's address on that device (cudaGetSymbolAddress), so make it before
 * any stream capture. Calls share the array: calls that overlap on the GPU
 * race. Errors: raymond_last_error(NULL).
 */
#define RAYMOND_DENOISE_STATIC_MAX_PIXELS (512u * 512u)
int raymond_denoise_static(const float* accum, const float* guide_albedo, const float* guide_normal, uint32_t width,
                           uint32_t height, uint32_t total_samples, float* out, void* stream);

/*
 * The learned denoiser. It has no counterpart in the reference, whose only
 * denoiser is the à-trous filter (src/shaders.mjs:1916-2098); it stands
 * beside that filter and, like it, only filters the displayed image: the
 * renderer's running sums are its inputs, never its outputs.
 *
 * A raymond_net is a five-level U-Net of 3×3 convolutions (widths 32, 64,
 * 96, 128, 128; BF16 weights and activations, FP32 accumulation on the
 * tensor cores) with its FP32 master weights and Adam state, on one GPU.
 * Inputs are 12 channels computed from a renderer's buffers (log radiance
 * over albedo, albedo, normal, log depth, log standard error, 1/sqrt(n));
 * the output is a predicted log radiance over albedo (exponentiated and
 * multiplied back by albedo) and a per-pixel weight: the display is
 * α·prediction + (1 − α)·running average, α = sigmoid(weight)·v/(v + 0.1²)
 * with v the running average's relative variance of the mean luminance (the
 * factor is 1 below 4 samples), so α → 0 and the display converges with the
 * average as samples accumulate.
 * Errors: raymond_net_last_error(net); a failed create sets
 * raymond_last_error(NULL).
 */
typedef struct raymond_net raymond_net;
typedef struct raymond_net_config {
    int device;
    uint32_t seed;  /* weight initialisation (mulberry32) */
    uint32_t reserved[6];
} raymond_net_config;

/* n images of width × height, as device float4 arrays laid out like a
 * renderer's buffers (sums over the samples). target holds the converged
 * mean radiance per pixel (training only). samples: n device floats, or
 * NULL for samples_all. */
typedef struct raymond_net_batch {
    const float* accum;
    const float* albedo;
    const float* normal;
    const float* target;
    const float* samples;
    float samples_all;
    uint32_t n, width, height;
} raymond_net_batch;

int raymond_net_create(raymond_net** out, const raymond_net_config* cfg);
void raymond_net_destroy(raymond_net* net);
const char* raymond_net_last_error(const raymond_net* net);
/* Parameters are one flat FP32 vector: per layer its weights [cout][9][cin]
 * then its biases, each part starting at a multiple of 64. */
uint64_t raymond_net_param_count(const raymond_net* net);
int raymond_net_layout(const raymond_net* net, uint64_t* weight_offsets, uint64_t* bias_offsets, uint32_t* cin,
                       uint32_t* cout, uint32_t layers);
int raymond_net_set_params(raymond_net* net, const float* params, uint64_t count); /* resets Adam */
int raymond_net_get_params(raymond_net* net, float* params, uint64_t count);
/* The training loss per pixel and channel is lg(f) + lg(p), f the display,
 * p the prediction, lg(v) = w_log · |log(1 + v/a) − log(1 + t/a)| + w_rel ·
 * (v − t)² / (v² + rel_eps), t the target radiance, a the clamped albedo
 * (the relative term's denominator held constant; the prediction's
 * exponent clamped to ±8, its gradient passed through); averaged. Each
 * element's gradient is clipped to ±64 before averaging, and Adam skips
 * non-finite gradient elements. Defaults: weights 1 and 0, rel_eps 0.01; a
 * larger rel_eps moves the relative term towards the absolute squared
 * error on all but the brightest pixels. */
int raymond_net_set_loss(raymond_net* net, float w_log, float w_rel, float rel_eps);
/* The display blend's guard τ: α = sigmoid(gate) · v/(v + τ²), v the running
 * average's relative variance of the mean luminance; smaller τ trusts the
 * network longer as the average converges. Used by training and inference
 * alike; default 0.1. */
int raymond_net_set_blend(raymond_net* net, float tau);
float raymond_net_get_blend(const raymond_net* net);
/* Loss and its gradient with respect to every parameter, without a step.
 * Training crops are multiples of 16 pixels on each side. */
int raymond_net_gradients(raymond_net* net, const raymond_net_batch* batch, float* grads, uint64_t count, float* loss);
/* One Adam step (beta 0.9, 0.999; eps 1e-8) on the batch, enqueued on the
 * network's stream; loss (host, optional) waits for it. */
int raymond_net_train_step(raymond_net* net, const raymond_net_batch* batch, float learning_rate, float* loss);
int raymond_net_sync(raymond_net* net);
/* Denoised radiance (float4 per pixel, any size) into out_rgba (device),
 * enqueued on stream (NULL: the network's stream). */
int raymond_net_infer(raymond_net* net, const raymond_net_batch* batch, float* out_rgba, void* stream);
void* raymond_net_get_stream(raymond_net* net);
/* Enqueue the network's work on a caller's cudaStream_t from now on (NULL:
 * its own stream again; pass cudaStreamLegacy for the legacy default
 * stream), so that it is ordered with the caller's producers and consumers
 * of the batch memory. */
int raymond_net_set_stream(raymond_net* net, void* stream);

/* The renderer's current image through the network: the result replaces the
 * denoised buffer and the display image (display only; accum untouched),
 * as a denoised frame would. samples is the frame's total sample count;
 * out_rgba (host, optional) receives the w × h float4 result. */
int raymond_denoise_learned(raymond_t* h, raymond_net* net, uint32_t samples, float* out_rgba);

/*
 * The network's kernels one at a time, on caller-owned device memory (NHWC
 * BF16 tensors, channel strides multiples of 8, channel counts multiples of
 * 16). The input is the concatenation of src0 and src1 along channels;
 * shift 1 reads a source at half resolution (nearest-neighbour upsampling).
 *   forward:        out (or out_f32) = act(conv(src, weight) + bias)
 *   backward_data:  out = conv_transpose(dy, weight) × slope(mask)   (mask optional)
 *   backward_weight: dweight += Σ dy ⊗ src, dbias += Σ dy   (FP32, accumulated)
 * status is a device word that a kernel whose tensor-core wait ran out sets
 * to non-zero. Errors: raymond_last_error(NULL).
 */
typedef struct raymond_conv {
    uint32_t n, height, width, cin, cout;
    const void* src0;
    uint32_t src0_channels, src0_stride, src0_shift;
    const void* src1;
    uint32_t src1_channels, src1_stride, src1_shift;
    const void* weight;
    const float* bias;
    const void* dy;
    uint32_t dy_stride;
    void* out;
    uint32_t out_stride;
    float* out_f32;
    const void* mask;
    uint32_t mask_stride;
    float* dweight;
    float* dbias;
    int32_t activation; /* leaky ReLU, slope 0.1 below zero */
    uint32_t pixels_per_cta; /* backward_weight: 0 chooses */
    uint32_t* status;
    uint32_t kernel; /* forward, backward_data: 0 chooses (halo tiles), 1 pixel-row tiles, 2 halo tiles
                        (weights kept in shared memory, or streamed per channel chunk when they do not fit;
                        RAYMOND_EINVAL if even a streamed stage does not fit) */
} raymond_conv;
int raymond_conv3x3_forward(const raymond_conv* c, void* stream);
int raymond_conv3x3_backward_data(const raymond_conv* c, void* stream);
int raymond_conv3x3_backward_weight(const raymond_conv* c, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* RAYMOND_H */
