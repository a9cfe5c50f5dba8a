// Kernel declarations shared by the kernel translation units and the host runtime.
#pragma once
#include "dev_common.cuh"

namespace rmd {

// Launch-side description of the per-pixel buffers.
struct PixelBuffers {
    float4* accum;
    float4* guide_albedo;
    float4* guide_normal;
    float4* light_a;
    float4* light_b;
    float4* guide_unit;  // the à-trous passes' guide: unit normal and mean depth
    float4* denoised;
    uint32_t* splats;
    uchar4* display;
};

constexpr int TRACE_BLOCK = 128;

// Wavefront path state in HBM: 8 float4 records per path (ray, throughput,
// result, last point, guides, sample state), its last hit, two path queues,
// the shadow-ray queue (3 float4 each) and the work counters.
struct WavefrontState {
    float4* s[8];
    float4* hit;
    uint32_t* queue[2];
    uint32_t* sorted;    // this bounce's queue ordered by shading key, for the shade kernel
    uint32_t* sort_key;  // per path: its shading key
    // Shadow rays by bounce parity, so one bounce's can trace while the next
    // bounce shades: each path's ray at its slot (3 float4: origin and
    // reach, direction and path, light and job), and the list of paths
    // that have one.
    float4* shadow[2];
    uint32_t* shadow_list[2];
    float4* shadow_sum;  // per path: the light its unoccluded shadow rays brought
    uint32_t* counters;
    uint64_t capacity;  // paths in flight
};

// Light tracing's splats (4 u32 per pixel, 1/65536 fixed point) and the
// photon map: a hash table of grid cells (`table` heads, then the photon
// count) with lists linked through the photons (3 float4 each: position and
// next, power, incoming direction).
struct CausticBuffers {
    uint32_t* splats;
    uint32_t* heads;
    float4* photons;
    float4* gathered;  // per pixel: the photon map's gather term of the frame
    uint32_t table, capacity, photons_per_frame;
};

// CUDA events around each wavefront stage launch (kind 0 extend, 1 shade,
// 2 shadow), recorded on the launching stream; count stops at capacity.
struct StageEvents {
    cudaEvent_t* begin;
    cudaEvent_t* end;
    int* kind;
    int capacity;
    int count;
};

// One renderer's part of a batched frame: its scene, this frame's uniforms
// and its per-pixel buffers.
struct JobDesc {
    Scene scene;
    Params params;
    PixelBuffers px;
};

// A run of a job's samples inside one wave of the path pool: samples
// [k0, k0 + nk) of job `job` (pixels each) occupy wave paths
// [path_offset, path_offset + nk·pixels); its pixels are wave pixels
// [pixel_offset, pixel_offset + pixels) for the finalize pass.
struct WaveSegment {
    uint32_t job, k0, nk, pixels;
    uint32_t path_offset, pixel_offset;
};
// A job's pixels inside a batched image pass: batch pixels
// [pixel_offset, pixel_offset + w·h) belong to job `job`.
struct JobPixels {
    uint32_t job, pixel_offset;
};
struct WavePlan {
    uint32_t first_segment, segments;  // into the segment array
    uint32_t paths, pixels;            // wave totals
};

// Launch shape of the wavefront kernels (chosen by the tuner).
// A second stream and the events that fork work onto it from a frame's
// stream and join it back (one join per bounce parity).
struct SideStream {
    cudaStream_t stream;
    cudaEvent_t fork, join[2];
};

// The streams a wavefront frame runs on beside its own: its paths split
// into up to kGroups groups of whole samples, each group's bounces on its
// own stream and its shadow rays on that group's side stream.
struct FrameStreams {
    static constexpr int kGroups = 2;
    cudaStream_t group[kGroups];
    SideStream side[kGroups];
    cudaEvent_t fork, join[kGroups];
};

// Paths [base, base + capacity) of a pool as a pool of their own, numbered
// from 0, with the counters of group g (64 words a group).
inline WavefrontState pool_slice(const WavefrontState& w, uint64_t base, uint32_t g, uint64_t capacity) {
    WavefrontState s = w;
    for (int k = 0; k < 8; ++k) s.s[k] += base;
    s.hit += base;
    s.queue[0] += base;
    s.queue[1] += base;
    s.sorted += base;
    s.sort_key += base;
    s.shadow[0] += base * 3;
    s.shadow[1] += base * 3;
    s.shadow_list[0] += base;
    s.shadow_list[1] += base;
    s.shadow_sum += base;
    s.counters += 64 * g;
    s.capacity = capacity;
    return s;
}

struct WavefrontTuning {
    int steps;                    // traversal steps between lane refills
    int traversal_blocks_per_sm;  // persistent extend/shadow blocks per SM
    int shade_blocks_per_sm;      // shade/generate/finalize blocks per SM
};

// Host-side launchers (kernels_*.cu). Each returns the number of kernel
// launches it enqueued.
int launch_trace_primary(const Scene& s, const float* rays, uint32_t n, uint32_t* prim, float* t,
                         uint32_t* work_counter, int num_sms, cudaStream_t st);
int launch_sample_streams(const uint32_t* pairs, uint32_t n, const uint32_t* dim_ids, uint32_t dims, uint32_t chain,
                          uint32_t seed_hash, float* out, cudaStream_t st);
int launch_megakernel(const Scene& s, const Params& P, uint32_t features, const PixelBuffers& px, int num_sms,
                      cudaStream_t st);
int launch_wavefront(const Scene& s, const Params& P, uint32_t features, const WavefrontState& w,
                     const PixelBuffers& px, const WavefrontTuning& tune, int num_sms, cudaStream_t st,
                     const FrameStreams* streams, StageEvents* events);
int launch_wavefront_batch(const JobDesc* d_jobs, const WaveSegment* d_segments, const WavePlan* waves,
                           uint32_t n_waves, uint32_t max_bounces, uint32_t features, const WavefrontState& w,
                           const WavefrontTuning& tune, int num_sms, cudaStream_t st);
int launch_image_batch(const JobDesc* d_jobs, const JobPixels* d_pix, uint32_t n_jobs, uint32_t total_pixels,
                       int num_sms, cudaStream_t st);
int launch_caustic_light(const Scene& s, const Params& P, uint32_t features, const CausticBuffers& cb, int num_sms,
                         cudaStream_t st);
int launch_caustic_resolve(const Params& P, const CausticBuffers& cb, const PixelBuffers& px, int num_sms,
                           cudaStream_t st);
// status: a device word set non-zero if a staged tile's wait runs out (null:
// every pass reads through L2).
int launch_light_trace_alone(const Scene& s, const Params& P, uint32_t features, const CausticBuffers& cb, int num_sms,
                             cudaStream_t st);
int launch_gather_alone(const Scene& s, const Params& P, uint32_t features, const CausticBuffers& cb, uint32_t n,
                        float4* out, int num_sms, cudaStream_t st);
int launch_texture_layer(const uint8_t* src, uint32_t tw, uint32_t th, uint8_t* dst, uint32_t w, uint32_t h, int srgb,
                         const double* decode, int num_sms, cudaStream_t st);
int launch_environment(const float* rgb, uint32_t W, uint32_t H, uint32_t cw, uint32_t ch, const double* sines,
                       uint16_t* halves, float* table, double* rows, int num_sms, cudaStream_t st);
int launch_denoise(const Params& P, const PixelBuffers& px, unsigned* status, cudaStream_t st);
int launch_tonemap(const Params& P, const PixelBuffers& px, cudaStream_t st);
int launch_average(const float4* sums, float4* out, uint32_t n, float samples, int num_sms, cudaStream_t st);
// Fill each kernel unit's sRGB decode table on the current device.
cudaError_t upload_srgb_table_trace();
cudaError_t upload_srgb_table_wavefront();
cudaError_t upload_srgb_table_caustics();
// The message raymond_last_error(NULL) returns, for calls that have no handle.
void set_handleless_error(const char* msg);

}  // namespace rmd
