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
    float4* denoised;
    uint32_t* splats;
    uchar4* display;
};

constexpr int TRACE_BLOCK = 128;

// Host-side launchers (kernels_*.cu). Each returns the number of kernel
// launches it enqueued.
int launch_trace_primary(const Scene& s, const float* rays, uint32_t n, uint32_t* prim, float* t,
                         uint32_t* work_counter, int num_sms, cudaStream_t st);
int launch_megakernel(const Scene& s, const Params& P, uint32_t features, const PixelBuffers& px, int num_sms,
                      cudaStream_t st);
int launch_denoise(const Params& P, const PixelBuffers& px, cudaStream_t st);
int launch_tonemap(const Params& P, const PixelBuffers& px, cudaStream_t st);
void upload_srgb_table();
// The message raymond_last_error(NULL) returns, for calls that have no handle.
void set_handleless_error(const char* msg);

}  // namespace rmd
