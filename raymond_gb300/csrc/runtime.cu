// Host runtime behind include/raymond.h: device buffers in the packed
// formats, validation of uploaded scenes, the per-handle stream, frames,
// read-back. One handle is one renderer on one GPU.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <algorithm>
#include <vector>

#include "../../include/raymond.h"
#include "bvh_wide.h"
#include "kernels.cuh"
#include "net.cuh"

using namespace rmd;

static constexpr int raymond_stage_events = 1024;

namespace {

struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    // Grows (never shrinks) to hold `need` bytes; contents are not kept.
    cudaError_t reserve(size_t need) {
        if (need <= bytes && ptr) return cudaSuccess;
        release();
        cudaError_t e = cudaMalloc(&ptr, need > 0 ? need : 16);
        if (e == cudaSuccess) bytes = need > 0 ? need : 16;
        return e;
    }
};

}  // namespace

struct raymond {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    std::string error;
    uint32_t seed_hash = 0;

    // Scene.
    DevBuf prims, nodes, materials, attributes, lights, emitters;
    DevBuf wide;            // the 4-wide traversal tree derived from `nodes`
    bool has_wide = false;
    uint32_t bvh_width = 0;  // tuning: 2 binary, 4 wide, 0 wide for the wavefront and binary for the one-kernel path
    DevBuf textures, normal_maps, env_map, env_table;
    uint32_t prim_slots = 0, bvh_prim_count = 0, node_count = 0, mat_count = 0, attr_vec4s = 0;
    uint32_t light_words = 0, light_count = 0, volume_count = 0;
    uint32_t tex_w = 1, tex_h = 1, tex_layers = 0, nrm_w = 1, nrm_h = 1, nrm_layers = 0;
    uint32_t env_w = 1, env_h = 1, env_cw = 1, env_ch = 0;
    uint32_t emitter_vec4s = 0;
    bool has_scene = false;

    // Per-pixel buffers.
    DevBuf accum, guide_albedo, guide_normal, light_a, light_b, guide_unit, denoised, splats, display;
    uint32_t width = 0, height = 0;
    uint64_t capacity = 0;

    // Scratch for host-pointer trace calls, and the work counter.
    DevBuf ray_scratch, prim_scratch, t_scratch, counter, gathered;
    DevBuf upload_scratch;  // images staged for building texture arrays and the environment on the GPU

    // Wavefront path state (allocated on first wavefront frame).
    DevBuf wf_state[8], wf_hit, wf_queue[2], wf_sorted, wf_sort_key, wf_shadow, wf_shadow_list, wf_shadow_sum,
        wf_counters;
    uint64_t wf_capacity = 0;
    uint64_t path_capacity_limit = 0;  // from the config; 0 = default
    WavefrontTuning tuning{16, 8, 8};

    // Photon map (allocated when caustics first run) and its sizing.
    DevBuf photon_heads, photons;
    uint32_t photon_table = 0, photon_capacity_alloc = 0;
    uint32_t photons_override = 0, photon_capacity = 524288;
    float photon_radius_override = 0.0f;

    // Batched frames (this handle as executor): job table, wave plan, graph.
    DevBuf b_jobs, b_segments, b_jobpix;
    JobDesc* b_staging = nullptr;  // pinned host copy of the job table
    uint32_t b_staging_cap = 0;
    cudaEvent_t b_copy_done = nullptr;
    cudaEvent_t order = nullptr;  // orders a batch frame against the job renderers' own streams
    bool b_copy_pending = false;
    // The jobs run as up to kBatchGroups groups, each with its own slice of
    // the path pool, its own counters and its own stream (forked from and
    // joined to `stream`), so that one group's kernels fill the SMs another
    // group's persistent kernels leave idle at their tails. Group g's waves
    // are b_waves[b_group_first[g] .. + b_group_waves[g]).
    static constexpr int kBatchGroups = 8;
    std::vector<WavePlan> b_waves;
    std::vector<uint32_t> b_group_first, b_group_waves;
    uint64_t b_group_cap = 0;
    cudaStream_t b_group_stream[kBatchGroups] = {};
    cudaEvent_t b_fork = nullptr, b_join[kBatchGroups] = {};
    std::vector<uint64_t> b_signature;
    uint32_t b_max_bounces = 0, b_total_pixels = 0, b_n = 0;
    uint64_t b_paths = 0;
    cudaGraphExec_t b_graph = nullptr;
    int b_graph_launches = 0;  // kernels in the captured frame
    uint32_t path_choice = RAYMOND_PATH_WAVEFRONT;

    bool rendered = false;
    bool learned_valid = false;  // the denoised buffer holds the network's image of this frame
    Params last_params{};
    raymond_stats stats{};
    // Stage boundaries of the last frame: trace, caustics, denoise, display.
    cudaEvent_t ev[5] = {};
    bool ev_valid = false;
    // Per-launch events of the wavefront stages of the last frame.
    std::vector<cudaEvent_t> stage_begin, stage_end;
    std::vector<int> stage_kind;
    StageEvents stage{};
    FrameStreams frame{};  // a wavefront frame's groups and their shadow rays
    SideStream caustic{};  // a frame's light tracing and photon gathering

    int fail(int code, const char* fmt, ...) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        error = buf;
        return code;
    }
    int cuda_fail(cudaError_t e, const char* what) {
        return fail(e == cudaErrorMemoryAllocation ? RAYMOND_ENOMEM : RAYMOND_ECUDA, "%s: %s", what,
                    cudaGetErrorString(e));
    }

    unsigned* status_word() const { return static_cast<unsigned*>(counter.ptr) + 8; }

    // The scene as the kernels see it; `one_kernel` says which path walks it
    // (the automatic tree choice differs per path).
    Scene scene_view(bool one_kernel = false) const {
        Scene s{};
        s.prims = static_cast<const float4*>(prims.ptr);
        s.nodes = static_cast<const float4*>(nodes.ptr);
        const bool use_wide = bvh_width == 4 || (bvh_width == 0 && !one_kernel);
        s.wide = has_wide && use_wide ? static_cast<const float4*>(wide.ptr) : nullptr;
        s.materials = static_cast<const float4*>(materials.ptr);
        s.attributes = static_cast<const float4*>(attributes.ptr);
        s.lights = static_cast<const uint32_t*>(lights.ptr);
        s.emitters = static_cast<const float4*>(emitters.ptr);
        s.textures = static_cast<const uchar4*>(textures.ptr);
        s.normal_maps = static_cast<const uchar4*>(normal_maps.ptr);
        s.tex_w = tex_w;
        s.tex_h = tex_h;
        s.tex_layers = tex_layers;
        s.nrm_w = nrm_w;
        s.nrm_h = nrm_h;
        s.nrm_layers = nrm_layers;
        s.env_map = static_cast<const ushort4*>(env_map.ptr);
        s.env_table = static_cast<const float*>(env_table.ptr);
        s.env_w = env_w;
        s.env_h = env_h;
        s.env_cw = env_cw;
        s.env_ch = env_ch;
        s.prim_count = bvh_prim_count;
        s.seed_hash = seed_hash;
        return s;
    }
    PixelBuffers pixel_view() const {
        PixelBuffers p{};
        p.accum = static_cast<float4*>(accum.ptr);
        p.guide_albedo = static_cast<float4*>(guide_albedo.ptr);
        p.guide_normal = static_cast<float4*>(guide_normal.ptr);
        p.light_a = static_cast<float4*>(light_a.ptr);
        p.light_b = static_cast<float4*>(light_b.ptr);
        p.guide_unit = static_cast<float4*>(guide_unit.ptr);
        p.denoised = static_cast<float4*>(denoised.ptr);
        p.splats = static_cast<uint32_t*>(splats.ptr);
        p.display = static_cast<uchar4*>(display.ptr);
        return p;
    }
};

namespace {

int upload(raymond* h, DevBuf& buf, const void* src, size_t bytes, const char* what) {
    cudaError_t e = buf.reserve(bytes);
    if (e != cudaSuccess) return h->cuda_fail(e, what);
    if (bytes > 0) {
        e = cudaMemcpyAsync(buf.ptr, src, bytes, cudaMemcpyHostToDevice, h->stream);
        if (e != cudaSuccess) return h->cuda_fail(e, what);
    }
    return RAYMOND_OK;
}

thread_local std::string g_create_error;

}  // namespace

void rmd::set_handleless_error(const char* msg) { g_create_error = msg; }

namespace {

// The shadow records and lists of both bounce parities, for a pool of cap paths.
void set_shadow_buffers(raymond* h, uint64_t cap, WavefrontState& w) {
    w.shadow[0] = static_cast<float4*>(h->wf_shadow.ptr);
    w.shadow[1] = w.shadow[0] + cap * 3;
    w.shadow_list[0] = static_cast<uint32_t*>(h->wf_shadow_list.ptr);
    w.shadow_list[1] = w.shadow_list[0] + cap;
    w.shadow_sum = static_cast<float4*>(h->wf_shadow_sum.ptr);
}

// Paths in flight for a frame: the whole frame if it fits the limit, else
// whole samples of it (at least one).
int ensure_wavefront(raymond* h, const Params& P, WavefrontState& w) {
    const uint64_t pixels = uint64_t(P.width) * P.height;
    const uint64_t limit = h->path_capacity_limit ? h->path_capacity_limit : (8ull << 20);
    uint64_t samples = limit / pixels;
    if (samples < 1) samples = 1;
    if (samples > P.samples_per_frame) samples = P.samples_per_frame;
    const uint64_t cap = samples * pixels;
    if (cap > h->wf_capacity) {
        cudaError_t e = cudaSuccess;
        for (DevBuf& b : h->wf_state)
            if (e == cudaSuccess) e = b.reserve(cap * 16);
        if (e == cudaSuccess) e = h->wf_hit.reserve(cap * 16);
        if (e == cudaSuccess) e = h->wf_queue[0].reserve(cap * 4);
        if (e == cudaSuccess) e = h->wf_queue[1].reserve(cap * 4);
        if (e == cudaSuccess) e = h->wf_sorted.reserve(cap * 4);
        if (e == cudaSuccess) e = h->wf_sort_key.reserve(cap * 4);
        if (e == cudaSuccess) e = h->wf_shadow.reserve(cap * 96);
        if (e == cudaSuccess) e = h->wf_shadow_list.reserve(cap * 8);
        if (e == cudaSuccess) e = h->wf_shadow_sum.reserve(cap * 16);
        if (e == cudaSuccess) e = h->wf_counters.reserve(256 * FrameStreams::kGroups);
        if (e != cudaSuccess) return h->cuda_fail(e, "wavefront state");
        h->wf_capacity = cap;
    }
    for (int k = 0; k < 8; ++k) w.s[k] = static_cast<float4*>(h->wf_state[k].ptr);
    w.hit = static_cast<float4*>(h->wf_hit.ptr);
    w.queue[0] = static_cast<uint32_t*>(h->wf_queue[0].ptr);
    w.queue[1] = static_cast<uint32_t*>(h->wf_queue[1].ptr);
    w.sorted = static_cast<uint32_t*>(h->wf_sorted.ptr);
    w.sort_key = static_cast<uint32_t*>(h->wf_sort_key.ptr);
    set_shadow_buffers(h, cap, w);
    w.counters = static_cast<uint32_t*>(h->wf_counters.ptr);
    w.capacity = cap;
    return RAYMOND_OK;
}

}  // namespace

extern "C" {

int raymond_create(raymond_t** out, const raymond_config* cfg) {
    if (!out) return RAYMOND_EINVAL;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        g_create_error = std::string("No CUDA device: ") + cudaGetErrorString(e);
        return RAYMOND_ECUDA;
    }
    const int dev = cfg ? cfg->device : 0;
    if (dev < 0 || dev >= count) {
        g_create_error = "No such CUDA device.";
        return RAYMOND_EINVAL;
    }
    e = cudaSetDevice(dev);
    if (e != cudaSuccess) {
        g_create_error = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
        return RAYMOND_ECUDA;
    }
    raymond* h = new (std::nothrow) raymond();
    if (!h) return RAYMOND_ENOMEM;
    h->device = dev;
    cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, dev);
    h->seed_hash = (cfg && cfg->seed) ? pcg(cfg->seed) : 0u;
    h->path_capacity_limit = cfg ? cfg->path_capacity : 0;
    e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        g_create_error = std::string("cudaStreamCreate: ") + cudaGetErrorString(e);
        delete h;
        return RAYMOND_ECUDA;
    }
    for (cudaEvent_t& ev : h->ev) cudaEventCreate(&ev);
    cudaEventCreateWithFlags(&h->order, cudaEventDisableTiming);
    e = cudaEventCreateWithFlags(&h->frame.fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->caustic.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->caustic.fork, cudaEventDisableTiming);
    for (cudaEvent_t& ev : h->caustic.join)
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    for (int g = 0; g < FrameStreams::kGroups; ++g) {
        SideStream& sd = h->frame.side[g];
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->frame.group[g], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->frame.join[g], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sd.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sd.fork, cudaEventDisableTiming);
        for (cudaEvent_t& ev : sd.join)
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        g_create_error = std::string("cudaStreamCreate: ") + cudaGetErrorString(e);
        raymond_destroy(h);
        return RAYMOND_ECUDA;
    }
    h->stage_begin.resize(raymond_stage_events);
    h->stage_end.resize(raymond_stage_events);
    h->stage_kind.resize(raymond_stage_events);
    for (int k = 0; k < raymond_stage_events; ++k) {
        cudaEventCreate(&h->stage_begin[k]);
        cudaEventCreate(&h->stage_end[k]);
    }
    h->stage = StageEvents{h->stage_begin.data(), h->stage_end.data(), h->stage_kind.data(), raymond_stage_events, 0};
    e = h->counter.reserve(64);  // word 0: trace work counter; word 8: status of bounded waits
    if (e == cudaSuccess) e = cudaMemset(h->counter.ptr, 0, 64);
    if (e != cudaSuccess) {
        g_create_error = std::string("cudaMalloc: ") + cudaGetErrorString(e);
        cudaStreamDestroy(h->stream);
        delete h;
        return RAYMOND_ENOMEM;
    }
    for (cudaError_t (*up)() : {upload_srgb_table_trace, upload_srgb_table_wavefront, upload_srgb_table_caustics}) {
        e = up();
        if (e != cudaSuccess) {
            g_create_error = std::string("texture tables: ") + cudaGetErrorString(e);
            raymond_destroy(h);
            return RAYMOND_ECUDA;
        }
    }
    *out = h;
    return RAYMOND_OK;
}

void raymond_destroy(raymond_t* h) {
    if (!h) return;
    cudaSetDevice(h->device);
    // Every stream that may still run the handle's kernels, before its memory goes.
    cudaStreamSynchronize(h->stream);
    for (int g = 0; g < FrameStreams::kGroups; ++g) {
        if (h->frame.group[g]) cudaStreamSynchronize(h->frame.group[g]);
        if (h->frame.side[g].stream) cudaStreamSynchronize(h->frame.side[g].stream);
    }
    if (h->caustic.stream) cudaStreamSynchronize(h->caustic.stream);
    for (cudaStream_t sg : h->b_group_stream)
        if (sg) cudaStreamSynchronize(sg);
    for (DevBuf* b : {&h->prims, &h->nodes, &h->materials, &h->attributes, &h->lights, &h->emitters, &h->textures,
                      &h->normal_maps, &h->env_map, &h->env_table, &h->accum, &h->guide_albedo, &h->guide_normal,
                      &h->light_a, &h->light_b, &h->guide_unit, &h->denoised, &h->splats, &h->display, &h->ray_scratch,
                      &h->prim_scratch, &h->t_scratch, &h->counter, &h->gathered, &h->upload_scratch, &h->wf_hit, &h->wf_queue[0], &h->wf_queue[1],
                      &h->wf_sorted, &h->wf_sort_key, &h->wf_shadow, &h->wf_shadow_list, &h->wf_shadow_sum, &h->wf_counters, &h->photon_heads,
                      &h->photons, &h->wide})
        b->release();
    for (DevBuf& b : h->wf_state) b.release();
    for (cudaEvent_t ev : h->ev)
        if (ev) cudaEventDestroy(ev);
    if (h->b_graph) cudaGraphExecDestroy(h->b_graph);
    if (h->b_copy_done) cudaEventDestroy(h->b_copy_done);
    if (h->b_fork) cudaEventDestroy(h->b_fork);
    for (int g = 0; g < raymond::kBatchGroups; ++g) {
        if (h->b_join[g]) cudaEventDestroy(h->b_join[g]);
        if (h->b_group_stream[g]) cudaStreamDestroy(h->b_group_stream[g]);
    }
    if (h->order) cudaEventDestroy(h->order);
    if (h->frame.fork) cudaEventDestroy(h->frame.fork);
    if (h->caustic.fork) cudaEventDestroy(h->caustic.fork);
    for (cudaEvent_t ev : h->caustic.join)
        if (ev) cudaEventDestroy(ev);
    if (h->caustic.stream) cudaStreamDestroy(h->caustic.stream);
    for (int g = 0; g < FrameStreams::kGroups; ++g) {
        const SideStream& sd = h->frame.side[g];
        if (h->frame.join[g]) cudaEventDestroy(h->frame.join[g]);
        if (h->frame.group[g]) cudaStreamDestroy(h->frame.group[g]);
        if (sd.fork) cudaEventDestroy(sd.fork);
        for (cudaEvent_t ev : sd.join)
            if (ev) cudaEventDestroy(ev);
        if (sd.stream) cudaStreamDestroy(sd.stream);
    }
    if (h->b_staging) cudaFreeHost(h->b_staging);
    for (DevBuf* b : {&h->b_jobs, &h->b_segments, &h->b_jobpix}) b->release();
    for (cudaEvent_t ev : h->stage_begin) cudaEventDestroy(ev);
    for (cudaEvent_t ev : h->stage_end) cudaEventDestroy(ev);
    cudaStreamDestroy(h->stream);
    delete h;
}

const char* raymond_last_error(raymond_t* h) { return h ? h->error.c_str() : g_create_error.c_str(); }

int raymond_upload_scene(raymond_t* h, const void* prims, uint32_t prim_slots, uint32_t bvh_prim_count,
                         const void* nodes, uint32_t node_count, const void* materials, uint32_t mat_count,
                         const float* attributes, uint32_t attr_vec4s, const uint32_t* lights, uint32_t words,
                         uint32_t light_count, uint32_t volume_count) {
    if (!h) return RAYMOND_EINVAL;
    if (!prims || !nodes || !materials || prim_slots == 0 || node_count == 0 || mat_count == 0)
        return h->fail(RAYMOND_EINVAL, "The scene needs primitives, nodes and materials.");
    if (bvh_prim_count > prim_slots || prim_slots - (bvh_prim_count > 0 ? bvh_prim_count : 1) < volume_count)
        return h->fail(RAYMOND_EINVAL, "Primitive counts don't add up.");
    if (uint64_t(light_count) * 2 + volume_count > words || (words > 0 && !lights))
        return h->fail(RAYMOND_EINVAL, "The lights list is too short.");
    if (attr_vec4s > 0 && !attributes) return h->fail(RAYMOND_EINVAL, "Missing attributes.");

    // Validate every index the kernels follow, so no kernel reads out of
    // bounds or loops: children come after their parent, leaves lie within
    // the BVH's primitives.
    const uint32_t leaf_limit = bvh_prim_count > 0 ? bvh_prim_count : 1;
    const uint32_t* nu = static_cast<const uint32_t*>(nodes);
    for (uint32_t i = 0; i < node_count; ++i) {
        const uint32_t first = nu[size_t(i) * 8 + 3], count = nu[size_t(i) * 8 + 7];
        if (count > 0) {
            if (uint64_t(first) + count > leaf_limit)
                return h->fail(RAYMOND_EINVAL, "Node %u's leaf runs past the primitives.", i);
        } else if (first <= i || uint64_t(first) + 1 >= node_count) {
            return h->fail(RAYMOND_EINVAL, "Node %u's children are out of range.", i);
        }
    }
    const uint32_t* pu = static_cast<const uint32_t*>(prims);
    for (uint32_t i = 0; i < prim_slots; ++i) {
        const uint32_t kind = pu[size_t(i) * 16], mat = pu[size_t(i) * 16 + 1], attr = pu[size_t(i) * 16 + 3];
        if (kind == NONE) continue;
        if (kind > TRIANGLE) return h->fail(RAYMOND_EINVAL, "Primitive %u has an unknown kind %u.", i, kind);
        if (mat >= mat_count) return h->fail(RAYMOND_EINVAL, "Primitive %u's material is out of range.", i);
        if (attr != NONE && uint64_t(attr) + 4 > attr_vec4s)
            return h->fail(RAYMOND_EINVAL, "Primitive %u's attributes are out of range.", i);
        const uint32_t light = pu[size_t(i) * 16 + 2];
        if (light != NONE && light >= light_count)
            return h->fail(RAYMOND_EINVAL, "Primitive %u's light index is out of range.", i);
    }
    for (uint32_t k = 0; k < light_count + volume_count; ++k) {
        if (lights[k] >= prim_slots) return h->fail(RAYMOND_EINVAL, "Light or volume %u is out of range.", k);
        const uint32_t kind = pu[size_t(lights[k]) * 16];
        if (kind != SPHERE && kind != QUAD && !(k >= light_count && kind == BOX))
            return h->fail(RAYMOND_EINVAL, "Light or volume %u has the wrong kind.", k);
    }

    cudaSetDevice(h->device);
    int rc;
    if ((rc = upload(h, h->prims, prims, size_t(prim_slots) * 64, "primitives"))) return rc;
    if ((rc = upload(h, h->nodes, nodes, size_t(node_count) * 32, "nodes"))) return rc;
    {
        std::vector<float> wide;
        h->has_wide = build_wide_bvh(nu, node_count, wide);
        if (h->has_wide && (rc = upload(h, h->wide, wide.data(), wide.size() * sizeof(float), "wide tree"))) return rc;
    }
    if ((rc = upload(h, h->materials, materials, size_t(mat_count) * 96, "materials"))) return rc;
    const float zero4[4] = {0, 0, 0, 0};
    if ((rc = upload(h, h->attributes, attr_vec4s ? (const void*)attributes : (const void*)zero4,
                     size_t(attr_vec4s ? attr_vec4s : 1) * 16, "attributes")))
        return rc;
    const uint32_t none = NONE;
    if ((rc = upload(h, h->lights, words ? (const void*)lights : (const void*)&none, size_t(words ? words : 1) * 4,
                     "lights")))
        return rc;
    // Stand-ins for unbound textures and environment, as the reference binds 1×1 ones.
    if (!h->textures.ptr) {
        const uint8_t white[4] = {255, 255, 255, 255};
        if ((rc = upload(h, h->textures, white, 4, "textures"))) return rc;
        if ((rc = upload(h, h->normal_maps, white, 4, "normal maps"))) return rc;
    }
    if (!h->env_map.ptr) {
        const uint16_t black[4] = {0, 0, 0, 0x3c00};
        const float t[1] = {0.0f};
        if ((rc = upload(h, h->env_map, black, 8, "environment"))) return rc;
        if ((rc = upload(h, h->env_table, t, 4, "environment table"))) return rc;
    }
    if (!h->emitters.ptr) {
        const float e[4] = {0, 0, 0, 0};
        if ((rc = upload(h, h->emitters, e, 16, "emitters"))) return rc;
    }
    h->prim_slots = prim_slots;
    h->bvh_prim_count = bvh_prim_count;
    h->node_count = node_count;
    h->mat_count = mat_count;
    h->attr_vec4s = attr_vec4s;
    h->light_words = words;
    h->light_count = light_count;
    h->volume_count = volume_count;
    h->has_scene = true;
    h->rendered = false;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "upload");
    return RAYMOND_OK;
}

int raymond_upload_textures(raymond_t* h, int which, const uint8_t* rgba, uint32_t w, uint32_t hgt,
                            uint32_t layers) {
    if (!h) return RAYMOND_EINVAL;
    if (!rgba || w == 0 || hgt == 0 || layers == 0 || (which != 0 && which != 1))
        return h->fail(RAYMOND_EINVAL, "Textures need a size, layers and data.");
    cudaSetDevice(h->device);
    DevBuf& buf = which == 0 ? h->textures : h->normal_maps;
    int rc = upload(h, buf, rgba, size_t(w) * hgt * layers * 4, "textures");
    if (rc) return rc;
    if (which == 0) {
        h->tex_w = w;
        h->tex_h = hgt;
        h->tex_layers = layers;
    } else {
        h->nrm_w = w;
        h->nrm_h = hgt;
        h->nrm_layers = layers;
    }
    cudaError_t e = cudaStreamSynchronize(h->stream);
    return e == cudaSuccess ? RAYMOND_OK : h->cuda_fail(e, "textures");
}

int raymond_upload_environment(raymond_t* h, const uint16_t* rgba16f, uint32_t w, uint32_t hgt, const float* table,
                               uint32_t cw, uint32_t ch_plus_1) {
    if (!h) return RAYMOND_EINVAL;
    if (!rgba16f || !table || w == 0 || hgt == 0 || cw == 0 || ch_plus_1 == 0)
        return h->fail(RAYMOND_EINVAL, "The environment needs a map and a table.");
    cudaSetDevice(h->device);
    int rc = upload(h, h->env_map, rgba16f, size_t(w) * hgt * 8, "environment");
    if (rc) return rc;
    rc = upload(h, h->env_table, table, size_t(cw) * ch_plus_1 * 4, "environment table");
    if (rc) return rc;
    h->env_w = w;
    h->env_h = hgt;
    h->env_cw = cw;
    h->env_ch = ch_plus_1 - 1;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    return e == cudaSuccess ? RAYMOND_OK : h->cuda_fail(e, "environment");
}

int raymond_upload_texture_images(raymond_t* h, int which, const uint8_t* const* images, const uint32_t* widths,
                                  const uint32_t* heights, uint32_t count, int srgb, const double* decode256) {
    if (!h) return RAYMOND_EINVAL;
    if (!images || !widths || !heights || !decode256 || count == 0 || (which != 0 && which != 1))
        return h->fail(RAYMOND_EINVAL, "Textures need images, sizes and a decoding table.");
    uint32_t w = 0, hgt = 0;
    size_t total = 0;
    for (uint32_t k = 0; k < count; ++k) {
        if (!images[k] || widths[k] == 0 || heights[k] == 0 || widths[k] > 16384 || heights[k] > 16384)
            return h->fail(RAYMOND_EINVAL, "Texture %u has no data or a size outside 1..16384.", k);
        w = std::max(w, widths[k]);
        hgt = std::max(hgt, heights[k]);
        total += size_t(widths[k]) * heights[k] * 4;
    }
    // The array's layers take the largest width and height, at most 2048 (src/Renderer.mjs:637-661).
    w = std::min(w, 2048u);
    hgt = std::min(hgt, 2048u);
    cudaSetDevice(h->device);
    DevBuf& buf = which == 0 ? h->textures : h->normal_maps;
    cudaError_t e = buf.reserve(size_t(w) * hgt * 4 * count);
    if (e == cudaSuccess) e = h->upload_scratch.reserve(256 * sizeof(double) + total);
    if (e != cudaSuccess) return h->cuda_fail(e, "texture array");
    uint8_t* stage = static_cast<uint8_t*>(h->upload_scratch.ptr);
    double* decode = reinterpret_cast<double*>(stage);
    e = cudaMemcpyAsync(decode, decode256, 256 * sizeof(double), cudaMemcpyHostToDevice, h->stream);
    size_t at = 256 * sizeof(double);
    for (uint32_t k = 0; k < count && e == cudaSuccess; ++k) {
        const size_t bytes = size_t(widths[k]) * heights[k] * 4;
        e = cudaMemcpyAsync(stage + at, images[k], bytes, cudaMemcpyHostToDevice, h->stream);
        if (e != cudaSuccess) break;
        launch_texture_layer(stage + at, widths[k], heights[k], static_cast<uint8_t*>(buf.ptr) + size_t(w) * hgt * 4 * k,
                             w, hgt, srgb, decode, h->num_sms, h->stream);
        at += bytes;
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "texture array");
    if (which == 0) {
        h->tex_w = w;
        h->tex_h = hgt;
        h->tex_layers = count;
    } else {
        h->nrm_w = w;
        h->nrm_h = hgt;
        h->nrm_layers = count;
    }
    return RAYMOND_OK;
}

int raymond_upload_environment_rgb(raymond_t* h, const float* rgb, uint32_t w, uint32_t hgt, const double* row_sines,
                                   uint32_t rows) {
    if (!h) return RAYMOND_EINVAL;
    if (!rgb || !row_sines || w == 0 || hgt == 0 || w > 16384 || hgt > 16384)
        return h->fail(RAYMOND_EINVAL, "The environment needs a map of 1..16384 pixels a side and its rows' sines.");
    const uint32_t cw = std::min(w, 512u), ch = std::min(std::min(hgt, 256u), cw);
    if (rows != ch) return h->fail(RAYMOND_EINVAL, "The table has %u rows of cells; %u sines were given.", ch, rows);
    cudaSetDevice(h->device);
    const size_t n = size_t(w) * hgt;
    const size_t rgb_bytes = (n * 12 + 7) & ~size_t(7);  // then the sines and the rows' totals, 8-byte aligned
    cudaError_t e = h->env_map.reserve(n * 8);
    if (e == cudaSuccess) e = h->env_table.reserve(size_t(cw) * (ch + 1) * 4);
    if (e == cudaSuccess) e = h->upload_scratch.reserve(rgb_bytes + size_t(ch) * 16);
    if (e != cudaSuccess) return h->cuda_fail(e, "environment");
    float* d_rgb = static_cast<float*>(h->upload_scratch.ptr);
    double* d_sines = reinterpret_cast<double*>(static_cast<uint8_t*>(h->upload_scratch.ptr) + rgb_bytes);
    double* d_rows = d_sines + ch;
    e = cudaMemcpyAsync(d_rgb, rgb, n * 12, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_sines, row_sines, size_t(ch) * 8, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->env_table.ptr, 0, size_t(cw) * (ch + 1) * 4, h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "environment");
    launch_environment(d_rgb, w, hgt, cw, ch, d_sines, static_cast<uint16_t*>(h->env_map.ptr),
                       static_cast<float*>(h->env_table.ptr), d_rows, h->num_sms, h->stream);
    if ((e = cudaGetLastError()) == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "environment");
    h->env_w = w;
    h->env_h = hgt;
    h->env_cw = cw;
    h->env_ch = ch;
    return RAYMOND_OK;
}

int raymond_read_textures(raymond_t* h, int which, uint8_t* out, uint64_t bytes) {
    if (!h) return RAYMOND_EINVAL;
    if (which != 0 && which != 1) return h->fail(RAYMOND_EINVAL, "which is 0 (colour) or 1 (normal maps).");
    const size_t need = which == 0 ? size_t(h->tex_w) * h->tex_h * 4 * h->tex_layers
                                   : size_t(h->nrm_w) * h->nrm_h * 4 * h->nrm_layers;
    if (!out || bytes < need) return h->fail(RAYMOND_EINVAL, "The texture array needs %zu bytes.", need);
    cudaSetDevice(h->device);
    const DevBuf& buf = which == 0 ? h->textures : h->normal_maps;
    cudaError_t e = need ? cudaMemcpyAsync(out, buf.ptr, need, cudaMemcpyDeviceToHost, h->stream) : cudaSuccess;
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    return e == cudaSuccess ? RAYMOND_OK : h->cuda_fail(e, "texture read-back");
}

int raymond_read_environment(raymond_t* h, uint16_t* rgba16f, uint64_t map_bytes, float* table, uint64_t table_bytes) {
    if (!h) return RAYMOND_EINVAL;
    if (h->env_ch == 0) return h->fail(RAYMOND_ESTATE, "No environment has been uploaded.");
    const size_t map = size_t(h->env_w) * h->env_h * 8, tab = size_t(h->env_cw) * (h->env_ch + 1) * 4;
    if (!rgba16f || !table || map_bytes < map || table_bytes < tab)
        return h->fail(RAYMOND_EINVAL, "The environment needs %zu and %zu bytes.", map, tab);
    cudaSetDevice(h->device);
    cudaError_t e = cudaMemcpyAsync(rgba16f, h->env_map.ptr, map, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(table, h->env_table.ptr, tab, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    return e == cudaSuccess ? RAYMOND_OK : h->cuda_fail(e, "environment read-back");
}

int raymond_set_emitters(raymond_t* h, const float* data, uint32_t vec4_count) {
    if (!h) return RAYMOND_EINVAL;
    if (!data || vec4_count == 0) return h->fail(RAYMOND_EINVAL, "Emitters need data.");
    cudaSetDevice(h->device);
    int rc = upload(h, h->emitters, data, size_t(vec4_count) * 16, "emitters");
    if (rc) return rc;
    h->emitter_vec4s = vec4_count;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    return e == cudaSuccess ? RAYMOND_OK : h->cuda_fail(e, "emitters");
}

int raymond_resize(raymond_t* h, uint32_t w, uint32_t hgt) {
    if (!h) return RAYMOND_EINVAL;
    if (w == 0 || hgt == 0) return h->fail(RAYMOND_EINVAL, "The image needs at least one pixel.");
    cudaSetDevice(h->device);
    const uint64_t px = uint64_t(w) * hgt;
    if (px > h->capacity) {
        // Buffers kept while big enough (src/Renderer.mjs:766-778).
        for (DevBuf* b : {&h->accum, &h->guide_albedo, &h->guide_normal, &h->light_a, &h->light_b, &h->guide_unit,
                          &h->denoised,
                          &h->splats}) {
            cudaError_t e = b->reserve(px * 16);
            if (e != cudaSuccess) return h->cuda_fail(e, "pixel buffers");
        }
        cudaError_t e = h->display.reserve(px * 4);
        if (e != cudaSuccess) return h->cuda_fail(e, "display buffer");
        cudaMemsetAsync(h->splats.ptr, 0, px * 16, h->stream);
        h->capacity = px;
    }
    h->width = w;
    h->height = hgt;
    h->rendered = false;
    return RAYMOND_OK;
}

// The photon map (grown to the capacity asked for, its table at least twice
// that and 2^20) and the frame's light-path count and photon radius.
static int caustic_buffers(raymond_t* h, Params& P, CausticBuffers& cb) {
    if (h->emitter_vec4s == 0) return h->fail(RAYMOND_ESTATE, "Caustics need raymond_set_emitters first.");
    uint32_t table = 1u << 20;
    while (table < 2ull * h->photon_capacity) table <<= 1;
    if (table != h->photon_table || h->photon_capacity != h->photon_capacity_alloc) {
        cudaError_t e = h->photon_heads.reserve((size_t(table) + 1) * 4);
        if (e == cudaSuccess) e = h->photons.reserve(size_t(h->photon_capacity) * 48);
        if (e != cudaSuccess) return h->cuda_fail(e, "photon map");
        h->photon_table = table;
        h->photon_capacity_alloc = h->photon_capacity;
    }
    if (cudaError_t e = h->gathered.reserve(size_t(P.width) * P.height * 16); e != cudaSuccess)
        return h->cuda_fail(e, "gather terms");
    cb.gathered = static_cast<float4*>(h->gathered.ptr);
    cb.splats = static_cast<uint32_t*>(h->splats.ptr);
    cb.heads = static_cast<uint32_t*>(h->photon_heads.ptr);
    cb.photons = static_cast<float4*>(h->photons.ptr);
    cb.table = h->photon_table;
    cb.capacity = h->photon_capacity;
    const uint64_t frame = uint64_t(P.width) * P.height * P.samples_per_frame;
    cb.photons_per_frame = h->photons_override ? h->photons_override
                                               : uint32_t(frame < h->photon_capacity ? frame : h->photon_capacity);
    if (h->photon_radius_override > 0.0f) {
        P.photon_radius = h->photon_radius_override;
        P.photon_cell = 2.0f * h->photon_radius_override;
    }
    return RAYMOND_OK;
}

// The checks raymond_render makes of a frame's parameters.
static int check_frame(raymond_t* h, const void* params208, Params& P) {
    if (!params208) return h->fail(RAYMOND_EINVAL, "No parameters.");
    if (!h->has_scene) return h->fail(RAYMOND_ESTATE, "No scene has been uploaded.");
    std::memcpy(&P, params208, sizeof P);
    if (P.width != h->width || P.height != h->height || h->capacity == 0)
        return h->fail(RAYMOND_ESTATE, "Resize to %ux%u before rendering at that size.", P.width, P.height);
    if (P.light_count != h->light_count || P.volume_count != h->volume_count)
        return h->fail(RAYMOND_EINVAL, "The parameters' light and volume counts don't match the scene.");
    if (P.samples_per_frame == 0 || P.max_bounces > 64)
        return h->fail(RAYMOND_EINVAL, "samples_per_frame must be at least 1 and max_bounces at most 64.");
    return RAYMOND_OK;
}

int raymond_light_trace(raymond_t* h, const void* params208, uint32_t features, uint32_t* splats, uint64_t splat_bytes,
                        float* photons, uint64_t photon_floats, uint32_t* photon_count) {
    if (!h) return RAYMOND_EINVAL;
    Params P;
    int rc = check_frame(h, params208, P);
    if (rc) return rc;
    const size_t px = size_t(P.width) * P.height;
    if (!splats || !photon_count || splat_bytes < px * 16)
        return h->fail(RAYMOND_EINVAL, "The splat buffer needs width x height x 16 bytes.");
    cudaSetDevice(h->device);
    CausticBuffers cb{};
    if ((rc = caustic_buffers(h, P, cb))) return rc;
    cudaMemsetAsync(cb.splats, 0, px * 16, h->stream);
    launch_light_trace_alone(h->scene_view(), P, features, cb, h->num_sms, h->stream);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return h->cuda_fail(e, "light tracing");
    uint32_t attempted = 0;
    e = cudaMemcpyAsync(&attempted, cb.heads + cb.table, 4, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(splats, cb.splats, px * 16, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "light tracing read-back");
    const uint32_t count = attempted < cb.capacity ? attempted : cb.capacity;
    *photon_count = count;
    if (photons && count) {
        if (photon_floats < uint64_t(count) * 11)
            return h->fail(RAYMOND_ECAPACITY, "%u photons need %llu floats.", count,
                           (unsigned long long)(uint64_t(count) * 11));
        std::vector<float4> rec(size_t(count) * 3);
        e = cudaMemcpy(rec.data(), cb.photons, rec.size() * 16, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return h->cuda_fail(e, "photon read-back");
        for (uint32_t i = 0; i < count; ++i) {
            const float4 a = rec[size_t(i) * 3], b = rec[size_t(i) * 3 + 1], c = rec[size_t(i) * 3 + 2];
            const float row[11] = {a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z, b.w, c.w};
            std::memcpy(photons + size_t(i) * 11, row, sizeof row);
        }
    }
    // The splat buffer starts the next frame empty, as a frame leaves it.
    cudaMemsetAsync(cb.splats, 0, px * 16, h->stream);
    return RAYMOND_OK;
}

int raymond_photon_gather(raymond_t* h, const void* params208, uint32_t features, const float* photons, uint32_t n,
                          float* out, uint64_t out_bytes) {
    if (!h) return RAYMOND_EINVAL;
    Params P;
    int rc = check_frame(h, params208, P);
    if (rc) return rc;
    const size_t px = size_t(P.width) * P.height;
    if (!out || out_bytes < px * 16 || (n && !photons))
        return h->fail(RAYMOND_EINVAL, "The output needs width x height x 16 bytes.");
    if (n > h->photon_capacity) return h->fail(RAYMOND_ECAPACITY, "More photons than the map's capacity.");
    cudaSetDevice(h->device);
    CausticBuffers cb{};
    if ((rc = caustic_buffers(h, P, cb))) return rc;
    std::vector<float4> rec(size_t(n) * 3);
    for (uint32_t i = 0; i < n; ++i) {
        const float* q = photons + size_t(i) * 9;
        rec[size_t(i) * 3] = make_float4(q[0], q[1], q[2], 0.0f);
        rec[size_t(i) * 3 + 1] = make_float4(q[3], q[4], q[5], 0.0f);
        rec[size_t(i) * 3 + 2] = make_float4(q[6], q[7], q[8], 0.0f);
    }
    cudaError_t e = h->prim_scratch.reserve(px * 16);
    if (e != cudaSuccess) return h->cuda_fail(e, "gather output");
    float4* d_out = static_cast<float4*>(h->prim_scratch.ptr);
    if (n) e = cudaMemcpyAsync(cb.photons, rec.data(), rec.size() * 16, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_out, 0, px * 16, h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "gather input");
    launch_gather_alone(h->scene_view(), P, features, cb, n, d_out, h->num_sms, h->stream);
    if ((e = cudaGetLastError()) != cudaSuccess) return h->cuda_fail(e, "gather");
    e = cudaMemcpyAsync(out, d_out, px * 16, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    return e == cudaSuccess ? RAYMOND_OK : h->cuda_fail(e, "gather read-back");
}

int raymond_render(raymond_t* h, const void* params208, uint32_t features, uint32_t flags) {
    if (!h) return RAYMOND_EINVAL;
    Params P;
    if (const int rc = check_frame(h, params208, P)) return rc;
    cudaSetDevice(h->device);
    // The wavefront runs colour frames when asked; inspection views always
    // take the one-kernel path.
    const bool want_wf = (flags & RAYMOND_FLAG_WAVEFRONT) ||
                         (!(flags & RAYMOND_FLAG_MEGAKERNEL) && h->path_choice == RAYMOND_PATH_WAVEFRONT);
    const bool wavefront = P.view == VIEW_COLOR && want_wf;
    const Scene s = h->scene_view(!wavefront);
    const PixelBuffers px = h->pixel_view();
    WavefrontState w{};
    if (wavefront) {
        const int rc = ensure_wavefront(h, P, w);
        if (rc) return rc;
    }
    CausticBuffers cb{};
    if (P.caustics != 0u) {
        const int rc = caustic_buffers(h, P, cb);
        if (rc) return rc;
    }
    int launches = 0;
    cudaEventRecord(h->ev[0], h->stream);
    h->stage.count = 0;
    if (P.caustics != 0u) {
        // Light tracing and the gather beside the camera paths (they read
        // nothing of them); the resolve below waits for both.
        cudaEventRecord(h->caustic.fork, h->stream);
        cudaStreamWaitEvent(h->caustic.stream, h->caustic.fork, 0);
        launches += launch_caustic_light(s, P, features, cb, h->num_sms, h->caustic.stream);
        cudaEventRecord(h->caustic.join[0], h->caustic.stream);
    }
    if (wavefront)
        launches += launch_wavefront(s, P, features, w, px, h->tuning, h->num_sms, h->stream, &h->frame, &h->stage);
    else
        launches += launch_megakernel(s, P, features, px, h->num_sms, h->stream);
    cudaEventRecord(h->ev[1], h->stream);
    if (P.caustics != 0u) {
        cudaStreamWaitEvent(h->stream, h->caustic.join[0], 0);
        launches += launch_caustic_resolve(P, cb, px, h->num_sms, h->stream);
    }
    cudaEventRecord(h->ev[2], h->stream);
    if (P.denoise != 0u) launches += launch_denoise(P, px, h->status_word(), h->stream);
    cudaEventRecord(h->ev[3], h->stream);
    launches += launch_tonemap(P, px, h->stream);
    cudaEventRecord(h->ev[4], h->stream);
    h->ev_valid = true;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return h->cuda_fail(e, "render");
    h->last_params = P;
    h->rendered = true;
    h->learned_valid = false;
    h->stats = raymond_stats{};
    h->stats.launches = uint64_t(launches);
    h->stats.paths = uint64_t(P.width) * P.height * P.samples_per_frame;
    return RAYMOND_OK;
}

int raymond_render_batch(raymond_t* h, const raymond_job* jobs, uint32_t n, uint32_t flags) {
    if (!h) return RAYMOND_EINVAL;
    if (!jobs || n == 0 || n > 2048) return h->fail(RAYMOND_EINVAL, "A batch needs 1 to 2048 jobs.");
    cudaSetDevice(h->device);
    std::vector<JobDesc> desc(n);
    std::vector<uint64_t> sig;
    sig.reserve(4 * size_t(n) + 2);
    sig.push_back(n);
    uint64_t total_paths = 0, total_pixels = 0, max_pixels = 0;
    uint32_t max_bounces = 0, features = 0;
    for (uint32_t j = 0; j < n; ++j) {
        raymond* r = jobs[j].renderer;
        if (!r || !jobs[j].params208) return h->fail(RAYMOND_EINVAL, "Job %u has no renderer or parameters.", j);
        if (r->device != h->device) return h->fail(RAYMOND_EINVAL, "Job %u is on another device.", j);
        if (!r->has_scene || r->capacity == 0) return h->fail(RAYMOND_ESTATE, "Job %u has no scene or image.", j);
        Params P;
        std::memcpy(&P, jobs[j].params208, sizeof P);
        if (P.width != r->width || P.height != r->height)
            return h->fail(RAYMOND_ESTATE, "Job %u's parameters don't match its image size.", j);
        if (P.light_count != r->light_count || P.volume_count != r->volume_count)
            return h->fail(RAYMOND_EINVAL, "Job %u's light or volume counts don't match its scene.", j);
        if (P.samples_per_frame == 0 || P.max_bounces > 64 || P.view != VIEW_COLOR)
            return h->fail(RAYMOND_EINVAL, "Job %u: batches render colour frames of 1+ samples, 64 bounces at most.", j);
        const uint64_t pixels = uint64_t(P.width) * P.height;
        if (pixels >= (1u << 21)) return h->fail(RAYMOND_ECAPACITY, "Job %u has more than 2^21 pixels.", j);
        P.caustics = 0;  // no light tracing in a batch: the path tracer keeps every path
        desc[j].scene = r->scene_view();
        desc[j].params = P;
        desc[j].px = r->pixel_view();
        total_paths += pixels * P.samples_per_frame;
        total_pixels += pixels;
        if (pixels > max_pixels) max_pixels = pixels;
        if (P.max_bounces > max_bounces) max_bounces = P.max_bounces;
        features |= jobs[j].features & 15u;
        sig.push_back(reinterpret_cast<uintptr_t>(r));
        sig.push_back(pixels);
        sig.push_back(P.samples_per_frame);
        sig.push_back(P.max_bounces | (uint64_t(P.width) << 32));
    }
    if (total_pixels > 0xffffffffull) return h->fail(RAYMOND_ECAPACITY, "The batch has too many pixels.");
    sig.push_back(features);

    // Path pool: the whole frame if memory allows, else waves of whole samples.
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    // state records, hit, two queues, shading order and key, shadow rays and
    // lists of both parities, shadow sum
    const uint64_t per_path = 8 * 16 + 16 + 4 * 4 + 2 * 48 + 2 * 4 + 16;
    uint64_t cap = uint64_t(double(free_b) * 0.5) / per_path;
    if (h->path_capacity_limit) cap = std::min<uint64_t>(cap, h->path_capacity_limit);
    cap = std::min<uint64_t>(cap, total_paths);
    cap = std::min<uint64_t>(cap, 0x7fffffffull);
    if (cap < max_pixels) cap = max_pixels;
    sig.push_back(cap);

    if (sig != h->b_signature) {
        if (h->b_graph) {
            cudaGraphExecDestroy(h->b_graph);
            h->b_graph = nullptr;
        }
        // Groups: jobs dealt to the least-loaded group, largest first; each
        // group's jobs keep their order.
        const uint32_t groups = std::min<uint32_t>(raymond::kBatchGroups, n);
        std::vector<uint32_t> group_of(n), by_size(n);
        std::vector<uint64_t> load(groups, 0);
        for (uint32_t j = 0; j < n; ++j) by_size[j] = j;
        auto paths_of = [&](uint32_t j) {
            return uint64_t(desc[j].params.width) * desc[j].params.height * desc[j].params.samples_per_frame;
        };
        std::stable_sort(by_size.begin(), by_size.end(), [&](uint32_t a, uint32_t b) { return paths_of(a) > paths_of(b); });
        for (uint32_t j : by_size) {
            const uint32_t g = uint32_t(std::min_element(load.begin(), load.end()) - load.begin());
            group_of[j] = g;
            load[g] += paths_of(j);
        }
        const uint64_t group_cap = std::max<uint64_t>(cap / groups, max_pixels);
        // Plan: per group, its jobs' samples in order, packed into waves of group_cap paths.
        std::vector<WaveSegment> segs;
        std::vector<WavePlan> waves;
        std::vector<uint32_t> group_first(groups), group_waves(groups);
        for (uint32_t g = 0; g < groups; ++g) {
            group_first[g] = uint32_t(waves.size());
            WavePlan cur{uint32_t(segs.size()), 0, 0, 0};
            for (uint32_t j = 0; j < n; ++j) {
                if (group_of[j] != g) continue;
                const uint32_t pixels = desc[j].params.width * desc[j].params.height;
                uint32_t k = 0;
                while (k < desc[j].params.samples_per_frame) {
                    const uint64_t room = (group_cap - cur.paths) / pixels;
                    if (room == 0) {
                        waves.push_back(cur);
                        cur = WavePlan{uint32_t(segs.size()), 0, 0, 0};
                        continue;
                    }
                    const uint32_t nk = uint32_t(std::min<uint64_t>(desc[j].params.samples_per_frame - k, room));
                    segs.push_back(WaveSegment{j, k, nk, pixels, cur.paths, cur.pixels});
                    cur.segments++;
                    cur.paths += nk * pixels;
                    cur.pixels += pixels;
                    k += nk;
                }
            }
            if (cur.segments) waves.push_back(cur);
            group_waves[g] = uint32_t(waves.size()) - group_first[g];
        }
        std::vector<JobPixels> jp(n);
        uint32_t off = 0;
        for (uint32_t j = 0; j < n; ++j) {
            jp[j] = JobPixels{j, off};
            off += desc[j].params.width * desc[j].params.height;
        }
        cudaError_t e = h->b_segments.reserve(segs.size() * sizeof(WaveSegment));
        if (e == cudaSuccess) e = h->b_jobpix.reserve(n * sizeof(JobPixels));
        if (e == cudaSuccess) e = h->b_jobs.reserve(n * sizeof(JobDesc));
        if (e == cudaSuccess)
            e = cudaMemcpy(h->b_segments.ptr, segs.data(), segs.size() * sizeof(WaveSegment), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(h->b_jobpix.ptr, jp.data(), n * sizeof(JobPixels), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return h->cuda_fail(e, "batch plan");
        // The pool: every group's slice, as for a single frame of that many paths.
        const uint64_t pool = group_cap * groups;
        if (pool > h->wf_capacity) {
            for (DevBuf& b : h->wf_state)
                if (e == cudaSuccess) e = b.reserve(pool * 16);
            if (e == cudaSuccess) e = h->wf_hit.reserve(pool * 16);
            if (e == cudaSuccess) e = h->wf_queue[0].reserve(pool * 4);
            if (e == cudaSuccess) e = h->wf_queue[1].reserve(pool * 4);
            if (e == cudaSuccess) e = h->wf_sorted.reserve(pool * 4);
            if (e == cudaSuccess) e = h->wf_sort_key.reserve(pool * 4);
            if (e == cudaSuccess) e = h->wf_shadow.reserve(pool * 96);
            if (e == cudaSuccess) e = h->wf_shadow_list.reserve(pool * 8);
            if (e == cudaSuccess) e = h->wf_shadow_sum.reserve(pool * 16);
            if (e == cudaSuccess) e = h->wf_counters.reserve(256 * raymond::kBatchGroups);
            if (e != cudaSuccess) return h->cuda_fail(e, "batch path pool");
            h->wf_capacity = pool;
        }
        if (n > h->b_staging_cap) {
            if (h->b_staging) cudaFreeHost(h->b_staging);
            h->b_staging = nullptr;
            if ((e = cudaMallocHost(&h->b_staging, n * sizeof(JobDesc))) != cudaSuccess)
                return h->cuda_fail(e, "batch staging");
            h->b_staging_cap = n;
        }
        if (!h->b_copy_done) cudaEventCreateWithFlags(&h->b_copy_done, cudaEventDisableTiming);
        if (!h->b_fork) {
            e = cudaEventCreateWithFlags(&h->b_fork, cudaEventDisableTiming);
            for (int g = 0; g < raymond::kBatchGroups && e == cudaSuccess; ++g) {
                e = cudaEventCreateWithFlags(&h->b_join[g], cudaEventDisableTiming);
                if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->b_group_stream[g], cudaStreamNonBlocking);
            }
            if (e != cudaSuccess) return h->cuda_fail(e, "batch streams");
        }
        h->b_waves = waves;
        h->b_group_first = group_first;
        h->b_group_waves = group_waves;
        h->b_group_cap = group_cap;
        h->b_signature = sig;
        h->b_max_bounces = max_bounces;
        h->b_total_pixels = uint32_t(total_pixels);
        h->b_n = n;
        h->b_paths = total_paths;
    }

    // Work already enqueued on a job renderer's own stream (a learned denoise
    // reading its sums, a read-back) comes before this frame.
    for (uint32_t j = 0; j < n; ++j) {
        raymond* r = jobs[j].renderer;
        if (r == h) continue;
        cudaEventRecord(r->order, r->stream);
        cudaStreamWaitEvent(h->stream, r->order, 0);
    }
    // This frame's job table: the previous frame's copy must have left the staging buffer.
    if (h->b_copy_pending) cudaEventSynchronize(h->b_copy_done);
    std::memcpy(h->b_staging, desc.data(), n * sizeof(JobDesc));
    cudaError_t e = cudaMemcpyAsync(h->b_jobs.ptr, h->b_staging, n * sizeof(JobDesc), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "batch job table");
    cudaEventRecord(h->b_copy_done, h->stream);
    h->b_copy_pending = true;

    WavefrontState w{};
    for (int k = 0; k < 8; ++k) w.s[k] = static_cast<float4*>(h->wf_state[k].ptr);
    w.hit = static_cast<float4*>(h->wf_hit.ptr);
    w.queue[0] = static_cast<uint32_t*>(h->wf_queue[0].ptr);
    w.queue[1] = static_cast<uint32_t*>(h->wf_queue[1].ptr);
    w.sorted = static_cast<uint32_t*>(h->wf_sorted.ptr);
    w.sort_key = static_cast<uint32_t*>(h->wf_sort_key.ptr);
    set_shadow_buffers(h, h->wf_capacity, w);
    w.counters = static_cast<uint32_t*>(h->wf_counters.ptr);
    w.capacity = h->wf_capacity;
    const JobDesc* d_jobs = static_cast<const JobDesc*>(h->b_jobs.ptr);
    const WaveSegment* d_segs = static_cast<const WaveSegment*>(h->b_segments.ptr);
    const JobPixels* d_pix = static_cast<const JobPixels*>(h->b_jobpix.ptr);
    auto enqueue = [&]() {
        int launches = 0;
        const uint32_t groups = uint32_t(h->b_group_first.size());
        cudaEventRecord(h->b_fork, h->stream);
        for (uint32_t g = 0; g < groups; ++g) {
            // The group's slice of the pool, with its own counters.
            const WavefrontState wg = pool_slice(w, h->b_group_cap * g, g, h->b_group_cap);
            cudaStream_t sg = h->b_group_stream[g];
            cudaStreamWaitEvent(sg, h->b_fork, 0);
            launches += launch_wavefront_batch(d_jobs, d_segs, h->b_waves.data() + h->b_group_first[g],
                                               h->b_group_waves[g], h->b_max_bounces, features, wg, h->tuning,
                                               h->num_sms, sg);
            cudaEventRecord(h->b_join[g], sg);
            cudaStreamWaitEvent(h->stream, h->b_join[g], 0);
        }
        launches += launch_image_batch(d_jobs, d_pix, h->b_n, h->b_total_pixels, h->num_sms, h->stream);
        return launches;
    };
    int launches = 0;
    cudaEventRecord(h->ev[0], h->stream);
    if (flags & RAYMOND_BATCH_GRAPH) {
        if (!h->b_graph) {
            cudaGraph_t graph = nullptr;
            e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) return h->cuda_fail(e, "batch capture");
            h->b_graph_launches = enqueue();
            e = cudaStreamEndCapture(h->stream, &graph);
            if (e != cudaSuccess) return h->cuda_fail(e, "batch capture");
            e = cudaGraphInstantiate(&h->b_graph, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) {
                h->b_graph = nullptr;
                return h->cuda_fail(e, "batch graph");
            }
        }
        e = cudaGraphLaunch(h->b_graph, h->stream);
        if (e != cudaSuccess) return h->cuda_fail(e, "batch graph launch");
        launches = h->b_graph_launches;
    } else {
        launches = enqueue();
    }
    cudaEventRecord(h->ev[1], h->stream);
    for (int k = 2; k < 5; ++k) cudaEventRecord(h->ev[k], h->stream);
    e = cudaGetLastError();
    if (e != cudaSuccess) return h->cuda_fail(e, "batch");
    h->ev_valid = true;
    h->stage.count = 0;
    // ... and work enqueued on them later comes after it.
    cudaEventRecord(h->order, h->stream);
    for (uint32_t j = 0; j < n; ++j) {
        raymond* r = jobs[j].renderer;
        if (r != h) cudaStreamWaitEvent(r->stream, h->order, 0);
        r->last_params = desc[j].params;
        r->rendered = true;
        r->learned_valid = false;
    }
    h->stats = raymond_stats{};
    h->stats.launches = uint64_t(launches);
    h->stats.paths = h->b_paths;
    return RAYMOND_OK;
}

int raymond_sync(raymond_t* h) {
    if (!h) return RAYMOND_EINVAL;
    cudaSetDevice(h->device);
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "sync");
    unsigned status = 0;
    e = cudaMemcpy(&status, h->status_word(), sizeof status, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return h->cuda_fail(e, "sync");
    if (status) {
        cudaMemset(h->status_word(), 0, sizeof status);
        return h->fail(RAYMOND_ETIMEOUT, "A staged tile's copy did not arrive in time; that pass wrote nothing.");
    }
    return RAYMOND_OK;
}

int raymond_read_pixels(raymond_t* h, float* out_rgba, uint64_t bytes, int denoised, uint32_t samples) {
    if (!h) return RAYMOND_EINVAL;
    if (!h->rendered || samples == 0) return h->fail(RAYMOND_ESTATE, "Nothing has been rendered yet.");
    if (denoised && h->last_params.denoise == 0u && !h->learned_valid)
        return h->fail(RAYMOND_ESTATE, "Only the color view is denoised, with denoise on.");
    const uint64_t need = uint64_t(h->width) * h->height * 16;
    if (!out_rgba || bytes < need) return h->fail(RAYMOND_EINVAL, "The output needs %llu bytes.", (unsigned long long)need);
    cudaSetDevice(h->device);
    const void* from = h->denoised.ptr;
    cudaError_t e = cudaSuccess;
    if (!denoised) {
        // The average, divided on the GPU into scratch.
        e = h->prim_scratch.reserve(need);
        if (e != cudaSuccess) return h->cuda_fail(e, "read pixels");
        launch_average(static_cast<const float4*>(h->accum.ptr), static_cast<float4*>(h->prim_scratch.ptr),
                       uint32_t(need / 16), float(samples), h->num_sms, h->stream);
        from = h->prim_scratch.ptr;
    }
    e = cudaMemcpyAsync(out_rgba, from, need, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "read pixels");
    return RAYMOND_OK;
}

int raymond_denoise_learned(raymond_t* h, raymond_net* net, uint32_t samples, float* out_rgba) {
    if (!h) return RAYMOND_EINVAL;
    if (!net) return h->fail(RAYMOND_EINVAL, "No network.");
    if (!h->rendered || samples == 0) return h->fail(RAYMOND_ESTATE, "Nothing has been rendered yet.");
    if (h->last_params.view != VIEW_COLOR) return h->fail(RAYMOND_ESTATE, "Only the color view is denoised.");
    cudaSetDevice(h->device);
    std::string err;
    const int rc = rmd_net_denoise(net, static_cast<const float*>(h->accum.ptr),
                                   static_cast<const float*>(h->guide_albedo.ptr),
                                   static_cast<const float*>(h->guide_normal.ptr), float(samples), h->width, h->height,
                                   static_cast<float*>(h->denoised.ptr), h->stream, &err);
    if (rc) return h->fail(rc, "%s", err.c_str());
    // The display shows the network's image, tone-mapped as a denoised frame.
    Params P = h->last_params;
    P.denoise = 1u;
    P.total_samples = samples;
    launch_tonemap(P, h->pixel_view(), h->stream);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return h->cuda_fail(e, "learned denoise");
    h->learned_valid = true;
    if (out_rgba) {
        const size_t need = size_t(h->width) * h->height * 16;
        e = cudaMemcpyAsync(out_rgba, h->denoised.ptr, need, cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) return h->cuda_fail(e, "learned denoise read-back");
    }
    return RAYMOND_OK;
}

int raymond_read_guides(raymond_t* h, float* accum, float* guide_albedo, float* guide_normal, uint64_t bytes_each) {
    if (!h) return RAYMOND_EINVAL;
    if (!h->rendered) return h->fail(RAYMOND_ESTATE, "Nothing has been rendered yet.");
    const uint64_t need = uint64_t(h->width) * h->height * 16;
    if (bytes_each < need) return h->fail(RAYMOND_EINVAL, "Each output needs %llu bytes.", (unsigned long long)need);
    cudaSetDevice(h->device);
    cudaError_t e = cudaSuccess;
    if (accum && e == cudaSuccess) e = cudaMemcpyAsync(accum, h->accum.ptr, need, cudaMemcpyDeviceToHost, h->stream);
    if (guide_albedo && e == cudaSuccess)
        e = cudaMemcpyAsync(guide_albedo, h->guide_albedo.ptr, need, cudaMemcpyDeviceToHost, h->stream);
    if (guide_normal && e == cudaSuccess)
        e = cudaMemcpyAsync(guide_normal, h->guide_normal.ptr, need, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    return e == cudaSuccess ? RAYMOND_OK : h->cuda_fail(e, "read guides");
}

int raymond_read_display(raymond_t* h, uint8_t* out_rgba8, uint64_t bytes) {
    if (!h) return RAYMOND_EINVAL;
    if (!h->rendered) return h->fail(RAYMOND_ESTATE, "Nothing has been rendered yet.");
    const uint64_t need = uint64_t(h->width) * h->height * 4;
    if (!out_rgba8 || bytes < need) return h->fail(RAYMOND_EINVAL, "The output needs %llu bytes.", (unsigned long long)need);
    cudaSetDevice(h->device);
    cudaError_t e = cudaMemcpyAsync(out_rgba8, h->display.ptr, need, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    return e == cudaSuccess ? RAYMOND_OK : h->cuda_fail(e, "read display");
}

int raymond_trace_primary_device(raymond_t* h, const float* d_rays, uint32_t n, uint32_t* d_prim, float* d_t) {
    if (!h) return RAYMOND_EINVAL;
    if (!h->has_scene) return h->fail(RAYMOND_ESTATE, "No scene has been uploaded.");
    if (n == 0) return RAYMOND_OK;
    if (!d_rays || !d_prim || !d_t) return h->fail(RAYMOND_EINVAL, "Null buffer.");
    cudaSetDevice(h->device);
    const int launches = launch_trace_primary(h->scene_view(), d_rays, n, d_prim, d_t,
                                              static_cast<uint32_t*>(h->counter.ptr), h->num_sms, h->stream);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return h->cuda_fail(e, "trace");
    h->stats = raymond_stats{};
    h->stats.launches = uint64_t(launches);
    h->stats.rays_primary = n;
    return RAYMOND_OK;
}

int raymond_trace_primary(raymond_t* h, const float* rays, uint32_t n, uint32_t* prim, float* t) {
    if (!h) return RAYMOND_EINVAL;
    if (n == 0) return RAYMOND_OK;
    if (!rays || !prim || !t) return h->fail(RAYMOND_EINVAL, "Null buffer.");
    cudaSetDevice(h->device);
    cudaError_t e;
    if ((e = h->ray_scratch.reserve(size_t(n) * 24)) != cudaSuccess) return h->cuda_fail(e, "ray buffer");
    if ((e = h->prim_scratch.reserve(size_t(n) * 4)) != cudaSuccess) return h->cuda_fail(e, "hit buffer");
    if ((e = h->t_scratch.reserve(size_t(n) * 4)) != cudaSuccess) return h->cuda_fail(e, "hit buffer");
    e = cudaMemcpyAsync(h->ray_scratch.ptr, rays, size_t(n) * 24, cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "ray upload");
    int rc = raymond_trace_primary_device(h, static_cast<const float*>(h->ray_scratch.ptr), n,
                                          static_cast<uint32_t*>(h->prim_scratch.ptr),
                                          static_cast<float*>(h->t_scratch.ptr));
    if (rc) return rc;
    e = cudaMemcpyAsync(prim, h->prim_scratch.ptr, size_t(n) * 4, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(t, h->t_scratch.ptr, size_t(n) * 4, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    return e == cudaSuccess ? RAYMOND_OK : h->cuda_fail(e, "trace read-back");
}

int raymond_sample_streams(raymond_t* h, const uint32_t* pairs, uint32_t n, const uint32_t* dim_ids, uint32_t dims,
                           uint32_t chain, uint32_t seed_hash, float* out) {
    if (!h) return RAYMOND_EINVAL;
    if (n == 0) return RAYMOND_OK;
    if (!pairs || !out || (dims && !dim_ids)) return h->fail(RAYMOND_EINVAL, "Null buffer.");
    if (n > (1u << 20) || dims > 64u || chain > 64u)
        return h->fail(RAYMOND_EINVAL, "At most 2^20 pairs, 64 dimensions and 64 chain draws.");
    cudaSetDevice(h->device);
    const size_t per = 3u * dims + 1u + 2u * chain;
    const size_t in_bytes = size_t(n) * 8 + size_t(dims) * 4;
    cudaError_t e;
    if ((e = h->ray_scratch.reserve(in_bytes)) != cudaSuccess) return h->cuda_fail(e, "stream inputs");
    if ((e = h->prim_scratch.reserve(size_t(n) * per * 4)) != cudaSuccess) return h->cuda_fail(e, "stream outputs");
    uint32_t* d_pairs = static_cast<uint32_t*>(h->ray_scratch.ptr);
    uint32_t* d_dims = d_pairs + size_t(n) * 2;
    e = cudaMemcpyAsync(d_pairs, pairs, size_t(n) * 8, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess && dims) e = cudaMemcpyAsync(d_dims, dim_ids, size_t(dims) * 4, cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "stream inputs");
    float* d_out = static_cast<float*>(h->prim_scratch.ptr);
    launch_sample_streams(d_pairs, n, d_dims, dims, chain, seed_hash, d_out, h->stream);
    if ((e = cudaGetLastError()) != cudaSuccess) return h->cuda_fail(e, "sample streams");
    e = cudaMemcpyAsync(out, d_out, size_t(n) * per * 4, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    return e == cudaSuccess ? RAYMOND_OK : h->cuda_fail(e, "stream read-back");
}

int raymond_get_buffers(raymond_t* h, raymond_buffers* out) {
    if (!h || !out) return RAYMOND_EINVAL;
    out->accum = static_cast<float*>(h->accum.ptr);
    out->guide_albedo = static_cast<float*>(h->guide_albedo.ptr);
    out->guide_normal = static_cast<float*>(h->guide_normal.ptr);
    out->denoised = static_cast<float*>(h->denoised.ptr);
    out->display = static_cast<uint8_t*>(h->display.ptr);
    out->width = h->width;
    out->height = h->height;
    return RAYMOND_OK;
}

int raymond_set_photons(raymond_t* h, uint32_t photons_per_frame, uint32_t capacity, float radius) {
    if (!h) return RAYMOND_EINVAL;
    if (capacity > (1u << 28) || !(radius >= 0.0f))
        return h->fail(RAYMOND_EINVAL, "Photon capacity above 2^28 or a negative radius.");
    h->photons_override = photons_per_frame;
    h->photon_capacity = capacity ? capacity : 524288u;
    h->photon_radius_override = radius;
    return RAYMOND_OK;
}

int raymond_set_tuning(raymond_t* h, const raymond_tuning* t) {
    if (!h || !t) return RAYMOND_EINVAL;
    if ((t->path != RAYMOND_PATH_MEGAKERNEL && t->path != RAYMOND_PATH_WAVEFRONT) || t->steps < 1 || t->steps > 256 ||
        t->traversal_blocks_per_sm < 1 || t->traversal_blocks_per_sm > 16 || t->shade_blocks_per_sm < 1 ||
        t->shade_blocks_per_sm > 64 || (t->bvh_width != 0 && t->bvh_width != 2 && t->bvh_width != 4))
        return h->fail(RAYMOND_EINVAL, "Tuning out of range.");
    h->path_choice = t->path;
    h->bvh_width = t->bvh_width;
    h->tuning = WavefrontTuning{int(t->steps), int(t->traversal_blocks_per_sm), int(t->shade_blocks_per_sm)};
    return RAYMOND_OK;
}

int raymond_get_tuning(raymond_t* h, raymond_tuning* out) {
    if (!h || !out) return RAYMOND_EINVAL;
    out->path = h->path_choice;
    out->steps = uint32_t(h->tuning.steps);
    out->traversal_blocks_per_sm = uint32_t(h->tuning.traversal_blocks_per_sm);
    out->shade_blocks_per_sm = uint32_t(h->tuning.shade_blocks_per_sm);
    out->bvh_width = h->bvh_width;
    return RAYMOND_OK;
}

int raymond_autotune(raymond_t* h, const void* params208, uint32_t features, uint32_t trials, raymond_tuning* best) {
    if (!h || !params208) return RAYMOND_EINVAL;
    if (trials < 1) trials = 1;
    Params P;
    std::memcpy(&P, params208, sizeof P);
    // Trial frames start the image over (sample_offset 0) and skip denoising.
    P.sample_offset = 0;
    P.total_samples = P.samples_per_frame;
    P.denoise = 0;
    std::vector<raymond_tuning> cands;
    for (uint32_t width : {4u, 2u}) {
        if (width == 4u && !h->has_wide) continue;
        cands.push_back({RAYMOND_PATH_MEGAKERNEL, 16, 8, 8, width});
        for (uint32_t steps : {8u, 16u, 32u})
            for (uint32_t blocks : {4u, 8u, 16u}) cands.push_back({RAYMOND_PATH_WAVEFRONT, steps, blocks, 8, width});
    }
    raymond_tuning keep{};
    raymond_get_tuning(h, &keep);
    float best_ms = 1e30f;
    raymond_tuning chosen = keep;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    for (const raymond_tuning& c : cands) {
        int rc = raymond_set_tuning(h, &c);
        if (rc) break;
        // One untimed frame warms caches and allocates the wavefront state.
        rc = raymond_render(h, &P, features, 0);
        if (rc) break;
        cudaEventRecord(a, h->stream);
        for (uint32_t k = 0; k < trials && rc == 0; ++k) rc = raymond_render(h, &P, features, 0);
        cudaEventRecord(b, h->stream);
        if (rc) break;
        if (cudaEventSynchronize(b) != cudaSuccess) break;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, a, b);
        if (ms < best_ms) {
            best_ms = ms;
            chosen = c;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    raymond_set_tuning(h, &chosen);
    h->rendered = false;
    if (best) *best = chosen;
    return best_ms < 1e30f ? RAYMOND_OK : h->fail(RAYMOND_ECUDA, "Autotuning found no working candidate.");
}

void* raymond_get_stream(raymond_t* h) { return h ? static_cast<void*>(h->stream) : nullptr; }

int raymond_get_stats(raymond_t* h, raymond_stats* out) {
    if (!h || !out) return RAYMOND_EINVAL;
    if (h->ev_valid && cudaEventQuery(h->ev[4]) == cudaSuccess) {
        float* ms[4] = {&h->stats.ms_trace, &h->stats.ms_caustics, &h->stats.ms_denoise, &h->stats.ms_display};
        for (int k = 0; k < 4; ++k) cudaEventElapsedTime(ms[k], h->ev[k], h->ev[k + 1]);
        float sums[3] = {0, 0, 0};
        uint32_t counts[3] = {0, 0, 0};
        for (int k = 0; k < h->stage.count; ++k) {
            float t = 0.0f;
            if (cudaEventElapsedTime(&t, h->stage.begin[k], h->stage.end[k]) == cudaSuccess) {
                sums[h->stage.kind[k]] += t;
                counts[h->stage.kind[k]]++;
            }
        }
        h->stats.ms_extend = sums[0];
        h->stats.ms_shade = sums[1];
        h->stats.ms_shadow = sums[2];
        h->stats.launches_extend = counts[0];
        h->stats.launches_shade = counts[1];
        h->stats.launches_shadow = counts[2];
    }
    *out = h->stats;
    return RAYMOND_OK;
}

}  // extern "C"
