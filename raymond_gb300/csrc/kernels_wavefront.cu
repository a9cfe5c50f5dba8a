// The wavefront form of the render path: path state lives in HBM as
// structure-of-arrays float4 records and each bounce runs as three kernels —
// extend (closest hits), shade (one path_step per live path, pushing the
// extension and shadow rays it makes onto queues) and shadow (any-hit
// occlusion, adding the light of unoccluded shadow rays). Traversal kernels
// are persistent: a warp's lanes each hold one ray, run a few traversal
// steps, and lanes whose ray finished refill from the queue together
// (__ballot_sync picks them, one atomicAdd claims their entries), so warps
// stay full while rays of very different lengths drain. Queues are built a
// tile of 2,048 entries at a time, one atomic per tile. Every kernel reads
// its work count from device memory, so a frame's launches never wait on
// the host.
#include "dev_shade.cuh"
#include "kernels.cuh"

namespace rmd {

namespace {

constexpr int WF_BLOCK = 128;
constexpr uint32_t FULL = 0xffffffffu;

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ uint32_t lanemask_lt() { return (1u << lane_id()) - 1u; }

// ---- path state <-> SoA ----
__device__ __forceinline__ void store_path(const WavefrontState& w, uint32_t p, const PathState& ps, uint32_t pixel) {
    w.s[0][p] = make_float4(ps.o.x, ps.o.y, ps.o.z, ps.last_pdf);
    w.s[1][p] = make_float4(ps.d.x, ps.d.y, ps.d.z, ps.travelled);
    w.s[2][p] = make_float4(ps.throughput.x, ps.throughput.y, ps.throughput.z, ps.wavelength);
    w.s[3][p] = make_float4(ps.result.x, ps.result.y, ps.result.z, ps.spectrum_u);
    w.s[4][p] = make_float4(ps.last_p.x, ps.last_p.y, ps.last_p.z, __uint_as_float((ps.depth << 16) | ps.flags));
    w.s[5][p] = make_float4(ps.g_albedo.x, ps.g_albedo.y, ps.g_albedo.z, __uint_as_float(ps.rng.dim));
    w.s[6][p] = ps.g_normal;
    reinterpret_cast<uint4*>(w.s[7])[p] = make_uint4(ps.rng.state, ps.rng.seed, ps.rng.index, pixel);
}
// A bounce's shading reads all but the normal guide (s[6]: only written,
// once, when the path takes its guides) and writes back s[0..5], plus s[6]
// in the bounce that sets the guides: the sample stream's key, index and
// pixel (s[7]) never change after generation, and a camera path's stream
// is Sobol, so its PCG state stays as generated.
__device__ __forceinline__ void store_bounce(const WavefrontState& w, uint32_t p, const PathState& ps,
                                             bool guides_set) {
    w.s[0][p] = make_float4(ps.o.x, ps.o.y, ps.o.z, ps.last_pdf);
    w.s[1][p] = make_float4(ps.d.x, ps.d.y, ps.d.z, ps.travelled);
    w.s[2][p] = make_float4(ps.throughput.x, ps.throughput.y, ps.throughput.z, ps.wavelength);
    w.s[3][p] = make_float4(ps.result.x, ps.result.y, ps.result.z, ps.spectrum_u);
    w.s[4][p] = make_float4(ps.last_p.x, ps.last_p.y, ps.last_p.z, __uint_as_float((ps.depth << 16) | ps.flags));
    w.s[5][p] = make_float4(ps.g_albedo.x, ps.g_albedo.y, ps.g_albedo.z, __uint_as_float(ps.rng.dim));
    if (guides_set) w.s[6][p] = ps.g_normal;
}
__device__ __forceinline__ uint32_t load_path(const WavefrontState& w, uint32_t p, PathState& ps) {
    const float4 a = w.s[0][p], b = w.s[1][p], c = w.s[2][p], d = w.s[3][p], e = w.s[4][p], f = w.s[5][p];
    ps.o = f3(a.x, a.y, a.z);
    ps.last_pdf = a.w;
    ps.d = f3(b.x, b.y, b.z);
    ps.travelled = b.w;
    ps.throughput = f3(c.x, c.y, c.z);
    ps.wavelength = c.w;
    ps.result = f3(d.x, d.y, d.z);
    ps.spectrum_u = d.w;
    ps.last_p = f3(e.x, e.y, e.z);
    const uint32_t df = __float_as_uint(e.w);
    ps.depth = df >> 16;
    ps.flags = df & 0xffffu;
    ps.g_albedo = f3(f.x, f.y, f.z);
    ps.rng.dim = __float_as_uint(f.w);
    ps.g_normal = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const uint4 r = reinterpret_cast<const uint4*>(w.s[7])[p];
    ps.rng.state = r.x;
    ps.rng.seed = r.y;
    ps.rng.index = r.z;
    ps.rng.qmc = true;
    return r.w;
}

// Counters (u32) in w.counters: queue sizes [0], [1], the extension
// kernel's fetch counter [4], the shading-key bucket sizes [8..23] and the
// scatter's bucket cursors [24..39], all of [4..39] zeroed before each
// extension launch; per bounce parity p, the shadow list's size [40 + 2p]
// and the shadow kernel's fetch counter [41 + 2p], zeroed before shading.
enum { C_QUEUE0 = 0, C_QUEUE1 = 1, C_FETCH = 4, C_BUCKET = 8, C_CURSOR = 24, C_SHADOW = 40 };
constexpr int SORT_BUCKETS = 16;
constexpr int C_ZEROED = 4 + 2 * SORT_BUCKETS;  // words from C_FETCH on

// The shade kernel's branch key of a finished ray: 0 for a miss, else the
// material kind and whether the primitive is a triangle (smooth normals and
// attributes to fetch). Shading a queue ordered by it keeps a warp's lanes
// on the same branches.
__device__ __forceinline__ uint32_t shade_key(const Scene& s, uint32_t prim) {
    if (prim == NONE) return 0u;
    const float4 hdr = ldg4(s.prims + size_t(prim) * 4);
    const uint32_t kind = __float_as_uint(hdr.x), mat = __float_as_uint(hdr.y);
    const uint32_t mk = __float_as_uint(ldg4(s.materials + size_t(mat) * 6).w);
    return 2u + 2u * (mk < 6u ? mk : 6u) + (kind == TRIANGLE ? 1u : 0u);
}

// Lanes that finished a ray record its key and count it into its bucket:
// one atomic per distinct key in the warp. All lanes of the warp call it.
__device__ __forceinline__ void bucket_count(const WavefrontState& w, bool finished, uint32_t path, uint32_t key) {
    const uint32_t fin = __ballot_sync(FULL, finished);
    if (!fin) return;
    const uint32_t peers = __match_any_sync(FULL, finished ? key : 0xFFFFFFFFu) & fin;
    if (finished && lane_id() == uint32_t(__ffs(peers) - 1))
        atomicAdd(w.counters + C_BUCKET + key, uint32_t(__popc(peers)));
    if (finished) w.sort_key[path] = key;
}

// Where a path's scene and uniforms come from. A single frame has one of
// each (kernel parameters); a batch looks them up in the job table by the
// job number kept in the top 11 bits of the path's pixel word.
struct SingleCtx {
    Scene s;
    Params P;
    __device__ __forceinline__ uint32_t job_of(uint32_t) const { return 0; }
    __device__ __forceinline__ const Scene& scene(uint32_t) const { return s; }
    __device__ __forceinline__ const Params& params(uint32_t) const { return P; }
    __device__ __forceinline__ uint32_t job_of_path(const WavefrontState&, uint32_t) const { return 0; }
};
struct BatchCtx {
    const JobDesc* jobs;
    __device__ __forceinline__ uint32_t job_of(uint32_t word) const { return word >> 21; }
    __device__ __forceinline__ const Scene& scene(uint32_t j) const { return jobs[j].scene; }
    __device__ __forceinline__ const Params& params(uint32_t j) const { return jobs[j].params; }
    __device__ __forceinline__ uint32_t job_of_path(const WavefrontState& w, uint32_t path) const {
        return reinterpret_cast<const uint4*>(w.s[7])[path].w >> 21;
    }
};

// ---- generate: main()'s per-sample start for a batch of samples ----
// first_sample counts from the frame's first sample (path_begin adds
// sample_offset).
template <uint32_t FEAT>
__global__ void __launch_bounds__(WF_BLOCK) k_wf_generate(Params P, WavefrontState w, uint32_t seed_hash,
                                                          uint32_t first_sample, uint32_t n_paths) {
    const uint32_t pixels = P.width * P.height;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n_paths; p += gridDim.x * blockDim.x) {
        const uint32_t pixel = p % pixels;
        const uint32_t k = first_sample + p / pixels;
        PathState ps;
        path_begin(P, seed_hash, pixel % P.width, pixel / P.width, k, ps);
        store_path(w, p, ps, pixel);
        w.shadow_sum[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        w.queue[0][p] = p;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        w.counters[C_QUEUE0] = n_paths;
        w.counters[C_QUEUE1] = 0;
    }
}

// ---- resumable traversal, for persistent lanes ----
struct Traversal {
    float3 o, d, inv;
    float t, u, v;
    uint32_t prim;
    uint32_t first, count, sp;
};

// Which tree a traversal kernel walks: fixed when a single frame launches it
// (the kernel then holds one traversal loop and its registers), or looked up
// per ray when a batch's jobs may differ.
enum { TREE_ANY = 0, TREE_BINARY = 2, TREE_WIDE = 4 };

template <int TREE>
__device__ __forceinline__ bool walks_wide(const Scene& s) {
    return TREE == TREE_WIDE || (TREE == TREE_ANY && s.wide != nullptr);
}

// Starts a ray; returns false if it misses the root box (then it is done).
// Over the wide tree, `first` holds the reference being visited (the root
// node first; its children's boxes are tested in the first step).
template <int TREE>
__device__ __forceinline__ bool trav_begin(const Scene& s, Traversal& tr, float3 o, float3 d, float t_max) {
    tr.o = o;
    tr.d = d;
    tr.inv = f3(1.0f / safe1(d.x), 1.0f / safe1(d.y), 1.0f / safe1(d.z));
    tr.t = t_max;
    tr.u = tr.v = 0.0f;
    tr.prim = NONE;
    tr.sp = 0;
    if (walks_wide<TREE>(s)) {
        tr.first = 0;
        tr.count = 0;
        return true;
    }
    const float4 mn = ldg4(s.nodes), mx = ldg4(s.nodes + 1);
    if (slab_entry(mn, mx, o, tr.inv, t_max) >= INF) return false;
    tr.first = __float_as_uint(mn.w);
    tr.count = __float_as_uint(mx.w);
    return true;
}

// One wide-node (or leaf) visit, as trace_wide's loop body.
template <bool ANY_HIT>
__device__ __forceinline__ bool trav_step_wide(const Scene& s, Traversal& tr, WideStack<WIDE_STACK_SHARED>& st) {
    bool have = false;
    const uint32_t cur = tr.first;
    if (cur & WIDE_LEAF) {
        const uint32_t first = wide_first(cur), end = first + wide_count(cur);
        for (uint32_t i = first; i < end; ++i) {
            const float3 h = intersect_prim(s, i, tr.o, tr.d, tr.t);
            if (h.x > 0.0f) {
                tr.t = h.x;
                tr.prim = i;
                tr.u = h.y;
                tr.v = h.z;
                if (ANY_HIT) return false;
            }
        }
    } else {
        float t[4];
        uint32_t ref[4];
        wide_children(s.wide + size_t(cur) * 8, tr.o, tr.inv, tr.t, t, ref);
        if (!ANY_HIT) sort4(t, ref);
        int next = -1;
#pragma unroll
        for (int k = 3; k >= 0; --k) {
            if (t[k] >= INF) continue;
            if (next >= 0 && tr.sp < 64u) st.push(tr.sp++, make_uint2(ref[next], __float_as_uint(t[next])));
            next = k;
        }
        if (next >= 0) {
            tr.first = ref[next];
            have = true;
        }
    }
    while (!have) {
        if (tr.sp == 0) return false;
        const uint2 e = st.at(--tr.sp);
        if (ANY_HIT || __uint_as_float(e.y) < tr.t) {
            tr.first = e.x;
            have = true;
        }
    }
    return true;
}

// One node visit; returns false when the ray is finished.
template <bool ANY_HIT, int TREE>
__device__ __forceinline__ bool trav_step(const Scene& s, Traversal& tr, TraversalStack<STACK_SHARED>& st,
                                          WideStack<WIDE_STACK_SHARED>& wst) {
    if (walks_wide<TREE>(s)) return trav_step_wide<ANY_HIT>(s, tr, wst);
    bool have = false;
    if (tr.count > 0) {
        for (uint32_t i = tr.first; i < tr.first + tr.count; ++i) {
            const float3 h = intersect_prim(s, i, tr.o, tr.d, tr.t);
            if (h.x > 0.0f) {
                tr.t = h.x;
                tr.prim = i;
                tr.u = h.y;
                tr.v = h.z;
                if (ANY_HIT) return false;
            }
        }
    } else {
        const float4* pair = s.nodes + size_t(tr.first) * 2;
        const float4 lmn = ldg4(pair), lmx = ldg4(pair + 1), rmn = ldg4(pair + 2), rmx = ldg4(pair + 3);
        const float tl = slab_entry(lmn, lmx, tr.o, tr.inv, tr.t);
        const float trr = slab_entry(rmn, rmx, tr.o, tr.inv, tr.t);
        const bool l_in = tl < INF, r_in = trr < INF;
        if (l_in || r_in) {
            const bool left_near = tl <= trr;
            if (l_in && r_in && tr.sp < 64u) st.push(tr.sp++, left_near ? tr.first + 1 : tr.first);
            const bool take_left = l_in && (left_near || !r_in);
            tr.first = __float_as_uint(take_left ? lmn.w : rmn.w);
            tr.count = __float_as_uint(take_left ? lmx.w : rmx.w);
            have = true;
        }
    }
    while (!have) {
        if (tr.sp == 0) return false;
        const uint32_t idx = st.at(--tr.sp);
        const float4 mn = ldg4(s.nodes + size_t(idx) * 2), mx = ldg4(s.nodes + size_t(idx) * 2 + 1);
        if (ANY_HIT || slab_entry(mn, mx, tr.o, tr.inv, tr.t) < INF) {
            tr.first = __float_as_uint(mn.w);
            tr.count = __float_as_uint(mx.w);
            have = true;
        }
    }
    return true;
}

// ---- extend: closest hits for every path in the queue ----
template <typename Ctx, int TREE>
__global__ void __launch_bounds__(WF_BLOCK) k_wf_extend(Ctx ctx, WavefrontState w, int q, int steps) {
    __shared__ uint32_t stack[STACK_SHARED * WF_BLOCK];
    TraversalStack<STACK_SHARED> st;
    st.col = stack + threadIdx.x;
    st.stride = WF_BLOCK;
    WideStack<WIDE_STACK_SHARED> wst;
    wst.col = st.col;
    wst.stride = WF_BLOCK;
    const uint32_t* queue = w.queue[q];
    const uint32_t n = w.counters[C_QUEUE0 + q];
    uint32_t* fetch = w.counters + C_FETCH + 0;
    Traversal tr;
    uint32_t path = 0, job = 0;
    bool active = false, exhausted = false, finished = false, missed = false;
    for (;;) {
        // Rays finished in the last steps fetch their shading keys together
        // (one load latency for the warp) and count them into the buckets.
        const uint32_t key = finished ? shade_key(ctx.scene(job), tr.prim) : 0u;
        bucket_count(w, finished, path, key);
        finished = false;
        // Lanes without a ray claim the next queue entries together.
        const bool need = !active && !exhausted;
        const uint32_t mask = __ballot_sync(FULL, need);
        if (mask) {
            const uint32_t leader = __ffs(mask) - 1u;
            uint32_t base = 0;
            if (lane_id() == leader) base = atomicAdd(fetch, __popc(mask));
            base = __shfl_sync(FULL, base, leader);
            if (need) {
                const uint32_t idx = base + __popc(mask & lanemask_lt());
                if (idx < n) {
                    path = queue[idx];
                    job = ctx.job_of_path(w, path);
                    const float4 a = w.s[0][path], b = w.s[1][path];
                    active = trav_begin<TREE>(ctx.scene(job), tr, f3(a.x, a.y, a.z), f3(b.x, b.y, b.z), INF);
                    if (!active) w.hit[path] = make_float4(INF, __uint_as_float(NONE), 0.0f, 0.0f);
                    missed = !active;
                } else {
                    exhausted = true;
                }
            }
        }
        bucket_count(w, missed, path, 0u);  // rays that miss the scene's box: key 0
        missed = false;
        if (!__any_sync(FULL, active || !exhausted)) return;
        // A round of `steps` node visits, cut short once no lane holds a ray.
        // (Refilling as soon as 5, 13 or 21 of the 32 lanes had finished
        // was slower: the refills' loads cost more than the idle lanes.)
        const Scene& sc = ctx.scene(job);
        for (int k = 0; k < steps; ++k) {
            if (active && !trav_step<false, TREE>(sc, tr, st, wst)) {
                w.hit[path] = make_float4(tr.t, __uint_as_float(tr.prim), tr.u, tr.v);
                active = false;
                finished = true;
            }
            if (!__any_sync(FULL, active)) break;
        }
    }
}

// ---- queue building in tiles ----
// The scatter and the compaction take the queue in tiles of TILE consecutive
// entries per block (item k of thread t at k·TILE_THREADS + t). Each entry's
// place within its tile's share of an output comes from warp ballots (or
// key matches) and a scan, in shared memory, of the counts of each (item,
// warp) in tile order; the tile then claims its range of the output with one
// atomic per counter. Entries keep their queue order within a tile, and a
// counter takes one atomic per 2,048 entries instead of one per warp.
constexpr int TILE_THREADS = 256, TILE_ITEMS = 8, TILE = TILE_THREADS * TILE_ITEMS;
constexpr int TILE_WARPS = TILE_THREADS / 32, TILE_PARTS = TILE_ITEMS * TILE_WARPS;  // 64 parts
static_assert(TILE_PARTS == 64, "a warp scans a tile's parts two per lane");

// Exclusive scan of part[0..63] in place by one warp; returns the total.
__device__ __forceinline__ uint32_t scan_parts(uint32_t* part) {
    const uint32_t l = lane_id();
    const uint32_t a = part[2 * l], b = part[2 * l + 1];
    uint32_t incl = a + b;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(FULL, incl, o);
        if (l >= uint32_t(o)) incl += v;
    }
    const uint32_t excl = incl - a - b;
    part[2 * l] = excl;
    part[2 * l + 1] = excl + a;
    return __shfl_sync(FULL, incl, 31);
}

// ---- scatter: this bounce's queue in shading-key order ----
// Within a bucket, paths keep their queue order inside each tile, so the
// rays shading emits stay coherent.
__global__ void __launch_bounds__(TILE_THREADS) k_wf_scatter(WavefrontState w, int q) {
    __shared__ uint32_t start[SORT_BUCKETS];  // each bucket's first place in the sorted queue
    __shared__ uint32_t base[SORT_BUCKETS];   // the tile's first place within each bucket
    __shared__ uint32_t part[SORT_BUCKETS][TILE_PARTS];
    if (threadIdx.x == 0) {
        uint32_t sum = 0;
        for (int k = 0; k < SORT_BUCKETS; ++k) {
            start[k] = sum;
            sum += w.counters[C_BUCKET + k];
        }
    }
    const uint32_t n = w.counters[C_QUEUE0 + q];
    const uint32_t* queue = w.queue[q];
    const uint32_t warp = threadIdx.x >> 5;
    for (uint32_t t0 = blockIdx.x * TILE; t0 < n; t0 += gridDim.x * TILE) {
        for (int i = threadIdx.x; i < SORT_BUCKETS * TILE_PARTS; i += TILE_THREADS) (&part[0][0])[i] = 0u;
        __syncthreads();
        uint32_t path[TILE_ITEMS], key[TILE_ITEMS], peers[TILE_ITEMS];
#pragma unroll
        for (int k = 0; k < TILE_ITEMS; ++k) {
            const uint32_t idx = t0 + k * TILE_THREADS + threadIdx.x;
            path[k] = idx < n ? queue[idx] : 0u;
            key[k] = idx < n ? w.sort_key[path[k]] : 0xFFFFFFFFu;
            peers[k] = __match_any_sync(FULL, key[k]);
            if (key[k] != 0xFFFFFFFFu && lane_id() == uint32_t(__ffs(peers[k]) - 1))
                part[key[k]][k * TILE_WARPS + warp] = __popc(peers[k]);
        }
        __syncthreads();
        for (int b = warp; b < SORT_BUCKETS; b += TILE_WARPS) {
            const uint32_t total = scan_parts(part[b]);
            uint32_t at = 0;
            if (lane_id() == 0 && total) at = atomicAdd(w.counters + C_CURSOR + b, total);
            if (lane_id() == 0) base[b] = start[b] + at;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < TILE_ITEMS; ++k)
            if (key[k] != 0xFFFFFFFFu)
                w.sorted[base[key[k]] + part[key[k]][k * TILE_WARPS + warp] + __popc(peers[k] & lanemask_lt())] =
                    path[k];
        __syncthreads();  // the next tile reuses part and base
    }
}

// ---- shade: one bounce of radiance() per live path ----
// Shading runs in key order (the scatter's `sorted` queue) but queues
// nothing: it records per path whether it continues (bit 0) and whether it
// has a shadow ray (bit 1, the ray stored at the path's slot of this bounce
// parity's records), and k_wf_compact builds the next queues in the
// previous queue's order, which keeps neighbouring paths' rays together for
// traversal.
template <uint32_t FEAT, typename Ctx>
__global__ void __launch_bounds__(WF_BLOCK) k_wf_shade(Ctx ctx, WavefrontState w, int q, int par) {
    float4* const shadow = w.shadow[par];
    const uint32_t n = w.counters[C_QUEUE0 + q];
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
        const uint32_t path = w.sorted[idx];
        ShadowRay sh;
        sh.valid = false;
        PathState ps;
        const uint32_t word = load_path(w, path, ps);
        const bool guided = (ps.flags & PF_GUIDED) != 0u;
        const uint32_t job = ctx.job_of(word);
        const float4 hv = w.hit[path];
        const Hit hit{hv.x, __float_as_uint(hv.y), hv.z, hv.w};
        const bool more = path_step<FEAT>(ctx.scene(job), ctx.params(job), ps, hit, sh);
        store_bounce(w, path, ps, !guided && (ps.flags & PF_GUIDED) != 0u);
        w.sort_key[path] = (more ? 1u : 0u) | (sh.valid ? 2u : 0u);
        if (sh.valid) {
            shadow[size_t(path) * 3 + 0] = make_float4(sh.o.x, sh.o.y, sh.o.z, sh.reach);
            shadow[size_t(path) * 3 + 1] = make_float4(sh.d.x, sh.d.y, sh.d.z, __uint_as_float(path));
            shadow[size_t(path) * 3 + 2] =
                make_float4(sh.contribution.x, sh.contribution.y, sh.contribution.z, __uint_as_float(job));
        }
    }
}

// ---- compact: the next extension queue and the shadow list, in queue order ----
__global__ void __launch_bounds__(TILE_THREADS) k_wf_compact(WavefrontState w, int q, int par) {
    __shared__ uint32_t base[2];
    __shared__ uint32_t part[2][TILE_PARTS];  // [0]: paths that continue, [1]: paths with a shadow ray
    const uint32_t n = w.counters[C_QUEUE0 + q];
    const uint32_t* queue = w.queue[q];
    uint32_t* out_queue = w.queue[q ^ 1];
    const uint32_t warp = threadIdx.x >> 5;
    for (uint32_t t0 = blockIdx.x * TILE; t0 < n; t0 += gridDim.x * TILE) {
        uint32_t path[TILE_ITEMS], more[TILE_ITEMS], shadow[TILE_ITEMS];
#pragma unroll
        for (int k = 0; k < TILE_ITEMS; ++k) {
            const uint32_t idx = t0 + k * TILE_THREADS + threadIdx.x;
            path[k] = idx < n ? queue[idx] : 0u;
            const uint32_t f = idx < n ? w.sort_key[path[k]] : 0u;
            more[k] = __ballot_sync(FULL, (f & 1u) != 0u);
            shadow[k] = __ballot_sync(FULL, (f & 2u) != 0u);
            if (lane_id() == 0) {
                part[0][k * TILE_WARPS + warp] = __popc(more[k]);
                part[1][k * TILE_WARPS + warp] = __popc(shadow[k]);
            }
        }
        __syncthreads();
        if (warp < 2) {
            const uint32_t total = scan_parts(part[warp]);
            uint32_t at = 0;
            if (lane_id() == 0 && total)
                at = atomicAdd(w.counters + (warp ? C_SHADOW + 2 * par : C_QUEUE0 + (q ^ 1)), total);
            if (lane_id() == 0) base[warp] = at;
        }
        __syncthreads();
        const uint32_t below = lanemask_lt(), bit = 1u << lane_id();
#pragma unroll
        for (int k = 0; k < TILE_ITEMS; ++k) {
            if (more[k] & bit) out_queue[base[0] + part[0][k * TILE_WARPS + warp] + __popc(more[k] & below)] = path[k];
            if (shadow[k] & bit)
                w.shadow_list[par][base[1] + part[1][k * TILE_WARPS + warp] + __popc(shadow[k] & below)] = path[k];
        }
        __syncthreads();  // the next tile reuses part and base
    }
}

// ---- shadow: any-hit occlusion; unoccluded rays add their light ----
template <typename Ctx, int TREE>
__global__ void __launch_bounds__(WF_BLOCK) k_wf_shadow(Ctx ctx, WavefrontState w, int steps, int par) {
    __shared__ uint32_t stack[STACK_SHARED * WF_BLOCK];
    TraversalStack<STACK_SHARED> st;
    st.col = stack + threadIdx.x;
    st.stride = WF_BLOCK;
    WideStack<WIDE_STACK_SHARED> wst;
    wst.col = st.col;
    wst.stride = WF_BLOCK;
    const uint32_t n = w.counters[C_SHADOW + 2 * par];
    uint32_t* fetch = w.counters + C_SHADOW + 2 * par + 1;
    const uint32_t* list = w.shadow_list[par];
    const float4* shadow = w.shadow[par];
    Traversal tr;
    uint32_t rec = 0, job = 0;
    bool active = false, exhausted = false;
    for (;;) {
        const bool need = !active && !exhausted;
        const uint32_t mask = __ballot_sync(FULL, need);
        if (mask) {
            const uint32_t leader = __ffs(mask) - 1u;
            uint32_t base = 0;
            if (lane_id() == leader) base = atomicAdd(fetch, __popc(mask));
            base = __shfl_sync(FULL, base, leader);
            if (need) {
                const uint32_t idx = base + __popc(mask & lanemask_lt());
                if (idx < n) {
                    rec = list[idx];  // the list holds paths; each path's ray sits at its slot
                    const float4 a = shadow[size_t(rec) * 3], b = shadow[size_t(rec) * 3 + 1];
                    job = __float_as_uint(shadow[size_t(rec) * 3 + 2].w);
                    active = trav_begin<TREE>(ctx.scene(job), tr, f3(a.x, a.y, a.z), f3(b.x, b.y, b.z), a.w);
                    if (!active) {
                        // Misses the scene's box: unoccluded.
                        const float4 c = shadow[size_t(rec) * 3 + 2];
                        const float4 r = w.shadow_sum[rec];
                        w.shadow_sum[rec] = make_float4(r.x + c.x, r.y + c.y, r.z + c.z, 0.0f);
                    }
                } else {
                    exhausted = true;
                }
            }
        }
        if (!__any_sync(FULL, active || !exhausted)) return;
        const Scene& sc = ctx.scene(job);
        for (int k = 0; k < steps; ++k) {
            if (active && !trav_step<true, TREE>(sc, tr, st, wst)) {
                active = false;
                if (tr.prim == NONE) {
                    const float4 c = shadow[size_t(rec) * 3 + 2];
                    const float4 r = w.shadow_sum[rec];
                    w.shadow_sum[rec] = make_float4(r.x + c.x, r.y + c.y, r.z + c.z, 0.0f);
                }
            }
            if (!__any_sync(FULL, active)) break;
        }
    }
}

// ---- finalize: main()'s per-pixel sums for a batch of samples ----
__global__ void __launch_bounds__(WF_BLOCK) k_wf_finalize(Params P, WavefrontState w, PixelBuffers px,
                                                          uint32_t batch_samples, bool overwrite) {
    const uint32_t pixels = P.width * P.height;
    for (uint32_t pixel = blockIdx.x * blockDim.x + threadIdx.x; pixel < pixels; pixel += gridDim.x * blockDim.x) {
        float4 sum = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        float3 sa = f3(0.0f);
        float4 sn = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        for (uint32_t k = 0; k < batch_samples; ++k) {
            const uint32_t p = k * pixels + pixel;
            const float4 rr = w.s[3][p], sr = w.shadow_sum[p];
            float3 c = f3(rr.x + sr.x, rr.y + sr.y, rr.z + sr.z);
            const float peak = maxc(c);
            if (P.firefly_clamp > 0.0f && peak > P.firefly_clamp) c *= P.firefly_clamp / peak;
            const float4 ga = w.s[5][p];
            const float4 gn = w.s[6][p];
            if (finite3(c) && finite3(f3(ga.x, ga.y, ga.z)) && finite3(f3(gn.x, gn.y, gn.z)) && finite1(gn.w)) {
                const float l = luminance(c);
                sum.x += c.x;
                sum.y += c.y;
                sum.z += c.z;
                sum.w += l * l;
                sa += f3(ga.x, ga.y, ga.z);
                sn.x += gn.x;
                sn.y += gn.y;
                sn.z += gn.z;
                sn.w += gn.w;
            }
        }
        if (overwrite) {
            px.accum[pixel] = sum;
            px.guide_albedo[pixel] = make_float4(sa.x, sa.y, sa.z, 0.0f);
            px.guide_normal[pixel] = sn;
        } else {
            const float4 a = px.accum[pixel], g = px.guide_albedo[pixel], nn = px.guide_normal[pixel];
            px.accum[pixel] = make_float4(a.x + sum.x, a.y + sum.y, a.z + sum.z, a.w + sum.w);
            px.guide_albedo[pixel] = make_float4(g.x + sa.x, g.y + sa.y, g.z + sa.z, g.w);
            px.guide_normal[pixel] = make_float4(nn.x + sn.x, nn.y + sn.y, nn.z + sn.z, nn.w + sn.w);
        }
    }
}

struct StageTimer {
    StageEvents* ev;
    cudaStream_t st;
    int slot = -1;
    void begin(int kind, cudaStream_t on) {
        slot = -1;
        st = on;
        if (!ev || ev->count >= ev->capacity) return;
        slot = ev->count++;
        ev->kind[slot] = kind;
        cudaEventRecord(ev->begin[slot], st);
    }
    void end() {
        if (slot >= 0) cudaEventRecord(ev->end[slot], st);
    }
};

// One group's paths through every bounce, on stream st. With a side
// stream, each bounce's shadow rays trace on it while the next bounce
// extends, sorts, shades and compacts on st: the shadow kernel reads only
// its parity's list, records and counters and adds to the paths' shadow
// sums, which nothing else on st touches until the frame's sums, and each
// kernel's tail, where its last rays or paths leave most of the GPU idle,
// is filled by the other stream's blocks. A bounce waits, before it resets
// its parity's shadow list, for the shadow rays of two bounces back, which
// used the same parity. Returns with st waiting for the last shadow rays.
template <uint32_t FEAT>
int wavefront_group(const SingleCtx& ctx, const WavefrontState& w, uint32_t first_sample, uint32_t n,
                    const WavefrontTuning& tune, int num_sms, cudaStream_t st, const SideStream* side,
                    StageTimer& timer) {
    const Params& P = ctx.P;
    const cudaStream_t shadow_st = side ? side->stream : st;
    const bool wide = ctx.s.wide != nullptr;
    const int grid_trav = num_sms * tune.traversal_blocks_per_sm;
    const int grid_shade = num_sms * tune.shade_blocks_per_sm;
    const int grid_tiles = num_sms * 4;
    k_wf_generate<FEAT><<<grid_shade, WF_BLOCK, 0, st>>>(P, w, ctx.s.seed_hash, first_sample, n);
    int launches = 1;
    int q = 0;
    for (uint32_t depth = 0; depth <= P.max_bounces; ++depth) {
        const int par = int(depth & 1u);
        cudaMemsetAsync(w.counters + C_FETCH, 0, C_ZEROED * sizeof(uint32_t), st);
        timer.begin(0, st);
        if (wide)
            k_wf_extend<SingleCtx, TREE_WIDE><<<grid_trav, WF_BLOCK, 0, st>>>(ctx, w, q, tune.steps);
        else
            k_wf_extend<SingleCtx, TREE_BINARY><<<grid_trav, WF_BLOCK, 0, st>>>(ctx, w, q, tune.steps);
        timer.end();
        k_wf_scatter<<<grid_tiles, TILE_THREADS, 0, st>>>(w, q);
        // The next queue and this parity's shadow list start empty.
        cudaMemsetAsync(w.counters + C_QUEUE0 + (q ^ 1), 0, sizeof(uint32_t), st);
        if (side && depth >= 2) cudaStreamWaitEvent(st, side->join[par], 0);
        cudaMemsetAsync(w.counters + C_SHADOW + 2 * par, 0, 2 * sizeof(uint32_t), st);
        timer.begin(1, st);
        k_wf_shade<FEAT, SingleCtx><<<grid_shade, WF_BLOCK, 0, st>>>(ctx, w, q, par);
        timer.end();
        k_wf_compact<<<grid_tiles, TILE_THREADS, 0, st>>>(w, q, par);
        if (side) {
            cudaEventRecord(side->fork, st);
            cudaStreamWaitEvent(shadow_st, side->fork, 0);
        }
        timer.begin(2, shadow_st);
        if (wide)
            k_wf_shadow<SingleCtx, TREE_WIDE><<<grid_trav, WF_BLOCK, 0, shadow_st>>>(ctx, w, tune.steps, par);
        else
            k_wf_shadow<SingleCtx, TREE_BINARY><<<grid_trav, WF_BLOCK, 0, shadow_st>>>(ctx, w, tune.steps, par);
        timer.end();
        if (side) cudaEventRecord(side->join[par], shadow_st);
        launches += 5;
        q ^= 1;
    }
    // The side stream runs its shadow kernels in order: the last one's end is all of theirs.
    if (side) cudaStreamWaitEvent(st, side->join[P.max_bounces & 1u], 0);
    return launches;
}

// A frame: its samples a pool's worth at a time; each pool's paths, with
// streams, as up to FrameStreams::kGroups groups of whole samples, each on
// its own stream, so one group's extension fills the GPU beside another's
// shading. Paths do not depend on one another, so the groups change
// nothing but the order the GPU runs them in.
template <uint32_t FEAT>
int wavefront_frame(const Scene& s, const Params& P, const WavefrontState& w, const PixelBuffers& px,
                    const WavefrontTuning& tune, int num_sms, cudaStream_t st, const FrameStreams* fs,
                    StageEvents* events) {
    StageTimer timer{events, st};
    const SingleCtx ctx{s, P};
    const uint32_t pixels = P.width * P.height;
    const uint32_t batch = uint32_t(w.capacity / pixels) > 0 ? uint32_t(w.capacity / pixels) : 1u;
    const int grid_shade = num_sms * tune.shade_blocks_per_sm;
    int launches = 0;
    for (uint32_t k0 = 0; k0 < P.samples_per_frame; k0 += batch) {
        const uint32_t nk = (P.samples_per_frame - k0) < batch ? (P.samples_per_frame - k0) : batch;
        const uint32_t groups = fs ? (nk < uint32_t(FrameStreams::kGroups) ? nk : uint32_t(FrameStreams::kGroups)) : 1u;
        if (groups == 1) {
            launches += wavefront_group<FEAT>(ctx, w, k0, nk * pixels, tune, num_sms, st, fs ? &fs->side[0] : nullptr,
                                              timer);
        } else {
            cudaEventRecord(fs->fork, st);
            for (uint32_t g = 0; g < groups; ++g) {
                const uint32_t first = g * nk / groups, end = (g + 1) * nk / groups;
                const WavefrontState wg =
                    pool_slice(w, uint64_t(first) * pixels, g, uint64_t(end - first) * pixels);
                cudaStreamWaitEvent(fs->group[g], fs->fork, 0);
                launches += wavefront_group<FEAT>(ctx, wg, k0 + first, (end - first) * pixels, tune, num_sms,
                                                  fs->group[g], &fs->side[g], timer);
                cudaEventRecord(fs->join[g], fs->group[g]);
                cudaStreamWaitEvent(st, fs->join[g], 0);
            }
        }
        k_wf_finalize<<<grid_shade, WF_BLOCK, 0, st>>>(P, w, px, nk, P.sample_offset == 0u && k0 == 0);
        ++launches;
    }
    return launches;
}


// ---- batched frames: many renderers' jobs through one path pool ----

// The segment holding wave path p (segments are in path order).
__device__ __forceinline__ uint32_t find_segment(const WaveSegment* seg, uint32_t n_seg, uint32_t p, bool by_pixel) {
    uint32_t lo = 0, hi = n_seg - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) / 2;
        const uint32_t start = by_pixel ? seg[mid].pixel_offset : seg[mid].path_offset;
        if (start <= p) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(WF_BLOCK) k_wfb_generate(const JobDesc* __restrict__ jobs,
                                                           const WaveSegment* __restrict__ seg, uint32_t n_seg,
                                                           WavefrontState w, uint32_t n_paths) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n_paths; p += gridDim.x * blockDim.x) {
        const WaveSegment g = seg[find_segment(seg, n_seg, p, false)];
        const JobDesc& jd = jobs[g.job];
        const uint32_t local = p - g.path_offset;
        const uint32_t pixel = local % g.pixels;
        const uint32_t k = g.k0 + local / g.pixels;
        PathState ps;
        path_begin(jd.params, jd.scene.seed_hash, pixel % jd.params.width, pixel / jd.params.width, k, ps);
        store_path(w, p, ps, (g.job << 21) | pixel);
        w.shadow_sum[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        w.queue[0][p] = p;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        w.counters[C_QUEUE0] = n_paths;
        w.counters[C_QUEUE1] = 0;
    }
}

__global__ void __launch_bounds__(WF_BLOCK) k_wfb_finalize(const JobDesc* __restrict__ jobs,
                                                           const WaveSegment* __restrict__ seg, uint32_t n_seg,
                                                           WavefrontState w, uint32_t n_pixels) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n_pixels; t += gridDim.x * blockDim.x) {
        const WaveSegment g = seg[find_segment(seg, n_seg, t, true)];
        const JobDesc& jd = jobs[g.job];
        const Params& P = jd.params;
        const uint32_t pixel = t - g.pixel_offset;
        float4 sum = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        float3 sa = f3(0.0f);
        float4 sn = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        for (uint32_t k = 0; k < g.nk; ++k) {
            const uint32_t p = g.path_offset + k * g.pixels + pixel;
            const float4 rr = w.s[3][p], sr = w.shadow_sum[p];
            float3 c = f3(rr.x + sr.x, rr.y + sr.y, rr.z + sr.z);
            const float peak = maxc(c);
            if (P.firefly_clamp > 0.0f && peak > P.firefly_clamp) c *= P.firefly_clamp / peak;
            const float4 ga = w.s[5][p];
            const float4 gn = w.s[6][p];
            if (finite3(c) && finite3(f3(ga.x, ga.y, ga.z)) && finite3(f3(gn.x, gn.y, gn.z)) && finite1(gn.w)) {
                const float l = luminance(c);
                sum.x += c.x;
                sum.y += c.y;
                sum.z += c.z;
                sum.w += l * l;
                sa += f3(ga.x, ga.y, ga.z);
                sn.x += gn.x;
                sn.y += gn.y;
                sn.z += gn.z;
                sn.w += gn.w;
            }
        }
        const PixelBuffers& px = jd.px;
        if (P.sample_offset == 0u && g.k0 == 0u) {
            px.accum[pixel] = sum;
            px.guide_albedo[pixel] = make_float4(sa.x, sa.y, sa.z, 0.0f);
            px.guide_normal[pixel] = sn;
        } else {
            const float4 a = px.accum[pixel], ga2 = px.guide_albedo[pixel], nn = px.guide_normal[pixel];
            px.accum[pixel] = make_float4(a.x + sum.x, a.y + sum.y, a.z + sum.z, a.w + sum.w);
            px.guide_albedo[pixel] = make_float4(ga2.x + sa.x, ga2.y + sa.y, ga2.z + sa.z, ga2.w);
            px.guide_normal[pixel] = make_float4(nn.x + sn.x, nn.y + sn.y, nn.z + sn.z, nn.w + sn.w);
        }
    }
}

}  // namespace

template <uint32_t FEAT>
static int batch_frame(const JobDesc* d_jobs, const WaveSegment* d_segments, const WavePlan* waves, uint32_t n_waves,
                       uint32_t max_bounces, const WavefrontState& w, const WavefrontTuning& tune, int num_sms,
                       cudaStream_t st) {
    const BatchCtx ctx{d_jobs};
    const int grid_trav = num_sms * tune.traversal_blocks_per_sm;
    const int grid_shade = num_sms * tune.shade_blocks_per_sm;
    const int grid_tiles = num_sms * 4;
    int launches = 0;
    for (uint32_t v = 0; v < n_waves; ++v) {
        const WavePlan& wp = waves[v];
        const WaveSegment* seg = d_segments + wp.first_segment;
        k_wfb_generate<<<grid_shade, WF_BLOCK, 0, st>>>(d_jobs, seg, wp.segments, w, wp.paths);
        ++launches;
        int q = 0;
        for (uint32_t depth = 0; depth <= max_bounces; ++depth) {
            cudaMemsetAsync(w.counters + C_FETCH, 0, C_ZEROED * sizeof(uint32_t), st);
            k_wf_extend<BatchCtx, TREE_ANY><<<grid_trav, WF_BLOCK, 0, st>>>(ctx, w, q, tune.steps);
            k_wf_scatter<<<grid_tiles, TILE_THREADS, 0, st>>>(w, q);
            const int par = int(depth & 1u);
            cudaMemsetAsync(w.counters + C_QUEUE0 + (q ^ 1), 0, sizeof(uint32_t), st);
            cudaMemsetAsync(w.counters + C_SHADOW + 2 * par, 0, 2 * sizeof(uint32_t), st);
            k_wf_shade<FEAT, BatchCtx><<<grid_shade, WF_BLOCK, 0, st>>>(ctx, w, q, par);
            k_wf_compact<<<grid_tiles, TILE_THREADS, 0, st>>>(w, q, par);
            k_wf_shadow<BatchCtx, TREE_ANY><<<grid_trav, WF_BLOCK, 0, st>>>(ctx, w, tune.steps, par);
            launches += 5;
            q ^= 1;
        }
        k_wfb_finalize<<<grid_shade, WF_BLOCK, 0, st>>>(d_jobs, seg, wp.segments, w, wp.pixels);
        ++launches;
    }
    return launches;
}

// The shade kernel is compiled for the union of the jobs' features, as a
// single frame's is for its own (no features, volumes, dispersion, or all).
int launch_wavefront_batch(const JobDesc* d_jobs, const WaveSegment* d_segments, const WavePlan* waves,
                           uint32_t n_waves, uint32_t max_bounces, uint32_t features, const WavefrontState& w,
                           const WavefrontTuning& tune, int num_sms, cudaStream_t st) {
    switch (features & 15u) {
        case 0: return batch_frame<0>(d_jobs, d_segments, waves, n_waves, max_bounces, w, tune, num_sms, st);
        case F_VOLUMES:
            return batch_frame<F_VOLUMES>(d_jobs, d_segments, waves, n_waves, max_bounces, w, tune, num_sms, st);
        case F_DISPERSION:
            return batch_frame<F_DISPERSION>(d_jobs, d_segments, waves, n_waves, max_bounces, w, tune, num_sms, st);
        default: return batch_frame<15u>(d_jobs, d_segments, waves, n_waves, max_bounces, w, tune, num_sms, st);
    }
}


cudaError_t upload_srgb_table_wavefront() { return upload_srgb_table_here(); }

int launch_wavefront(const Scene& s, const Params& P, uint32_t features, const WavefrontState& w,
                     const PixelBuffers& px, const WavefrontTuning& tune, int num_sms, cudaStream_t st,
                     const FrameStreams* streams, StageEvents* events) {
    switch (features & 15u) {
        case 0: return wavefront_frame<0>(s, P, w, px, tune, num_sms, st, streams, events);
        case F_VOLUMES: return wavefront_frame<F_VOLUMES>(s, P, w, px, tune, num_sms, st, streams, events);
        case F_DISPERSION: return wavefront_frame<F_DISPERSION>(s, P, w, px, tune, num_sms, st, streams, events);
        default: return wavefront_frame<15u>(s, P, w, px, tune, num_sms, st, streams, events);
    }
}

}  // namespace rmd
