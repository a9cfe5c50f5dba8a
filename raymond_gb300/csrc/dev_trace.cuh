// Ray–primitive tests and BVH traversal over the reference's packed records.
//
// The arithmetic of each primitive test is that of the trace shader
// (src/shaders.mjs:262-378) in f32, so hits agree with the reference GPU path
// up to rounding. The traversal is this backend's own. Over the reference's
// binary nodes: one 64-byte load fetches both children of an inner node
// (BVH.build stores them adjacent, src/BVH.mjs:196-204), the nearer is
// entered, the farther pushed onto a per-thread stack kept in shared memory
// (depth-major, so a warp's pushes hit distinct banks) with a local-memory
// tail, and a popped node is re-tested against the current nearest hit
// before it is entered. Over the 4-wide tree derived from them at upload
// (bvh_wide.h), when there is one: see trace_wide.
#pragma once
#include "dev_common.cuh"

namespace rmd {

struct Hit {
    float t;
    uint32_t prim;
    float u, v;
};

// safe() (src/shaders.mjs:363-366): zero components become ±1e-20.
__device__ __forceinline__ float safe1(float d) {
    const float tiny = 1e-20f;
    return fabsf(d) < tiny ? (d >= 0.0f ? tiny : -tiny) : d;
}

__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }

// intersect() (src/shaders.mjs:262-359): t = -1 for no hit in (T_MIN, t_max).
__device__ __forceinline__ float3 intersect_prim(const Scene& s, uint32_t i, float3 o, float3 d, float t_max) {
    const float4* rec = s.prims + size_t(i) * 4;
    const float4 hdr = ldg4(rec);
    const uint32_t kind = __float_as_uint(hdr.x);
    const float3 miss = f3(-1.0f, 0.0f, 0.0f);
    if (kind == TRIANGLE) {
        const float4 a = ldg4(rec + 1), b = ldg4(rec + 2), c = ldg4(rec + 3);
        const float3 v0 = xyz(a);
        const float3 e1 = xyz(b) - v0;
        const float3 e2 = xyz(c) - v0;
        const float3 pv = cross(d, e2);
        const float det = dot(e1, pv);
        if (fabsf(det) < 1e-12f) return miss;
        const float inv_det = 1.0f / det;
        const float3 tv = o - v0;
        const float bu = dot(tv, pv) * inv_det;
        if (bu < 0.0f || bu > 1.0f) return miss;
        const float3 qv = cross(tv, e1);
        const float bv = dot(d, qv) * inv_det;
        if (bv < 0.0f || bu + bv > 1.0f) return miss;
        const float t = dot(e2, qv) * inv_det;
        if (t <= T_MIN || t >= t_max) return miss;
        return f3(t, bu, bv);
    }
    if (kind == SPHERE) {
        const float4 p0 = ldg4(rec + 1);
        const float3 oc = o - xyz(p0);
        const float r = p0.w;
        const float a = dot(d, d);
        const float half_b = dot(oc, d);
        const float c = dot(oc, oc) - r * r;
        const float disc = half_b * half_b - a * c;
        if (disc < 0.0f) return miss;
        const float sq = sqrtf(disc);
        float t = (-half_b - sq) / a;
        if (t <= T_MIN || t >= t_max) {
            t = (-half_b + sq) / a;
            if (t <= T_MIN || t >= t_max) return miss;
        }
        return f3(t, 0.0f, 0.0f);
    }
    if (kind == QUAD) {
        const float4 p0 = ldg4(rec + 1), p1 = ldg4(rec + 2), p2 = ldg4(rec + 3);
        const float3 q = xyz(p0), qu = xyz(p1), qv = xyz(p2);
        const float3 n = cross(qu, qv);
        const float denom = dot(n, d);
        if (fabsf(denom) < 1e-12f) return miss;
        const float t = dot(n, q - o) / denom;
        if (t <= T_MIN || t >= t_max) return miss;
        const float3 h = o + d * t - q;
        const float nn = dot(n, n);
        const float alpha = dot(n, cross(h, qv)) / nn;
        const float beta = dot(n, cross(qu, h)) / nn;
        if (alpha < 0.0f || alpha > 1.0f || beta < 0.0f || beta > 1.0f) return miss;
        return f3(t, alpha, beta);
    }
    if (kind == BOX) {
        const float4 r0 = ldg4(rec + 1), r1 = ldg4(rec + 2), r2 = ldg4(rec + 3);
        const float3 lo = f3(dot(xyz(r0), o) + r0.w, dot(xyz(r1), o) + r1.w, dot(xyz(r2), o) + r2.w);
        const float3 ld = f3(safe1(dot(xyz(r0), d)), safe1(dot(xyz(r1), d)), safe1(dot(xyz(r2), d)));
        const float3 inv = f3(1.0f / ld.x, 1.0f / ld.y, 1.0f / ld.z);
        const float3 t0 = (f3(-1.0f) - lo) * inv;
        const float3 t1 = (f3(1.0f) - lo) * inv;
        const float3 tmn = fmin3(t0, t1), tmx = fmax3(t0, t1);
        const float t_near = fmaxf(fmaxf(tmn.x, tmn.y), tmn.z);
        const float t_far = fminf(fminf(tmx.x, tmx.y), tmx.z);
        if (t_near > t_far) return miss;
        const float t = t_near > T_MIN ? t_near : t_far;
        if (t <= T_MIN || t >= t_max) return miss;
        return f3(t, 0.0f, 0.0f);
    }
    return miss;
}

// slabs() (src/shaders.mjs:370-378): entry distance clamped at 0, or INF.
__device__ __forceinline__ float slab_entry(float4 mn, float4 mx, float3 o, float3 inv, float t_max) {
    const float t0x = (mn.x - o.x) * inv.x, t1x = (mx.x - o.x) * inv.x;
    const float t0y = (mn.y - o.y) * inv.y, t1y = (mx.y - o.y) * inv.y;
    const float t0z = (mn.z - o.z) * inv.z, t1z = (mx.z - o.z) * inv.z;
    const float t_near = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), 0.0f));
    const float t_far = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), t_max));
    return t_near <= t_far ? t_near : INF;
}

// Per-thread traversal stack: SH entries in shared memory (depth-major,
// column threadIdx), the rest in a local array. 64 entries in all, as the
// reference's; a push beyond that is dropped, as there (src/shaders.mjs:428).
template <int SH>
struct TraversalStack {
    uint32_t* col;
    uint32_t stride;
    uint32_t tail[64 - SH];
    __device__ __forceinline__ void push(uint32_t sp, uint32_t v) {
        if (sp < SH) col[sp * stride] = v;
        else tail[sp - SH] = v;
    }
    __device__ __forceinline__ uint32_t at(uint32_t sp) const { return sp < SH ? col[sp * stride] : tail[sp - SH]; }
};

constexpr int STACK_SHARED = 16;

// ---- the 4-wide tree (bvh_wide.h) ----
constexpr uint32_t WIDE_LEAF = 0x80000000u, WIDE_NONE = 0xFFFFFFFFu;
__device__ __forceinline__ uint32_t wide_first(uint32_t ref) { return ref & 0xFFFFFFu; }
__device__ __forceinline__ uint32_t wide_count(uint32_t ref) { return ((ref >> 24) & 127u) + 1u; }

// Entry distances (slab_entry, INF for a miss or an empty slot) of a wide
// node's four children, and their references.
__device__ __forceinline__ void wide_children(const float4* node, float3 o, float3 inv, float t_max, float t[4],
                                              uint32_t ref[4]) {
    const float4 lx = ldg4(node), hx = ldg4(node + 1), ly = ldg4(node + 2), hy = ldg4(node + 3);
    const float4 lz = ldg4(node + 4), hz = ldg4(node + 5), r = ldg4(node + 6);
    ref[0] = __float_as_uint(r.x);
    ref[1] = __float_as_uint(r.y);
    ref[2] = __float_as_uint(r.z);
    ref[3] = __float_as_uint(r.w);
    t[0] = slab_entry(make_float4(lx.x, ly.x, lz.x, 0.0f), make_float4(hx.x, hy.x, hz.x, 0.0f), o, inv, t_max);
    t[1] = slab_entry(make_float4(lx.y, ly.y, lz.y, 0.0f), make_float4(hx.y, hy.y, hz.y, 0.0f), o, inv, t_max);
    t[2] = slab_entry(make_float4(lx.z, ly.z, lz.z, 0.0f), make_float4(hx.z, hy.z, hz.z, 0.0f), o, inv, t_max);
    t[3] = slab_entry(make_float4(lx.w, ly.w, lz.w, 0.0f), make_float4(hx.w, hy.w, hz.w, 0.0f), o, inv, t_max);
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (ref[k] == WIDE_NONE) t[k] = INF;
}

__device__ __forceinline__ void order2(float* t, uint32_t* r, int a, int b) {
    if (t[b] < t[a]) {
        const float tt = t[a];
        t[a] = t[b];
        t[b] = tt;
        const uint32_t rr = r[a];
        r[a] = r[b];
        r[b] = rr;
    }
}
// Nearest first (a five-comparison network).
__device__ __forceinline__ void sort4(float* t, uint32_t* r) {
    order2(t, r, 0, 1);
    order2(t, r, 2, 3);
    order2(t, r, 0, 2);
    order2(t, r, 1, 3);
    order2(t, r, 1, 2);
}

// The wide traversal's stack of (reference, entry distance): SH entries in
// the thread's shared column (two rows each, depth-major), the rest local;
// 64 in all, pushes beyond dropped as in the binary traversal.
template <int SH>
struct WideStack {
    uint32_t* col;
    uint32_t stride;
    uint2 tail[64 - SH];
    __device__ __forceinline__ void push(uint32_t sp, uint2 v) {
        if (sp < SH) {
            col[(2 * sp) * stride] = v.x;
            col[(2 * sp + 1) * stride] = v.y;
        } else {
            tail[sp - SH] = v;
        }
    }
    __device__ __forceinline__ uint2 at(uint32_t sp) const {
        return sp < SH ? make_uint2(col[(2 * sp) * stride], col[(2 * sp + 1) * stride]) : tail[sp - SH];
    }
};
constexpr int WIDE_STACK_SHARED = 8;  // the same shared bytes as the binary stack's 16 entries

// The nearest (or, with ANY_HIT, any) hit through the wide tree: a node's
// four children are tested at once; the nearest is entered and the others
// pushed farthest first with their entry distance, so a popped entry is
// skipped without a load once the nearest hit is closer.
template <bool ANY_HIT>
__device__ __forceinline__ Hit trace_wide(const Scene& s, float3 o, float3 d, float t_max, uint32_t* stack_col,
                                          uint32_t stack_stride) {
    Hit hit{t_max, NONE, 0.0f, 0.0f};
    const float3 inv = f3(1.0f / safe1(d.x), 1.0f / safe1(d.y), 1.0f / safe1(d.z));
    WideStack<WIDE_STACK_SHARED> st;
    st.col = stack_col;
    st.stride = stack_stride;
    uint32_t sp = 0, cur = 0;
    for (;;) {
        bool have = false;
        if (cur & WIDE_LEAF) {
            const uint32_t first = wide_first(cur), end = first + wide_count(cur);
            for (uint32_t i = first; i < end; ++i) {
                const float3 h = intersect_prim(s, i, o, d, hit.t);
                if (h.x > 0.0f) {
                    hit = Hit{h.x, i, h.y, h.z};
                    if (ANY_HIT) return hit;
                }
            }
        } else {
            float t[4];
            uint32_t ref[4];
            wide_children(s.wide + size_t(cur) * 8, o, inv, hit.t, t, ref);
            if (!ANY_HIT) sort4(t, ref);
            int next = -1;
#pragma unroll
            for (int k = 3; k >= 0; --k) {
                if (t[k] >= INF) continue;
                if (next >= 0 && sp < 64u) st.push(sp++, make_uint2(ref[next], __float_as_uint(t[next])));
                next = k;
            }
            if (next >= 0) {
                cur = ref[next];
                have = true;
            }
        }
        while (!have) {
            if (sp == 0) return hit;
            const uint2 e = st.at(--sp);
            if (ANY_HIT || __uint_as_float(e.y) < hit.t) {
                cur = e.x;
                have = true;
            }
        }
    }
}

// The nearest hit in (T_MIN, t_max), or with ANY_HIT the first found
// (occlusion). prim = NONE for a miss; then t = t_max. Walks the 4-wide tree
// when the scene has one, else the reference's binary nodes.
template <bool ANY_HIT>
__device__ __forceinline__ Hit trace_ray(const Scene& s, float3 o, float3 d, float t_max, uint32_t* stack_col,
                                         uint32_t stack_stride, uint32_t* counters = nullptr) {
    if (s.wide) return trace_wide<ANY_HIT>(s, o, d, t_max, stack_col, stack_stride);
    Hit hit{t_max, NONE, 0.0f, 0.0f};
    const float3 inv = f3(1.0f / safe1(d.x), 1.0f / safe1(d.y), 1.0f / safe1(d.z));
    const float4 rmn = ldg4(s.nodes), rmx = ldg4(s.nodes + 1);
    if (slab_entry(rmn, rmx, o, inv, t_max) >= INF) return hit;

    TraversalStack<STACK_SHARED> st;
    st.col = stack_col;
    st.stride = stack_stride;
    uint32_t sp = 0;
    uint32_t first = __float_as_uint(rmn.w), count = __float_as_uint(rmx.w);

    for (;;) {
        bool have = false;
        if (count > 0) {
            for (uint32_t i = first; i < first + count; ++i) {
                const float3 h = intersect_prim(s, i, o, d, hit.t);
                if (h.x > 0.0f) {
                    hit = Hit{h.x, i, h.y, h.z};
                    if (ANY_HIT) return hit;
                }
            }
        } else {
            const float4* pair = s.nodes + size_t(first) * 2;
            const float4 lmn = ldg4(pair), lmx = ldg4(pair + 1), rmn2 = ldg4(pair + 2), rmx2 = ldg4(pair + 3);
            const float tl = slab_entry(lmn, lmx, o, inv, hit.t);
            const float tr = slab_entry(rmn2, rmx2, o, inv, hit.t);
            const bool l_in = tl < INF, r_in = tr < INF;
            if (l_in || r_in) {
                const bool left_near = tl <= tr;
                if (l_in && r_in) {
                    if (sp < 64u) st.push(sp++, left_near ? first + 1 : first);
                }
                const bool take_left = l_in && (left_near || !r_in);
                first = __float_as_uint(take_left ? lmn.w : rmn2.w);
                count = __float_as_uint(take_left ? lmx.w : rmx2.w);
                have = true;
            }
        }
        // Pop until a stacked node still lies in front of the nearest hit.
        while (!have) {
            if (sp == 0) return hit;
            const uint32_t idx = st.at(--sp);
            const float4 mn = ldg4(s.nodes + size_t(idx) * 2), mx = ldg4(s.nodes + size_t(idx) * 2 + 1);
            if (ANY_HIT || slab_entry(mn, mx, o, inv, hit.t) < INF) {
                first = __float_as_uint(mn.w);
                count = __float_as_uint(mx.w);
                have = true;
            }
        }
    }
}

}  // namespace rmd
