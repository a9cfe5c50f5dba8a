// Scene.raycast restated in double (src/Scene.mjs:202-283, 549-674, 687-750)
// and the trace shader's own traversal restated in f32 (src/shaders.mjs:
// 262-447) — TEST INFRASTRUCTURE ONLY.
#include "oracle.h"

#include <cmath>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

const double kInf = std::numeric_limits<double>::infinity();
const uint32_t SPHERE = 0, QUAD = 1, BOX = 2, TRIANGLE = 3;

struct PrimView {
    const uint32_t* u;
    const float* f;
};

inline PrimView prim(const void* prims, uint32_t p) {
    const uint8_t* b = static_cast<const uint8_t*>(prims) + size_t(p) * 64;
    return {reinterpret_cast<const uint32_t*>(b), reinterpret_cast<const float*>(b)};
}

inline const float* node_f(const void* nodes, uint32_t n) {
    return reinterpret_cast<const float*>(static_cast<const uint8_t*>(nodes) + size_t(n) * 32);
}
inline const uint32_t* node_u(const void* nodes, uint32_t n) {
    return reinterpret_cast<const uint32_t*>(static_cast<const uint8_t*>(nodes) + size_t(n) * 32);
}

// ---- double helpers, Vec3 semantics of src/Vec3.mjs ----
struct D3 {
    double x, y, z;
};
inline D3 d3(const float* f) { return {double(f[0]), double(f[1]), double(f[2])}; }
inline D3 sub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 add(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 scale(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 cross(D3 a, D3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double length(D3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline D3 normalized(D3 a) {
    const double l = length(a);
    return {a.x / l, a.y / l, a.z / l};
}
inline double jmax(double a, double b) { return b > a ? b : a; }
inline double jmin(double a, double b) { return b < a ? b : a; }

// Scene.#slabs (src/Scene.mjs:549-566): entry distance, axes giving NaN skipped.
double slabs_double(const float* f, const double* o, const double* inv) {
    double t_near = 0.0, t_far = kInf;
    for (int a = 0; a < 3; ++a) {
        double t0 = (double(f[a]) - o[a]) * inv[a];
        double t1 = (double(f[4 + a]) - o[a]) * inv[a];
        if (std::isnan(t0) || std::isnan(t1)) continue;
        if (t0 > t1) {
            const double t = t0;
            t0 = t1;
            t1 = t;
        }
        t_near = jmax(t_near, t0);
        t_far = jmin(t_far, t1);
    }
    return t_near <= t_far ? t_near : kInf;
}

// Scene.#normals (src/Scene.mjs:687-750): geometric and shading normals.
void normals_double(const void* prims, const float* attributes, uint32_t p, D3 point, double bu,
                    double bv, D3* geometric, D3* shading) {
    const PrimView pv = prim(prims, p);
    const float* f = pv.f;
    const uint32_t kind = pv.u[0];
    if (kind == SPHERE) {
        const D3 n = normalized(scale(sub(point, d3(f + 4)), 1.0 / double(f[7])));
        *geometric = *shading = n;
        return;
    }
    if (kind == QUAD) {
        const D3 n = normalized(cross(d3(f + 8), d3(f + 12)));
        *geometric = *shading = n;
        return;
    }
    if (kind == BOX) {
        double lp[3];
        for (int r = 0; r < 3; ++r)
            lp[r] = double(f[4 + r * 4]) * point.x + double(f[5 + r * 4]) * point.y +
                    double(f[6 + r * 4]) * point.z + double(f[7 + r * 4]);
        int axis = 0;
        for (int a = 1; a < 3; ++a)
            if (std::fabs(lp[a]) > std::fabs(lp[axis])) axis = a;
        double sign = lp[axis] > 0 ? 1.0 : (lp[axis] < 0 ? -1.0 : 0.0);
        if (sign == 0.0) sign = 1.0;
        const D3 n = normalized(scale(d3(f + 4 + axis * 4), sign));
        *geometric = *shading = n;
        return;
    }
    const D3 v0 = d3(f + 4), v1 = d3(f + 8), v2 = d3(f + 12);
    const D3 g = normalized(cross(sub(v1, v0), sub(v2, v0)));
    *geometric = *shading = g;
    const uint32_t ai = pv.u[3];
    if (ai == RO_NONE) return;
    const int flags = int(attributes[(size_t(ai) + 3) * 4 + 3]);
    if (!(flags & 1)) return;
    auto normal = [&](int k) { return d3(attributes + (size_t(ai) + k) * 4); };
    D3 s = normalized(add(add(scale(normal(0), 1.0 - bu - bv), scale(normal(1), bu)), scale(normal(2), bv)));
    if (dot(s, g) < 0.0) s = scale(s, -1.0);
    *shading = s;
}

// ---- f32 restatement of the trace shader ----
struct F3 {
    float x, y, z;
};
inline F3 f3(const float* f) { return {f[0], f[1], f[2]}; }
inline F3 fsub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline F3 fadd(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline F3 fmul(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline float fdot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline F3 fcross(F3 a, F3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float fminf_(float a, float b) { return a < b ? a : b; }
inline float fmaxf_(float a, float b) { return a > b ? a : b; }

const float T_MIN = 1e-4f;
const float INF32 = 1e30f;

// safe() (src/shaders.mjs:363-366).
inline float safe1(float d) {
    const float tiny = 1e-20f;
    return std::fabs(d) < tiny ? (d >= 0.0f ? tiny : -tiny) : d;
}

// intersect() (src/shaders.mjs:262-359): (t, u, v), t = -1 for a miss.
void intersect32(const void* prims, uint32_t i, F3 o, F3 d, float t_max, float* out) {
    const PrimView p = prim(prims, i);
    out[0] = -1.0f;
    out[1] = out[2] = 0.0f;
    switch (p.u[0]) {
        case SPHERE: {
            const F3 oc = fsub(o, f3(p.f + 4));
            const float r = p.f[7];
            const float a = fdot(d, d);
            const float half_b = fdot(oc, d);
            const float c = fdot(oc, oc) - r * r;
            const float disc = half_b * half_b - a * c;
            if (disc < 0.0f) return;
            const float sq = std::sqrt(disc);
            float t = (-half_b - sq) / a;
            if (t <= T_MIN || t >= t_max) {
                t = (-half_b + sq) / a;
                if (t <= T_MIN || t >= t_max) return;
            }
            out[0] = t;
            return;
        }
        case QUAD: {
            const F3 q = f3(p.f + 4), qu = f3(p.f + 8), qv = f3(p.f + 12);
            const F3 n = fcross(qu, qv);
            const float denom = fdot(n, d);
            if (std::fabs(denom) < 1e-12f) return;
            const float t = fdot(n, fsub(q, o)) / denom;
            if (t <= T_MIN || t >= t_max) return;
            const F3 h = fsub(fadd(o, fmul(d, t)), q);
            const float nn = fdot(n, n);
            const float alpha = fdot(n, fcross(h, qv)) / nn;
            const float beta = fdot(n, fcross(qu, h)) / nn;
            if (alpha < 0.0f || alpha > 1.0f || beta < 0.0f || beta > 1.0f) return;
            out[0] = t;
            out[1] = alpha;
            out[2] = beta;
            return;
        }
        case BOX: {
            float tmin[3], tmax[3];
            for (int r = 0; r < 3; ++r) {
                const F3 row = f3(p.f + 4 + r * 4);
                const float lo = fdot(row, o) + p.f[7 + r * 4];
                const float inv = 1.0f / safe1(fdot(row, d));
                const float t0 = (-1.0f - lo) * inv;
                const float t1 = (1.0f - lo) * inv;
                tmin[r] = fminf_(t0, t1);
                tmax[r] = fmaxf_(t0, t1);
            }
            const float t_near = fmaxf_(fmaxf_(tmin[0], tmin[1]), tmin[2]);
            const float t_far = fminf_(fminf_(tmax[0], tmax[1]), tmax[2]);
            if (t_near > t_far) return;
            const float t = t_near > T_MIN ? t_near : t_far;
            if (t <= T_MIN || t >= t_max) return;
            out[0] = t;
            return;
        }
        case TRIANGLE: {
            const F3 v0 = f3(p.f + 4);
            const F3 e1 = fsub(f3(p.f + 8), v0);
            const F3 e2 = fsub(f3(p.f + 12), v0);
            const F3 pv = fcross(d, e2);
            const float det = fdot(e1, pv);
            if (std::fabs(det) < 1e-12f) return;
            const float inv_det = 1.0f / det;
            const F3 tv = fsub(o, v0);
            const float bu = fdot(tv, pv) * inv_det;
            if (bu < 0.0f || bu > 1.0f) return;
            const F3 qv = fcross(tv, e1);
            const float bv = fdot(d, qv) * inv_det;
            if (bv < 0.0f || bu + bv > 1.0f) return;
            const float t = fdot(e2, qv) * inv_det;
            if (t <= T_MIN || t >= t_max) return;
            out[0] = t;
            out[1] = bu;
            out[2] = bv;
            return;
        }
        default:
            return;
    }
}

// slabs() (src/shaders.mjs:370-378).
inline float slabs32(const float* n, F3 o, F3 inv, float t_max) {
    const float t0x = (n[0] - o.x) * inv.x, t1x = (n[4] - o.x) * inv.x;
    const float t0y = (n[1] - o.y) * inv.y, t1y = (n[5] - o.y) * inv.y;
    const float t0z = (n[2] - o.z) * inv.z, t1z = (n[6] - o.z) * inv.z;
    const float t_near = fmaxf_(fmaxf_(fminf_(t0x, t1x), fminf_(t0y, t1y)), fmaxf_(fminf_(t0z, t1z), 0.0f));
    const float t_far = fminf_(fminf_(fmaxf_(t0x, t1x), fmaxf_(t0y, t1y)), fminf_(fmaxf_(t0z, t1z), t_max));
    return t_near <= t_far ? t_near : INF32;
}

template <typename F>
void parallel_for(uint32_t n, int threads, F fn) {
    if (threads <= 1 || n < 1024) {
        for (uint32_t i = 0; i < n; ++i) fn(i);
        return;
    }
    std::vector<std::thread> pool;
    const uint32_t chunk = (n + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        const uint32_t lo = t * chunk, hi = lo + chunk < n ? lo + chunk : n;
        if (lo >= hi) break;
        pool.emplace_back([=] {
            for (uint32_t i = lo; i < hi; ++i) fn(i);
        });
    }
    for (auto& th : pool) th.join();
}

}  // namespace

// Scene.#intersect (src/Scene.mjs:579-674), in double on the f32-stored record.
extern "C" int ro_intersect_double(const void* prims, uint32_t p, const double* o, const double* d,
                                   double t_max, double* tuv) {
    const PrimView pv = prim(prims, p);
    const float* f = pv.f;
    const uint32_t kind = pv.u[0];
    const double T = 1e-4;
    const D3 O = {o[0], o[1], o[2]}, Dd = {d[0], d[1], d[2]};
    if (kind == SPHERE) {
        const D3 oc = sub(O, d3(f + 4));
        const double r = f[7];
        const double a = dot(Dd, Dd);
        const double half_b = dot(oc, Dd);
        const double c = dot(oc, oc) - r * r;
        const double disc = half_b * half_b - a * c;
        if (disc < 0.0) return 0;
        const double sq = std::sqrt(disc);
        double t = (-half_b - sq) / a;
        if (t <= T || t >= t_max) {
            t = (-half_b + sq) / a;
            if (t <= T || t >= t_max) return 0;
        }
        tuv[0] = t;
        tuv[1] = tuv[2] = 0.0;
        return 1;
    }
    if (kind == QUAD) {
        const D3 q = d3(f + 4), qu = d3(f + 8), qv = d3(f + 12);
        const D3 n = cross(qu, qv);
        const double denom = dot(n, Dd);
        if (std::fabs(denom) < 1e-12) return 0;
        const double t = dot(n, sub(q, O)) / denom;
        if (t <= T || t >= t_max) return 0;
        const D3 h = sub(add(O, scale(Dd, t)), q);
        const double nn = dot(n, n);
        const double alpha = dot(n, cross(h, qv)) / nn;
        const double beta = dot(n, cross(qu, h)) / nn;
        if (alpha < 0.0 || alpha > 1.0 || beta < 0.0 || beta > 1.0) return 0;
        tuv[0] = t;
        tuv[1] = alpha;
        tuv[2] = beta;
        return 1;
    }
    if (kind == BOX) {
        double t_near = -kInf, t_far = kInf;
        for (int a = 0; a < 3; ++a) {
            const double lo = double(f[4 + a * 4]) * o[0] + double(f[5 + a * 4]) * o[1] +
                              double(f[6 + a * 4]) * o[2] + double(f[7 + a * 4]);
            const double ld = double(f[4 + a * 4]) * d[0] + double(f[5 + a * 4]) * d[1] +
                              double(f[6 + a * 4]) * d[2];
            const double inv = 1.0 / ld;
            double t0 = (-1.0 - lo) * inv;
            double t1 = (1.0 - lo) * inv;
            if (std::isnan(t0) || std::isnan(t1)) continue;
            if (t0 > t1) {
                const double t = t0;
                t0 = t1;
                t1 = t;
            }
            t_near = jmax(t_near, t0);
            t_far = jmin(t_far, t1);
        }
        if (t_near > t_far) return 0;
        const double t = t_near > T ? t_near : t_far;
        if (t <= T || t >= t_max) return 0;
        tuv[0] = t;
        tuv[1] = tuv[2] = 0.0;
        return 1;
    }
    if (kind != TRIANGLE) return 0;
    const D3 v0 = d3(f + 4), v1 = d3(f + 8), v2 = d3(f + 12);
    const D3 e1 = sub(v1, v0), e2 = sub(v2, v0);
    const D3 pv_ = cross(Dd, e2);
    const double det = dot(e1, pv_);
    if (std::fabs(det) < 1e-12) return 0;
    const double inv_det = 1.0 / det;
    const D3 tv = sub(O, v0);
    const double bu = dot(tv, pv_) * inv_det;
    if (bu < 0.0 || bu > 1.0) return 0;
    const D3 qv = cross(tv, e1);
    const double bv = dot(Dd, qv) * inv_det;
    if (bv < 0.0 || bu + bv > 1.0) return 0;
    const double t = dot(e2, qv) * inv_det;
    if (t <= T || t >= t_max) return 0;
    tuv[0] = t;
    tuv[1] = bu;
    tuv[2] = bv;
    return 1;
}

extern "C" void ro_raycast_batch(const void* prims, uint32_t prim_count, const void* nodes,
                                 const float* attributes, const float* rays, uint32_t n, double t_max,
                                 uint32_t* prim_out, double* t_out, double* uv_out, double* normal_out,
                                 uint8_t* front_out, int threads) {
    parallel_for(n, threads, [&](uint32_t r) {
        prim_out[r] = RO_NONE;
        t_out[r] = t_max;
        if (uv_out) uv_out[2 * r] = uv_out[2 * r + 1] = 0.0;
        if (normal_out) normal_out[3 * r] = normal_out[3 * r + 1] = normal_out[3 * r + 2] = 0.0;
        if (front_out) front_out[r] = 0;
        if (prim_count == 0) return;  // src/Scene.mjs:205-206

        const double o[3] = {rays[6 * size_t(r)], rays[6 * size_t(r) + 1], rays[6 * size_t(r) + 2]};
        const double d[3] = {rays[6 * size_t(r) + 3], rays[6 * size_t(r) + 4], rays[6 * size_t(r) + 5]};
        const double inv[3] = {1.0 / d[0], 1.0 / d[1], 1.0 / d[2]};

        double best_t = t_max, best_u = 0.0, best_v = 0.0;
        int64_t best = -1;
        std::vector<uint32_t> stack;
        stack.reserve(128);
        stack.push_back(0);
        while (!stack.empty()) {
            const uint32_t nd = stack.back();
            stack.pop_back();
            if (slabs_double(node_f(nodes, nd), o, inv) >= best_t) continue;
            const uint32_t count = node_u(nodes, nd)[7];
            const uint32_t first = node_u(nodes, nd)[3];
            if (count == 0) {
                const double t_left = slabs_double(node_f(nodes, first), o, inv);
                const double t_right = slabs_double(node_f(nodes, first + 1), o, inv);
                if (t_left <= t_right) {
                    stack.push_back(first + 1);
                    stack.push_back(first);
                } else {
                    stack.push_back(first);
                    stack.push_back(first + 1);
                }
                continue;
            }
            for (uint32_t p = first; p < first + count; ++p) {
                double tuv[3];
                if (ro_intersect_double(prims, p, o, d, best_t, tuv)) {
                    best_t = tuv[0];
                    best_u = tuv[1];
                    best_v = tuv[2];
                    best = p;
                }
            }
        }
        if (best < 0) return;
        prim_out[r] = uint32_t(best);
        t_out[r] = best_t;
        if (uv_out) {
            uv_out[2 * r] = best_u;
            uv_out[2 * r + 1] = best_v;
        }
        if (normal_out || front_out) {
            const D3 O = {o[0], o[1], o[2]}, Dd = {d[0], d[1], d[2]};
            const D3 point = add(O, scale(Dd, best_t));
            D3 g, s;
            normals_double(prims, attributes, uint32_t(best), point, best_u, best_v, &g, &s);
            const bool front = dot(g, Dd) < 0.0;
            const D3 facing = front ? s : scale(s, -1.0);
            if (normal_out) {
                normal_out[3 * r] = facing.x;
                normal_out[3 * r + 1] = facing.y;
                normal_out[3 * r + 2] = facing.z;
            }
            if (front_out) front_out[r] = front ? 1 : 0;
        }
    });
}

extern "C" void ro_trace32_batch(const void* prims, const void* nodes, const float* rays, uint32_t n,
                                 float t_max, int any_hit, uint32_t* prim_out, float* t_out,
                                 uint32_t* inner_out, uint32_t* tested_out, int threads) {
    parallel_for(n, threads, [&](uint32_t r) {
        const F3 o = f3(rays + 6 * size_t(r));
        const F3 d = f3(rays + 6 * size_t(r) + 3);
        const F3 inv = {1.0f / safe1(d.x), 1.0f / safe1(d.y), 1.0f / safe1(d.z)};
        float hit_t = t_max;
        uint32_t hit_prim = RO_NONE;
        uint32_t inner = 0, tested = 0;

        if (slabs32(node_f(nodes, 0), o, inv, t_max) < INF32) {
            uint32_t stack[64];
            uint32_t sp = 0, current = 0;
            for (;;) {
                const float* nf = node_f(nodes, current);
                const uint32_t* nu = node_u(nodes, current);
                bool descend = false;
                if (nu[7] > 0) {
                    bool done = false;
                    for (uint32_t i = nu[3]; i < nu[3] + nu[7]; ++i) {
                        float h[3];
                        ++tested;
                        intersect32(prims, i, o, d, hit_t, h);
                        if (h[0] > 0.0f) {
                            hit_t = h[0];
                            hit_prim = i;
                            if (any_hit) {
                                done = true;
                                break;
                            }
                        }
                    }
                    if (done) break;
                } else {
                    ++inner;
                    const uint32_t left = nu[3], right = nu[3] + 1;
                    const float t_left = slabs32(node_f(nodes, left), o, inv, hit_t);
                    const float t_right = slabs32(node_f(nodes, right), o, inv, hit_t);
                    const uint32_t near_ = t_left <= t_right ? left : right;
                    const uint32_t far_ = t_left <= t_right ? right : left;
                    if (fminf_(t_left, t_right) < INF32) {
                        if (fmaxf_(t_left, t_right) < INF32 && sp < 64u) stack[sp++] = far_;
                        current = near_;
                        descend = true;
                    }
                }
                (void)nf;
                if (!descend) {
                    if (sp == 0) break;
                    current = stack[--sp];
                }
            }
        }
        prim_out[r] = hit_prim;
        t_out[r] = hit_t;
        if (inner_out) inner_out[r] = inner;
        if (tested_out) tested_out[r] = tested;
    });
}

// One ray through the shader's traversal in f32, with (t, u, v) of the hit
// and the byte counters; used by the path tracer restatement.
extern "C" void ro_trace32_one(const void* prims, const void* nodes, const float* o3, const float* d3_, float t_max,
                               int any_hit, uint32_t* prim_out, float* tuv_out, uint32_t* inner_out,
                               uint32_t* tested_out) {
    const F3 o = f3(o3), d = f3(d3_);
    const F3 inv = {1.0f / safe1(d.x), 1.0f / safe1(d.y), 1.0f / safe1(d.z)};
    float hit_t = t_max, hit_u = 0.0f, hit_v = 0.0f;
    uint32_t hit_prim = RO_NONE, inner = 0, tested = 0;
    if (slabs32(node_f(nodes, 0), o, inv, t_max) < INF32) {
        uint32_t stack[64];
        uint32_t sp = 0, current = 0;
        for (;;) {
            const uint32_t* nu = node_u(nodes, current);
            bool descend = false, done = false;
            if (nu[7] > 0) {
                for (uint32_t i = nu[3]; i < nu[3] + nu[7]; ++i) {
                    float h[3];
                    ++tested;
                    intersect32(prims, i, o, d, hit_t, h);
                    if (h[0] > 0.0f) {
                        hit_t = h[0];
                        hit_u = h[1];
                        hit_v = h[2];
                        hit_prim = i;
                        if (any_hit) {
                            done = true;
                            break;
                        }
                    }
                }
                if (done) break;
            } else {
                ++inner;
                const uint32_t left = nu[3], right = nu[3] + 1;
                const float t_left = slabs32(node_f(nodes, left), o, inv, hit_t);
                const float t_right = slabs32(node_f(nodes, right), o, inv, hit_t);
                const uint32_t near_ = t_left <= t_right ? left : right;
                const uint32_t far_ = t_left <= t_right ? right : left;
                if (fminf_(t_left, t_right) < INF32) {
                    if (fmaxf_(t_left, t_right) < INF32 && sp < 64u) stack[sp++] = far_;
                    current = near_;
                    descend = true;
                }
            }
            if (!descend) {
                if (sp == 0) break;
                current = stack[--sp];
            }
        }
    }
    *prim_out = hit_prim;
    tuv_out[0] = hit_t;
    tuv_out[1] = hit_u;
    tuv_out[2] = hit_v;
    if (inner_out) *inner_out = inner;
    if (tested_out) *tested_out = tested;
}

// The hit's surface frame as Scene.raycast builds it, in double
// (src/Scene.mjs:687-879): out[0..2] geometric normal, [3..5] shading
// normal (both unflipped), [6..7] uv (Scene.#uv, before the texture scale),
// [8..10] tangent, [11..13] up (Scene.#tangents).
extern "C" void ro_surface_double(const void* prims, const float* attributes, uint32_t p, const double* o,
                                  const double* d, double t, double bu, double bv, double* out) {
    const PrimView pv = prim(prims, p);
    const float* f = pv.f;
    const uint32_t kind = pv.u[0];
    const D3 O = {o[0], o[1], o[2]}, Dd = {d[0], d[1], d[2]};
    const D3 point = add(O, scale(Dd, t));
    D3 g, sh;
    normals_double(prims, attributes, p, point, bu, bv, &g, &sh);
    double u = 0, v = 0;
    D3 tangent{1, 0, 0}, up{0, 1, 0};
    auto sgn = [](double x) { return x > 0 ? 1.0 : (x < 0 ? -1.0 : 0.0); };
    if (kind == SPHERE) {
        const D3 n = normalized(sub(point, d3(f + 4)));
        const D3 x = d3(f + 8), north = d3(f + 12);
        const D3 z = cross(x, north);
        const double uu = std::atan2(-dot(n, z), dot(n, x)) / (2.0 * M_PI);
        u = uu - std::floor(uu);
        v = std::acos(std::min(std::max(dot(n, north), -1.0), 1.0)) / M_PI;
        tangent = cross(north, n);
        if (length(tangent) < 1e-6) tangent = x;
        up = cross(n, tangent);
    } else if (kind == QUAD) {
        u = bu;
        v = 1.0 - bv;
        tangent = d3(f + 8);
        up = d3(f + 12);
    } else if (kind == BOX) {
        double lp[3], half[3];
        for (int r = 0; r < 3; ++r) {
            lp[r] = double(f[4 + r * 4]) * point.x + double(f[5 + r * 4]) * point.y + double(f[6 + r * 4]) * point.z +
                    double(f[7 + r * 4]);
            half[r] = 1.0 / std::sqrt(double(f[4 + r * 4]) * f[4 + r * 4] + double(f[5 + r * 4]) * f[5 + r * 4] +
                                      double(f[6 + r * 4]) * f[6 + r * 4]);
        }
        const double ax = std::fabs(lp[0]), ay = std::fabs(lp[1]), az = std::fabs(lp[2]);
        const D3 r0 = d3(f + 4), r1 = d3(f + 8), r2 = d3(f + 12);
        if (ax >= ay && ax >= az) {
            u = (1.0 - sgn(lp[0]) * lp[2]) * half[2];
            v = (1.0 - lp[1]) * half[1];
            tangent = scale(r2, -sgn(lp[0]));
            up = r1;
        } else if (ay >= az) {
            u = (1.0 + lp[0]) * half[0];
            v = (1.0 + sgn(lp[1]) * lp[2]) * half[2];
            tangent = r0;
            up = scale(r2, -sgn(lp[1]));
        } else {
            u = (1.0 + sgn(lp[2]) * lp[0]) * half[0];
            v = (1.0 - lp[1]) * half[1];
            tangent = scale(r0, sgn(lp[2]));
            up = r1;
        }
    } else if (kind == TRIANGLE) {
        const uint32_t ai = pv.u[3];
        const bool textured = ai != RO_NONE && (int(attributes[(size_t(ai) + 3) * 4 + 3]) & 2);
        const D3 v0 = d3(f + 4);
        const D3 e1 = sub(d3(f + 8), v0), e2 = sub(d3(f + 12), v0);
        double du1[2] = {1, 0}, du2[2] = {0, 1};
        if (textured) {
            const float* A = attributes + size_t(ai) * 4;
            const double w = 1.0 - bu - bv;
            u = A[3] * w + A[7] * bu + A[11] * bv;
            v = A[12] * w + A[13] * bu + A[14] * bv;
            const double t1[2] = {double(A[7]) - A[3], double(A[13]) - A[12]};
            const double t2[2] = {double(A[11]) - A[3], double(A[14]) - A[12]};
            if (std::fabs(t1[0] * t2[1] - t2[0] * t1[1]) > 1e-12) {
                du1[0] = t1[0]; du1[1] = t1[1];
                du2[0] = t2[0]; du2[1] = t2[1];
            }
        } else {
            u = bu;
            v = bv;
        }
        const double det = du1[0] * du2[1] - du2[0] * du1[1];
        tangent = scale(sub(scale(e1, du2[1]), scale(e2, du1[1])), 1.0 / det);
        const D3 dpdv = scale(sub(scale(e2, du1[0]), scale(e1, du2[0])), 1.0 / det);
        up = scale(dpdv, -1.0);
    }
    const double vals[14] = {g.x, g.y, g.z, sh.x, sh.y, sh.z, u, v, tangent.x, tangent.y, tangent.z, up.x, up.y, up.z};
    for (int k = 0; k < 14; ++k) out[k] = vals[k];
}

// Whether a primitive other than `exclude` is crossed within rtol·t of
// distance t along the ray (coincident faces, shared edges): there the
// nearest hit is a tie that rounding decides.
extern "C" int ro_tie32(const void* prims, const void* nodes, const float* o3, const float* d3_, float t, float rtol,
                        uint32_t exclude) {
    const F3 o = f3(o3), d = f3(d3_);
    const F3 inv = {1.0f / safe1(d.x), 1.0f / safe1(d.y), 1.0f / safe1(d.z)};
    const float lo = t * (1.0f - rtol), hi = t * (1.0f + rtol);
    if (slabs32(node_f(nodes, 0), o, inv, hi) >= INF32) return 0;
    uint32_t stack[64];
    uint32_t sp = 0, current = 0;
    for (;;) {
        const uint32_t* nu = node_u(nodes, current);
        bool descend = false;
        if (nu[7] > 0) {
            for (uint32_t i = nu[3]; i < nu[3] + nu[7]; ++i) {
                if (i == exclude) continue;
                float h[3];
                intersect32(prims, i, o, d, hi, h);
                if (h[0] > 0.0f && h[0] >= lo) return 1;
            }
        } else {
            const uint32_t left = nu[3], right = nu[3] + 1;
            const float t_left = slabs32(node_f(nodes, left), o, inv, hi);
            const float t_right = slabs32(node_f(nodes, right), o, inv, hi);
            if (t_left < INF32 && t_right < INF32 && sp < 64u) stack[sp++] = right;
            if (t_left < INF32 || t_right < INF32) {
                current = t_left < INF32 ? left : right;
                descend = true;
            }
        }
        if (!descend) {
            if (sp == 0) return 0;
            current = stack[--sp];
        }
    }
}
