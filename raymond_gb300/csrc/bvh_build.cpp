// Native binned-SAH BVH builder producing BVH.build's exact nodes and
// primitive order (src/BVH.mjs:57-234), so packed scenes built here and by
// the JavaScript library are interchangeable byte for byte.
//
// Same decisions as the reference, organized for speed: each primitive's
// centroid and box travel as one record that the partition moves together
// with its index, so every pass over a node reads memory in order; one pass
// bins all three axes at once; the passes over the few largest nodes (the
// top of the tree) are split over the threads, whose bins and bounds merge
// exactly (counts, minima, maxima); and independent subtrees are built on
// worker threads into private node lists that are spliced into the
// reference's node numbering afterwards (its numbering is a right-first
// depth-first order, so a subtree's nodes form one contiguous run once its
// size is known). The partition itself stays the reference's sequential
// two-pointer swap, which decides the primitive order.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/raymond.h"

namespace {

constexpr int BINS = 32;
const double kInf = std::numeric_limits<double>::infinity();

struct BuildNode {
    double min[3], max[3];
    uint32_t first, count;  // count 0: inner, first = left child (local index while building a subtree)
};

struct Rec {
    double c[3], lo[3], hi[3];  // centroid and box of the primitive order[i]
};

struct Input {
    std::vector<Rec> rec;  // in the current order
    uint32_t max_leaf;
    uint32_t* order;
    int threads;
};

// Nodes of at least this many primitives split their passes over the threads.
constexpr uint32_t kParallelMin = 1u << 16;

// f(lo, hi, t) over [first, first + n) in `parts` contiguous pieces, one per
// thread (piece t on thread t; the caller runs piece 0).
template <typename F>
void parallel_pieces(uint32_t first, uint32_t n, int parts, F&& f) {
    std::vector<std::thread> pool;
    const uint32_t step = (n + uint32_t(parts) - 1) / uint32_t(parts);
    for (int t = 1; t < parts; ++t) {
        const uint32_t lo = first + std::min(n, step * uint32_t(t)), hi = first + std::min(n, step * uint32_t(t + 1));
        pool.emplace_back([&f, lo, hi, t] { f(lo, hi, t); });
    }
    f(first, first + std::min(n, step), 0);
    for (auto& th : pool) th.join();
}

inline int parts_for(const Input& in, uint32_t n, bool par) {
    return par && in.threads > 1 && n >= kParallelMin ? in.threads : 1;
}

inline double area3(const double* mn, const double* mx) {
    const double dx = mx[0] - mn[0];
    const double dy = mx[1] - mn[1];
    const double dz = mx[2] - mn[2];
    if (!(dx >= 0.0 && dy >= 0.0 && dz >= 0.0)) return 0.0;
    return dx * dy + dy * dz + dz * dx;
}

void bounds_of(const Input& in, uint32_t first, uint32_t n, BuildNode& node, bool par = false) {
    const int parts = parts_for(in, n, par);
    double one_mn[3] = {kInf, kInf, kInf}, one_mx[3] = {-kInf, -kInf, -kInf};
    std::vector<double> many_mn(parts > 1 ? size_t(parts) * 3 : 0u, kInf), many_mx(parts > 1 ? size_t(parts) * 3 : 0u, -kInf);
    double* mn = parts > 1 ? many_mn.data() : one_mn;
    double* mx = parts > 1 ? many_mx.data() : one_mx;
    parallel_pieces(first, n, parts, [&](uint32_t lo_i, uint32_t hi_i, int t) {
        double* a_mn = &mn[size_t(t) * 3];
        double* a_mx = &mx[size_t(t) * 3];
        for (uint32_t i = lo_i; i < hi_i; ++i) {
            const Rec& r = in.rec[i];
            for (int a = 0; a < 3; ++a) {
                if (r.lo[a] < a_mn[a]) a_mn[a] = r.lo[a];
                if (r.hi[a] > a_mx[a]) a_mx[a] = r.hi[a];
            }
        }
    });
    for (int a = 0; a < 3; ++a) {
        node.min[a] = kInf;
        node.max[a] = -kInf;
        for (int t = 0; t < parts; ++t) {
            if (mn[size_t(t) * 3 + a] < node.min[a]) node.min[a] = mn[size_t(t) * 3 + a];
            if (mx[size_t(t) * 3 + a] > node.max[a]) node.max[a] = mx[size_t(t) * 3 + a];
        }
    }
    node.first = first;
    node.count = n;
}

// The split decision for one node: returns false for "keep as a leaf", else
// the partition point in the order array.
bool split_node(Input& in, const BuildNode& node, uint32_t& mid_out, bool par = false) {
    const uint32_t first = node.first, n = node.count;
    const int parts = parts_for(in, n, par);
    struct Bins {
        double cmin[3], cmax[3];
        double bmin[3][BINS][3], bmax[3][BINS][3];
        uint32_t bcount[3][BINS];
    };
    Bins one;  // the common case needs no allocation
    std::vector<Bins> many(parts > 1 ? static_cast<size_t>(parts) : 0u);
    Bins* pb = parts > 1 ? many.data() : &one;
    // centroid bounds, per piece then merged
    parallel_pieces(first, n, parts, [&](uint32_t lo_i, uint32_t hi_i, int t) {
        Bins& B = pb[size_t(t)];
        for (int a = 0; a < 3; ++a) {
            B.cmin[a] = kInf;
            B.cmax[a] = -kInf;
        }
        for (uint32_t i = lo_i; i < hi_i; ++i)
            for (int a = 0; a < 3; ++a) {
                const double c = in.rec[i].c[a];
                if (c < B.cmin[a]) B.cmin[a] = c;
                if (c > B.cmax[a]) B.cmax[a] = c;
            }
    });
    double cmin[3] = {kInf, kInf, kInf}, cmax[3] = {-kInf, -kInf, -kInf};
    for (int t = 0; t < parts; ++t)
        for (int a = 0; a < 3; ++a) {
            if (pb[size_t(t)].cmin[a] < cmin[a]) cmin[a] = pb[size_t(t)].cmin[a];
            if (pb[size_t(t)].cmax[a] > cmax[a]) cmax[a] = pb[size_t(t)].cmax[a];
        }
    double scale[3];
    bool live[3];
    for (int a = 0; a < 3; ++a) {
        const double extent = cmax[a] - cmin[a];
        live[a] = extent > 0.0;
        scale[a] = live[a] ? double(BINS) / extent : 0.0;
    }

    // One pass bins every live axis, per piece.
    parallel_pieces(first, n, parts, [&](uint32_t lo_i, uint32_t hi_i, int t) {
        // only the counts are reset: a bin's bounds start at its first primitive
        Bins& B = pb[size_t(t)];
        std::memset(B.bcount, 0, sizeof B.bcount);
        for (uint32_t i = lo_i; i < hi_i; ++i) {
            const Rec& r = in.rec[i];
            for (int a = 0; a < 3; ++a) {
                if (!live[a]) continue;
                // x ≥ 0 (c ≥ cmin), so truncation is the reference's Math.floor
                const double x = (r.c[a] - cmin[a]) * scale[a];
                const int b = x < double(BINS - 1) ? int(x) : BINS - 1;
                if (B.bcount[a][b]++ == 0) {
                    for (int k = 0; k < 3; ++k) {
                        B.bmin[a][b][k] = r.lo[k];
                        B.bmax[a][b][k] = r.hi[k];
                    }
                    continue;
                }
                for (int k = 0; k < 3; ++k) {
                    if (r.lo[k] < B.bmin[a][b][k]) B.bmin[a][b][k] = r.lo[k];
                    if (r.hi[k] > B.bmax[a][b][k]) B.bmax[a][b][k] = r.hi[k];
                }
            }
        }
    });
    Bins& M = pb[0];  // merged into piece 0's bins
    for (int t = 1; t < parts; ++t) {
        const Bins& B = pb[size_t(t)];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < BINS; ++b) {
                if (B.bcount[a][b] == 0) continue;  // its bounds were never written
                if (M.bcount[a][b] == 0) {
                    for (int k = 0; k < 3; ++k) {
                        M.bmin[a][b][k] = B.bmin[a][b][k];
                        M.bmax[a][b][k] = B.bmax[a][b][k];
                    }
                } else {
                    for (int k = 0; k < 3; ++k) {
                        if (B.bmin[a][b][k] < M.bmin[a][b][k]) M.bmin[a][b][k] = B.bmin[a][b][k];
                        if (B.bmax[a][b][k] > M.bmax[a][b][k]) M.bmax[a][b][k] = B.bmax[a][b][k];
                    }
                }
                M.bcount[a][b] += B.bcount[a][b];
            }
    }
    auto& bmin = M.bmin;
    auto& bmax = M.bmax;
    auto& bcount = M.bcount;

    // The reference sweeps every split position b = 1 … 31 (left: bins < b,
    // right: bins ≥ b) and keeps the first of the lowest cost. Positions
    // between two non-empty bins see the same two sets, so the same cost;
    // the first of them, just after a non-empty bin, is the only one that
    // can win. Only those are evaluated, with the same arithmetic.
    double best_cost = kInf, best_split = 0.0;
    int best_axis = -1;
    for (int a = 0; a < 3; ++a) {
        if (!live[a]) continue;
        int nz[BINS], m = 0;
        for (int b = 0; b < BINS; ++b)
            if (bcount[a][b]) nz[m++] = b;
        if (m < 2) continue;
        double right_area[BINS];  // of the bins nz[k] … nz[m-1]
        uint32_t right_count[BINS];
        double rmn[3] = {kInf, kInf, kInf}, rmx[3] = {-kInf, -kInf, -kInf};
        uint32_t total = 0;
        for (int k = m - 1; k >= 1; --k) {
            const int b = nz[k];
            for (int q = 0; q < 3; ++q) {
                rmn[q] = std::min(rmn[q], bmin[a][b][q]);
                rmx[q] = std::max(rmx[q], bmax[a][b][q]);
            }
            total += bcount[a][b];
            right_area[k] = area3(rmn, rmx);
            right_count[k] = total;
        }
        double lmn[3] = {kInf, kInf, kInf}, lmx[3] = {-kInf, -kInf, -kInf};
        uint32_t left_count = 0;
        for (int k = 0; k + 1 < m; ++k) {
            const int b = nz[k];
            for (int q = 0; q < 3; ++q) {
                lmn[q] = std::min(lmn[q], bmin[a][b][q]);
                lmx[q] = std::max(lmx[q], bmax[a][b][q]);
            }
            left_count += bcount[a][b];
            const double cost = double(left_count) * area3(lmn, lmx) + double(right_count[k + 1]) * right_area[k + 1];
            if (cost < best_cost) {
                best_cost = cost;
                best_axis = a;
                best_split = cmin[a] + double(b + 1) / scale[a];
            }
        }
    }

    const double parent_area = area3(node.min, node.max);
    const double leaf_cost = double(n) * parent_area;
    if (best_axis < 0) {
        if (n <= in.max_leaf) return false;
        mid_out = first + (n >> 1);
        return true;
    }
    if (n <= in.max_leaf && best_cost + parent_area >= leaf_cost) return false;
    int64_t i = first, j = int64_t(first) + n - 1;
    while (i <= j) {
        if (in.rec[i].c[best_axis] < best_split) {
            ++i;
        } else {
            std::swap(in.order[i], in.order[j]);
            std::swap(in.rec[i], in.rec[j]);
            --j;
        }
    }
    int64_t mid = i;
    if (mid == first || mid == int64_t(first) + n) mid = int64_t(first) + (n >> 1);
    mid_out = uint32_t(mid);
    return true;
}

// Builds the subtree under `root` (already bounded) into a private list
// whose entry 0 is the root; the list's numbering is the reference's
// right-first depth-first order, relative to the root.
void build_subtree(Input& in, const BuildNode& root, std::vector<BuildNode>& out) {
    out.clear();
    out.push_back(root);
    std::vector<uint32_t> stack;
    if (root.count > in.max_leaf || root.count > 1) stack.push_back(0);
    while (!stack.empty()) {
        const uint32_t idx = stack.back();
        stack.pop_back();
        uint32_t mid;
        const BuildNode node = out[idx];
        if (!split_node(in, node, mid)) continue;
        BuildNode l, r;
        bounds_of(in, node.first, mid - node.first, l);
        bounds_of(in, mid, node.first + node.count - mid, r);
        const uint32_t li = uint32_t(out.size());
        out.push_back(l);
        out.push_back(r);
        out[idx].first = li;
        out[idx].count = 0;
        if (l.count > 1) stack.push_back(li);
        if (r.count > 1) stack.push_back(li + 1);
    }
}

void write_node(uint8_t* dst, const BuildNode& n, uint32_t first, uint32_t count) {
    float f[8];
    for (int a = 0; a < 3; ++a) {
        f[a] = float(n.min[a]);
        f[4 + a] = float(n.max[a]);
    }
    uint32_t u[8];
    std::memcpy(u, f, sizeof f);
    u[3] = first;
    u[7] = count;
    std::memcpy(dst, u, 32);
}

}  // namespace

extern "C" uint32_t raymond_bvh_build(const double* mins, const double* maxs, uint32_t count, uint32_t max_leaf,
                                      void* nodes_out, uint32_t* order_out, int threads) {
    if (!nodes_out || !order_out || max_leaf == 0 || (count > 0 && (!mins || !maxs))) return 0;
    uint8_t* out = static_cast<uint8_t*>(nodes_out);
    for (uint32_t i = 0; i < count; ++i) order_out[i] = i;
    if (count == 0) {
        std::memset(out, 0, 32);
        return 1;
    }
    if (threads < 1) threads = 1;
    Input in;
    in.max_leaf = max_leaf;
    in.order = order_out;
    in.threads = threads;
    in.rec.resize(count);
    for (uint32_t i = 0; i < count; ++i) {
        Rec& r = in.rec[i];
        for (int a = 0; a < 3; ++a) {
            r.lo[a] = mins[size_t(i) * 3 + a];
            r.hi[a] = maxs[size_t(i) * 3 + a];
            r.c[a] = (r.lo[a] + r.hi[a]) * 0.5;
        }
    }

    BuildNode root;
    bounds_of(in, 0, count, root, true);
    if (count <= max_leaf) {
        write_node(out, root, 0, root.count);
        return 1;
    }

    // Top levels one node at a time (each node's passes over the threads),
    // until there are enough frontier subtrees to spread over the threads.
    const uint32_t want = threads > 1 ? uint32_t(threads) * 8u : 1u;
    // The top tree: nodes whose split happened here; frontier entries are
    // nodes left to split (with count > 1), built later as subtrees.
    struct Top {
        BuildNode node;
        int32_t left;      // top index of the left child, -1 if not split here
        int32_t frontier;  // index into frontier list, -1 if none
    };
    std::vector<Top> top;
    top.push_back({root, -1, -1});
    std::vector<uint32_t> open = {0};  // top nodes still to split (count > 1)
    const uint32_t big_enough = count / (want * 4) + 64;
    while (!open.empty() && top.size() < 4 * want) {
        // Split the largest open node next (it is independent of the others).
        auto it = std::max_element(open.begin(), open.end(),
                                   [&](uint32_t a, uint32_t b) { return top[a].node.count < top[b].node.count; });
        const uint32_t idx = *it;
        if (top[idx].node.count < big_enough) break;
        open.erase(it);
        uint32_t mid;
        if (!split_node(in, top[idx].node, mid, true)) continue;
        BuildNode l, r;
        bounds_of(in, top[idx].node.first, mid - top[idx].node.first, l, true);
        bounds_of(in, mid, top[idx].node.first + top[idx].node.count - mid, r, true);
        top[idx].left = int32_t(top.size());
        top.push_back({l, -1, -1});
        top.push_back({r, -1, -1});
        if (l.count > 1) open.push_back(uint32_t(top[idx].left));
        if (r.count > 1) open.push_back(uint32_t(top[idx].left + 1));
    }
    // Every top node not split here becomes a subtree root.
    std::vector<uint32_t> frontier;
    for (uint32_t i = 0; i < top.size(); ++i)
        if (top[i].left < 0) {
            top[i].frontier = int32_t(frontier.size());
            frontier.push_back(i);
        }
    std::vector<std::vector<BuildNode>> subtrees(frontier.size());
    {
        std::atomic<uint32_t> next{0};
        auto worker = [&] {
            for (;;) {
                const uint32_t k = next.fetch_add(1);
                if (k >= frontier.size()) return;
                build_subtree(in, top[frontier[k]].node, subtrees[k]);
            }
        };
        std::vector<std::thread> pool;
        const int nt = std::min<int>(threads, int(frontier.size()));
        for (int t = 1; t < nt; ++t) pool.emplace_back(worker);
        worker();
        for (auto& t : pool) t.join();
    }

    // Total nodes under each top node (itself included).
    std::vector<uint64_t> size(top.size(), 0);
    for (int64_t i = int64_t(top.size()) - 1; i >= 0; --i) {
        if (top[i].left < 0) size[i] = subtrees[top[i].frontier].size();
        else size[i] = 1 + size[top[i].left] + size[top[i].left + 1];
    }

    // Place nodes in the reference's numbering: a split node at g has its
    // children at c, c+1 (c = the next free index when it was split); the
    // right child's descendants come first, then the left's.
    uint32_t written = 0;
    struct Item {
        uint32_t top_index;
        uint32_t global;
    };
    // Emits the subtree of a node already placed at `global`; next_free is
    // where its descendants start.
    std::vector<std::pair<Item, uint32_t>> work;  // (node, next_free)
    work.push_back({{0, 0}, 1});
    while (!work.empty()) {
        const auto [item, next_free] = work.back();
        work.pop_back();
        const Top& t = top[item.top_index];
        if (t.left < 0) {
            // A subtree built privately: local index k maps to global via
            // local 0 -> item.global and locals >= 1 -> next_free + k - 1.
            const std::vector<BuildNode>& st = subtrees[t.frontier];
            for (size_t k = 0; k < st.size(); ++k) {
                const uint32_t g = k == 0 ? item.global : next_free + uint32_t(k) - 1;
                const uint32_t first = st[k].count == 0 ? next_free + st[k].first - 1 : st[k].first;
                write_node(out + size_t(g) * 32, st[k], first, st[k].count);
                ++written;
            }
            continue;
        }
        const uint32_t c = next_free;
        write_node(out + size_t(item.global) * 32, t.node, c, 0);
        ++written;
        const uint32_t li = uint32_t(t.left), ri = li + 1;
        // Right child's descendants first (it is popped first), then the left's.
        const uint32_t right_desc_start = c + 2;
        const uint32_t left_desc_start = right_desc_start + uint32_t(size[ri] - 1);
        work.push_back({{li, c}, left_desc_start});
        work.push_back({{ri, c + 1}, right_desc_start});
    }
    return written;
}
