// BVH.build restated (src/BVH.mjs:57-234) — TEST INFRASTRUCTURE ONLY.
//
// Binned SAH over 32 bins per axis in double precision, leaves of up to
// max_leaf primitives, an explicit LIFO stack of nodes to split, children
// appended in pairs, nodes rounded to f32 only when packed. The arithmetic
// follows the JavaScript evaluation order term by term, and the file is
// compiled without floating-point contraction so x86 and Arm agree.
#include "oracle.h"

#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

namespace {

const double kInf = std::numeric_limits<double>::infinity();

struct Box {
    double min[3] = {kInf, kInf, kInf};
    double max[3] = {-kInf, -kInf, -kInf};
};

struct Node {
    double min[3], max[3];
    uint32_t first, count;
};

// BVH.#area (src/BVH.mjs:256-263): half the surface area, 0 for an empty box.
double area(const double* mn, const double* mx) {
    const double dx = mx[0] - mn[0];
    const double dy = mx[1] - mn[1];
    const double dz = mx[2] - mn[2];
    if (!(dx >= 0.0 && dy >= 0.0 && dz >= 0.0)) return 0.0;
    return dx * dy + dy * dz + dz * dx;
}

// JavaScript's Math.min / Math.max on non-NaN operands.
inline double jmin(double a, double b) { return b < a ? b : a; }
inline double jmax(double a, double b) { return b > a ? b : a; }

}  // namespace

extern "C" uint32_t ro_bvh_build(const double* mins, const double* maxs, uint32_t count,
                                 uint32_t max_leaf, void* nodes_out, uint32_t* order) {
    const int BINS = 32;  // src/BVH.mjs:92
    for (uint32_t i = 0; i < count; ++i) order[i] = i;

    std::vector<double> centroids(size_t(count) * 3);
    for (size_t i = 0; i < size_t(count) * 3; ++i) centroids[i] = (mins[i] + maxs[i]) * 0.5;

    std::vector<Node> nodes;
    nodes.reserve(count > 0 ? 2 * size_t(count) : 1);

    // addNode (src/BVH.mjs:72-87)
    auto add_node = [&](uint32_t first, uint32_t n) -> uint32_t {
        Node node;
        for (int a = 0; a < 3; ++a) {
            node.min[a] = kInf;
            node.max[a] = -kInf;
        }
        for (uint32_t i = first; i < first + n; ++i) {
            const uint32_t p = order[i];
            for (int a = 0; a < 3; ++a) {
                node.min[a] = jmin(node.min[a], mins[size_t(p) * 3 + a]);
                node.max[a] = jmax(node.max[a], maxs[size_t(p) * 3 + a]);
            }
        }
        node.first = first;
        node.count = n;
        nodes.push_back(node);
        return uint32_t(nodes.size() - 1);
    };

    add_node(0, count);
    std::vector<uint32_t> stack;
    if (count > max_leaf) stack.push_back(0);

    double bin_min[BINS * 3], bin_max[BINS * 3];
    uint32_t bin_count[BINS];
    double right_area[BINS];
    uint32_t right_count[BINS];

    while (!stack.empty()) {
        const uint32_t index = stack.back();
        stack.pop_back();
        const uint32_t first = nodes[index].first;
        const uint32_t n = nodes[index].count;

        // Centroid bounds (src/BVH.mjs:106-114).
        double cmin[3] = {kInf, kInf, kInf}, cmax[3] = {-kInf, -kInf, -kInf};
        for (uint32_t i = first; i < first + n; ++i) {
            const uint32_t p = order[i];
            for (int a = 0; a < 3; ++a) {
                cmin[a] = jmin(cmin[a], centroids[size_t(p) * 3 + a]);
                cmax[a] = jmax(cmax[a], centroids[size_t(p) * 3 + a]);
            }
        }

        double best_cost = kInf;
        int best_axis = -1;
        double best_split = 0.0;

        for (int axis = 0; axis < 3; ++axis) {
            const double extent = cmax[axis] - cmin[axis];
            if (!(extent > 0.0)) continue;

            for (int b = 0; b < BINS; ++b) {
                bin_count[b] = 0;
                for (int a = 0; a < 3; ++a) {
                    bin_min[b * 3 + a] = kInf;
                    bin_max[b * 3 + a] = -kInf;
                }
            }

            // Binning (src/BVH.mjs:131-140).
            const double scale = double(BINS) / extent;
            for (uint32_t i = first; i < first + n; ++i) {
                const uint32_t p = order[i];
                const double f = std::floor((centroids[size_t(p) * 3 + axis] - cmin[axis]) * scale);
                const int b = f < double(BINS - 1) ? int(f) : BINS - 1;
                bin_count[b]++;
                for (int a = 0; a < 3; ++a) {
                    bin_min[b * 3 + a] = jmin(bin_min[b * 3 + a], mins[size_t(p) * 3 + a]);
                    bin_max[b * 3 + a] = jmax(bin_max[b * 3 + a], maxs[size_t(p) * 3 + a]);
                }
            }

            // Suffix sweep from the right (src/BVH.mjs:143-150); BVH.#grow skips empty bins.
            Box box;
            uint32_t total = 0;
            for (int b = BINS - 1; b > 0; --b) {
                if (bin_count[b] != 0) {
                    for (int a = 0; a < 3; ++a) {
                        box.min[a] = jmin(box.min[a], bin_min[b * 3 + a]);
                        box.max[a] = jmax(box.max[a], bin_max[b * 3 + a]);
                    }
                }
                total += bin_count[b];
                right_area[b] = area(box.min, box.max);
                right_count[b] = total;
            }

            // Prefix sweep costing a split before each bin (src/BVH.mjs:152-166).
            Box left;
            uint32_t left_count = 0;
            for (int b = 1; b < BINS; ++b) {
                if (bin_count[b - 1] != 0) {
                    for (int a = 0; a < 3; ++a) {
                        left.min[a] = jmin(left.min[a], bin_min[(b - 1) * 3 + a]);
                        left.max[a] = jmax(left.max[a], bin_max[(b - 1) * 3 + a]);
                    }
                }
                left_count += bin_count[b - 1];
                if (left_count == 0 || right_count[b] == 0) continue;
                const double cost = double(left_count) * area(left.min, left.max) +
                                    double(right_count[b]) * right_area[b];
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = axis;
                    best_split = cmin[axis] + double(b) / scale;
                }
            }
        }

        const double parent_area = area(nodes[index].min, nodes[index].max);
        const double leaf_cost = double(n) * parent_area;

        int64_t mid;
        if (best_axis < 0) {
            // All centroids coincide (src/BVH.mjs:172-178).
            if (n <= max_leaf) continue;
            mid = int64_t(first) + (n >> 1);
        } else {
            if (n <= max_leaf && best_cost + parent_area >= leaf_cost) continue;
            // Two-pointer partition (src/BVH.mjs:184-195).
            int64_t i = first;
            int64_t j = int64_t(first) + n - 1;
            while (i <= j) {
                if (centroids[size_t(order[i]) * 3 + best_axis] < best_split) {
                    ++i;
                } else {
                    const uint32_t t = order[i];
                    order[i] = order[j];
                    order[j] = t;
                    --j;
                }
            }
            mid = i;
            if (mid == first || mid == int64_t(first) + n) mid = int64_t(first) + (n >> 1);
        }

        const uint32_t left_index = add_node(first, uint32_t(mid - first));
        add_node(uint32_t(mid), uint32_t(int64_t(first) + n - mid));
        nodes[index].first = left_index;
        nodes[index].count = 0;

        for (uint32_t child = left_index; child <= left_index + 1; ++child)
            if (nodes[child].count > 1) stack.push_back(child);
    }

    // Pack as 32-byte records (src/BVH.mjs:209-231).
    uint8_t* out = static_cast<uint8_t*>(nodes_out);
    if (count == 0) {
        std::memset(out, 0, 32);
        return 1;
    }
    for (size_t i = 0; i < nodes.size(); ++i) {
        float f[8];
        uint32_t u[8];
        for (int a = 0; a < 3; ++a) {
            f[a] = float(nodes[i].min[a]);
            f[4 + a] = float(nodes[i].max[a]);
        }
        std::memcpy(u, f, sizeof f);
        u[3] = nodes[i].first;
        u[7] = nodes[i].count;
        std::memcpy(out + i * 32, u, 32);
    }
    return uint32_t(nodes.size());
}
