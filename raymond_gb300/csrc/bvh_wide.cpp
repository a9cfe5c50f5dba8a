// The traversal's 4-wide tree, derived from the reference's binary BVH
// (BVH.build's 32-byte nodes: min|first, max|count; an inner node's two
// children adjacent at first, first + 1 — src/BVH.mjs:196-204) when a scene
// is uploaded. The packed buffers stay the contract; this tree only changes
// how rays walk them: a wide node holds its four children's boxes (128 B, two
// cache lines), so a ray tests four boxes per node visit instead of two and
// takes about half the steps.
//
// Collapse: a wide node starts from a binary inner node's two children and
// repeatedly replaces the child with the largest surface area that is itself
// inner by that node's two children, up to four. Leaves keep the reference's
// primitive ranges, so every hit is a primitive of the same leaf order.
#include "bvh_wide.h"

#include <cmath>
#include <cstring>
#include <deque>
#include <utility>

namespace rmd {

namespace {

struct BinNode {
    float mn[3], mx[3];
    uint32_t first, count;
};

BinNode read_node(const uint32_t* nu, uint32_t i) {
    BinNode b;
    std::memcpy(b.mn, nu + size_t(i) * 8, 12);
    std::memcpy(&b.first, nu + size_t(i) * 8 + 3, 4);
    std::memcpy(b.mx, nu + size_t(i) * 8 + 4, 12);
    std::memcpy(&b.count, nu + size_t(i) * 8 + 7, 4);
    return b;
}

double area(const BinNode& b) {
    const double dx = double(b.mx[0]) - b.mn[0], dy = double(b.mx[1]) - b.mn[1], dz = double(b.mx[2]) - b.mn[2];
    return dx * dy + dy * dz + dz * dx;
}

}  // namespace

bool build_wide_bvh(const uint32_t* nu, uint32_t node_count, std::vector<float>& out) {
    out.clear();
    if (node_count == 0) return false;
    for (uint32_t i = 0; i < node_count; ++i) {
        const BinNode b = read_node(nu, i);
        if (b.count > 0 && (b.count > WIDE_LEAF_MAX_COUNT || b.first >= WIDE_LEAF_MAX_FIRST)) return false;
    }
    // (wide node to fill, binary node whose subtree it covers)
    std::deque<std::pair<uint32_t, uint32_t>> work;
    out.assign(WIDE_NODE_FLOATS, 0.0f);
    work.emplace_back(0u, 0u);
    while (!work.empty()) {
        const auto [wi, bi] = work.front();
        work.pop_front();
        const BinNode root = read_node(nu, bi);
        uint32_t kids[4];
        int n = 0;
        if (root.count > 0) {
            kids[n++] = bi;  // a leaf at the root
        } else {
            kids[n++] = root.first;
            kids[n++] = root.first + 1;
            while (n < 4) {
                int best = -1;
                double best_area = -1.0;
                for (int k = 0; k < n; ++k) {
                    const BinNode c = read_node(nu, kids[k]);
                    if (c.count == 0 && area(c) > best_area) {
                        best_area = area(c);
                        best = k;
                    }
                }
                if (best < 0) break;
                const uint32_t f = read_node(nu, kids[best]).first;
                kids[best] = f;
                kids[n++] = f + 1;
            }
        }
        float node[WIDE_NODE_FLOATS];
        uint32_t refs[4];
        for (int k = 0; k < 4; ++k) {
            if (k >= n) {
                for (int a = 0; a < 3; ++a) {
                    node[(2 * a) * 4 + k] = INFINITY;
                    node[(2 * a + 1) * 4 + k] = -INFINITY;
                }
                refs[k] = WIDE_EMPTY;
                continue;
            }
            const BinNode c = read_node(nu, kids[k]);
            for (int a = 0; a < 3; ++a) {
                node[(2 * a) * 4 + k] = c.mn[a];
                node[(2 * a + 1) * 4 + k] = c.mx[a];
            }
            if (c.count > 0) {
                refs[k] = WIDE_LEAF_BIT | ((c.count - 1) << 24) | c.first;
            } else {
                const uint32_t child = uint32_t(out.size() / WIDE_NODE_FLOATS);
                out.resize(out.size() + WIDE_NODE_FLOATS, 0.0f);
                work.emplace_back(child, kids[k]);
                refs[k] = child;
            }
        }
        std::memcpy(node + 24, refs, 16);
        std::memset(node + 28, 0, 16);
        std::memcpy(out.data() + size_t(wi) * WIDE_NODE_FLOATS, node, sizeof node);
        if (out.size() / WIDE_NODE_FLOATS >= WIDE_LEAF_BIT) return false;
    }
    return true;
}

}  // namespace rmd
