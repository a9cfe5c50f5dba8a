// The 4-wide traversal tree derived from the reference's binary BVH.
//
// Node: 32 floats (128 B) = lo.x[4], hi.x[4], lo.y[4], hi.y[4], lo.z[4],
// hi.z[4], then four child references (u32) and four spare words.
// Reference: a wide node index; a leaf, WIDE_LEAF_BIT | (count − 1) << 24 |
// first primitive; or WIDE_EMPTY for an unused slot (its box is empty).
#pragma once
#include <cstdint>
#include <vector>

namespace rmd {

constexpr uint32_t WIDE_NODE_FLOATS = 32;
constexpr uint32_t WIDE_LEAF_BIT = 0x80000000u;
constexpr uint32_t WIDE_EMPTY = 0xFFFFFFFFu;
constexpr uint32_t WIDE_LEAF_MAX_COUNT = 128;
constexpr uint32_t WIDE_LEAF_MAX_FIRST = 1u << 24;

// Builds the wide tree from node_count binary nodes (8 u32 each). False when
// a leaf does not fit a reference (more than 128 primitives, or starting at
// primitive 2^24 or beyond): the binary tree is traversed then.
bool build_wide_bvh(const uint32_t* nodes, uint32_t node_count, std::vector<float>& out);

}  // namespace rmd
