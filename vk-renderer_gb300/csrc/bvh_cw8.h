// Compressed 8-wide BVH for the wavefront's extend kernel, collapsed from the
// binary BVH (the traversal scheme of Ylitie, Karras and Laine, "Efficient
// Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs", HPG 2017:
// quantised child boxes, child slots ordered by ray octant, node groups with
// a hit mask on the traversal stack; the layout below is this project's).
#pragma once

#include <cstdint>
#include <vector>

#include "tracer_abi.h"

namespace vkt {

// One node = 96 bytes (three 256-bit loads), as 24 little-endian words:
//   w0..w2   p: origin of the quantisation grid (float x, y, z)
//   w3       ex | ey << 8 | ez << 16 | imask << 24: grid steps 2^(e - 127)
//            per axis (e is a float's biased exponent), imask bit k = slot k
//            holds an interior child
//   w4       child_base: node index of the first interior child; the
//            interior children are stored consecutively in slot order
//   w5       prim_base: index (in the 8-wide primitive order) of the first
//            primitive of the node's leaf children, stored consecutively in
//            slot order (at most 24 per node)
//   w6, w7   octant mask byte of slot k (byte k % 4 of w6 + k / 4): 7 for an
//            interior child, else 0
//   w8..w19  quantised box bytes, slot k in byte k % 4 of the word pair:
//            lo x (w8, w9), lo y (w10, w11), lo z (w12, w13),
//            hi x (w14, w15), hi y (w16, w17), hi z (w18, w19);
//            box = [p + lo * 2^(e - 127), p + hi * 2^(e - 127)] per axis,
//            which contains the binary child's (padded) box exactly
//   w20, w21 hit-mask bits of slot k: a leaf of c primitives (1..6) ->
//            (1 << c) - 1; an interior child -> 1; an empty slot -> 0
//   w22, w23 bit position of slot k: a leaf -> o, its first primitive being
//            prim_base + o (o + c <= 24); an interior child -> 24 + slot
// A child hit by a ray of octant s (bit a set for a negative direction
// component on axis a) adds its bits at position (position ^ (mask & s ^ 7)):
// the primitives to test in bits 0..23, the interior children in bits 24..31,
// slot k at bit 24 + (k ^ s ^ 7).  Slot order: slot s holds the child met
// first by rays of octant s; the traversal visits the hit interior children
// highest bit first, i.e. in descending order of slot ^ s ^ 7.
struct alignas(32) Cw8Node {
    uint32_t w[24];
};
static_assert(sizeof(Cw8Node) == 96, "8-wide node is 96 bytes");

constexpr uint32_t kCw8MaxLeafPrims = 6;
constexpr uint32_t kCw8MaxNodePrims = 24;

// Collapses a binary BVH (tracer_bvh_node, root 0, children side by side,
// leaves = ranges of the leaf-ordered primitive array) into 8-wide nodes.
// Each node takes a binary interior node's two children and repeatedly
// replaces the interior child of largest surface area by its two children
// while it has fewer than eight and its leaf children hold at most 24
// primitives.  order_out[k] = leaf-ordered slot of the 8-wide order's
// primitive k.  *depth_out = levels of 8-wide nodes (the traversal stack
// holds at most one entry per level).  Returns false (no 8-wide BVH) when a
// leaf holds more than 6 primitives or a coordinate's magnitude exceeds 1e6
// (the quantised slab test's range).
bool build_cw8(const tracer_bvh_node* nodes, uint32_t num_nodes, std::vector<Cw8Node>& out,
               std::vector<uint32_t>& order_out, uint32_t* depth_out);

}  // namespace vkt
