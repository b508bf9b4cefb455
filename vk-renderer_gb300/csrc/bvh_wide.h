// 4-wide BVH for the wavefront traversal, collapsed from the binary BVH.
#pragma once

#include <cstdint>
#include <vector>

#include "tracer_abi.h"

namespace vkt {

// One node = 128 bytes, read on the device as 8 float4: for each of up to
// four children, (box min, reference) (box max, 0).
//   ref > 0   interior: index of a wide node (the root, 0, is nobody's child)
//   ref < 0   leaf: -1 - ((first << 6) | (count - 1)), primitives
//             first .. first + count - 1 of the leaf-ordered arrays
//   ref == 0  empty slot (its box is never tested)
struct WideChild {
    float lo[3];
    int32_t ref;
    float hi[3];
    int32_t pad;
};
struct WideNode {
    WideChild c[4];
};
static_assert(sizeof(WideNode) == 128, "wide node is 8 x 16 bytes");

// Collapses a binary BVH (tracer_bvh_node, root 0, children side by side)
// into wide nodes.  Each wide node takes a binary node's two children and
// repeatedly replaces the interior child of largest surface area by its two
// children until it has four or only leaves remain.  The children's boxes
// are the binary nodes' boxes, unchanged.  Returns false if a leaf holds more
// than 64 primitives or starts beyond 2^25 (the leaf code's range).
// *depth_out: number of wide levels (a traversal pushes at most 3 entries
// per level).
bool collapse_wide4(const tracer_bvh_node* nodes, uint32_t num_nodes, std::vector<WideNode>& out,
                    uint32_t* depth_out);

// The binary BVH as the wavefront traverses it: the same records with
// left_or_first replaced by the record's child reference (interior: index of
// its children pair; leaf: -1 - ((first << 6) | (count - 1))) and count = 0,
// so the traversal reads a reference instead of decoding one.  Returns false
// if a leaf is outside the code's range (more than 64 primitives, or first
// beyond 2^25).
bool encode_refs(const tracer_bvh_node* nodes, uint32_t num_nodes, std::vector<tracer_bvh_node>& out);

}  // namespace vkt
