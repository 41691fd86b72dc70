// bvh.h — host-side binned-SAH BVH builder producing the 32-byte node layout
// described in core.h.  The reference has no acceleration structure (its
// intersect() is a linear scan, experiments/rt.cpp:209-218); the tree changes
// the cost of a closest-hit query, not its result (smallest t, lower global id
// on equal t).
#pragma once

#include <cstdint>
#include <vector>

namespace are_core {

struct PrimBox {
	double lo[3], hi[3];
};

struct BvhResult {
	std::vector<float> nodes;       // 8 floats per node (see core.h), 2 * n_pairs + 2 nodes
	std::vector<int32_t> order;     // leaf order -> input primitive index
	int32_t n_nodes = 0;
	int32_t depth = 0;
	int32_t max_leaf = 0;
	float box_pad = 0.0f;
};

// Builds the tree over `boxes`.  leaf_size bounds the primitives per leaf.
// Node boxes are rounded outward to float and padded by box_pad = 2^-19 times
// the largest coordinate magnitude of the scene, so FP32 slab tests never cull
// a box whose primitive a separate FP32 primitive test would hit.
BvhResult build_bvh(const std::vector<PrimBox> &boxes, int leaf_size);

// The same tree with four children per node: every node of the result is four
// 32-byte child records in the binary tree's record format (box, a; box, b:
// b == 0 marks an interior child whose four records start at 4 a, b > 0 a leaf
// of b primitives from a), 128 bytes; unused slots are empty leaves (b = -1).  A
// node's children are the binary node's children, each interior one replaced
// by its own two children, largest surface area first, until four (the usual
// collapse of a binary SAH tree).  Nodes are numbered breadth-first for the
// first `bfs_nodes` (the shared-memory top levels), depth-first after.  The
// root's own box stays in the binary tree's record 0.  Empty when the binary
// root is a leaf (the tree has fewer than two levels).
std::vector<float> collapse_bvh4(const BvhResult &bvh, int bfs_nodes);

}  // namespace are_core
