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

}  // namespace are_core
