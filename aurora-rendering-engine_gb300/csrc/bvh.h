// bvh.h — host-side binned-SAH BVH builder producing the 32-byte node layout
// described in core.h.  The reference has no acceleration structure (its
// intersect() is a linear scan, experiments/rt.cpp:209-218); the tree changes
// the cost of a closest-hit query, not its result (smallest t, lower global id
// on equal t).
#pragma once

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <thread>
#include <vector>

namespace are_core {

// host threads for the scene build (at most 32)
inline unsigned hw_threads() { return std::max(1u, std::min(32u, std::thread::hardware_concurrency())); }

// fn(k) for every k in [0, n), whole jobs taken in turn by up to `threads` threads
template <class F>
void run_jobs(size_t n, unsigned threads, F fn) {
	threads = (unsigned)std::min<size_t>(threads, n);
	if (threads <= 1) {
		for (size_t k = 0; k < n; ++k) fn(k);
		return;
	}
	std::atomic<size_t> next{ 0 };
	auto worker = [&]() {
		for (size_t k; (k = next.fetch_add(1)) < n;) fn(k);
	};
	std::vector<std::thread> pool;
	for (unsigned t = 1; t < threads; ++t) pool.emplace_back(worker);
	worker();
	for (std::thread &t : pool) t.join();
}

// fn(begin, end) over [0, n) in contiguous parts, on several threads once n reaches 2^16
template <class F>
void parallel_ranges(size_t n, F fn) {
	const unsigned threads = n < ((size_t)1 << 16) ? 1u : hw_threads();
	const size_t parts = threads > 1 ? 4 * (size_t)threads : 1;
	run_jobs(parts, threads, [&](size_t p) { fn(n * p / parts, n * (p + 1) / parts); });
}

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
