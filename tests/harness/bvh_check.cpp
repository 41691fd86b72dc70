// Host-side check of the BVH builder (csrc/bvh.cpp), compiled by
// tests/test_bvh_host.py: random primitive boxes -> two builds must give the
// same node array (the parallel subtree build is deterministic), every
// primitive sits in exactly one leaf, every node's box contains its
// children's, and the pair layout holds (children at even indices).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "bvh.h"

using are_core::BvhResult;
using are_core::PrimBox;

int main(int argc, char **argv) {
	const int n = argc > 1 ? std::atoi(argv[1]) : 200000;
	const int leaf = argc > 2 ? std::atoi(argv[2]) : 4;
	std::mt19937_64 rng(12345);
	std::uniform_real_distribution<double> U(-100.0, 100.0), S(0.01, 2.0);
	std::vector<PrimBox> boxes((size_t)n);
	for (PrimBox &b : boxes)
		for (int k = 0; k < 3; ++k) {
			double c = U(rng), h = S(rng);
			b.lo[k] = c - h, b.hi[k] = c + h;
		}
	BvhResult a = are_core::build_bvh(boxes, leaf), b = are_core::build_bvh(boxes, leaf);
	if (a.nodes != b.nodes || a.order != b.order) { std::puts("FAIL nondeterministic"); return 1; }
	std::vector<int> seen((size_t)n, 0);
	auto f = [&](int node, int k) { return a.nodes[8 * (size_t)node + k]; };
	auto ii = [&](int node, int k) { int32_t v; std::memcpy(&v, &a.nodes[8 * (size_t)node + k], 4); return v; };
	std::vector<int> stack{ 0 };
	while (!stack.empty()) {
		int node = stack.back();
		stack.pop_back();
		int av = ii(node, 3), bv = ii(node, 7);
		if (bv > 0) {
			if (bv > leaf) { std::puts("FAIL leaf too large"); return 1; }
			for (int i = av; i < av + bv; ++i) {
				int g = a.order[i];
				++seen[g];
				for (int k = 0; k < 3; ++k)
					if (f(node, k) > boxes[g].lo[k] || f(node, 4 + k) < boxes[g].hi[k]) { std::puts("FAIL leaf box"); return 1; }
			}
			continue;
		}
		if (av % 2 != 0 || av + 1 >= a.n_nodes) { std::puts("FAIL pair layout"); return 1; }
		for (int c = av; c <= av + 1; ++c) {
			for (int k = 0; k < 3; ++k)
				if (f(node, k) > f(c, k) || f(node, 4 + k) < f(c, 4 + k)) { std::puts("FAIL child box"); return 1; }
			stack.push_back(c);
		}
	}
	for (int g = 0; g < n; ++g)
		if (seen[g] != 1) { std::puts("FAIL primitive coverage"); return 1; }
	std::printf("OK nodes %d depth %d max_leaf %d\n", a.n_nodes, a.depth, a.max_leaf);
	return 0;
}
