// Host-side check of the BVH builder (csrc/bvh.cpp), compiled by
// tests/test_bvh_host.py: random primitive boxes -> two builds must give the
// same node array (the parallel subtree build is deterministic), every
// primitive sits in exactly one leaf, every node's box contains its
// children's, and the pair layout holds (children at even indices).  The
// 4-wide collapse (collapse_bvh4) is checked the same way: every primitive in
// exactly one leaf, each child record's box inside its parent record's, the
// leaves those of the binary tree, unused slots empty leaves.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "bvh.h"

using are_core::BvhResult;
using are_core::PrimBox;

// FNV-1a over the bytes of both trees and the leaf order: a fingerprint of the build's decisions
static unsigned long long fingerprint(const BvhResult &a, const std::vector<float> &w) {
	unsigned long long x = 1469598103934665603ull;
	auto mix = [&](const void *p, size_t n) {
		const unsigned char *c = (const unsigned char *)p;
		for (size_t i = 0; i < n; ++i) x = (x ^ c[i]) * 1099511628211ull;
	};
	mix(a.nodes.data(), a.nodes.size() * sizeof(float));
	mix(a.order.data(), a.order.size() * sizeof(int32_t));
	mix(w.data(), w.size() * sizeof(float));
	return x;
}

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

	// the 4-wide tree
	const std::vector<float> w = are_core::collapse_bvh4(a, 256);
	if (ii(0, 7) > 0) {  // the binary root is a leaf: no wide tree
		if (!w.empty()) { std::puts("FAIL wide tree over a single leaf"); return 1; }
		std::printf("OK nodes %d depth %d max_leaf %d wide 0 fingerprint %016llx\n", a.n_nodes, a.depth, a.max_leaf,
			fingerprint(a, w));
		return 0;
	}
	if (w.size() % 32 != 0 || w.empty()) { std::puts("FAIL wide size"); return 1; }
	const int nw = (int)(w.size() / 32);
	auto wf = [&](int node, int k, int j) { return w[32 * (size_t)node + 8 * (size_t)k + j]; };
	auto wi = [&](int node, int k, int j) { int32_t v; std::memcpy(&v, &w[32 * (size_t)node + 8 * (size_t)k + j], 4); return v; };
	std::vector<int> seen4((size_t)n, 0), visits((size_t)nw, 0);
	// (wide node, parent box) pairs; the root's box is binary record 0
	struct Item { int node; float lo[3], hi[3]; };
	std::vector<Item> work;
	work.push_back({ 0, { f(0, 0), f(0, 1), f(0, 2) }, { f(0, 4), f(0, 5), f(0, 6) } });
	int leaves4 = 0;
	while (!work.empty()) {
		Item it = work.back();
		work.pop_back();
		if (it.node < 0 || it.node >= nw || ++visits[it.node] != 1) { std::puts("FAIL wide reference"); return 1; }
		int used = 0;
		for (int k = 0; k < 4; ++k) {
			if (wi(it.node, k, 7) == -1) continue;  // unused slot: an empty leaf
			++used;
			for (int j = 0; j < 3; ++j)
				if (wf(it.node, k, j) < it.lo[j] || wf(it.node, k, 4 + j) > it.hi[j]) { std::puts("FAIL wide child box"); return 1; }
			const int av = wi(it.node, k, 3), bv = wi(it.node, k, 7);
			if (bv > 0) {
				++leaves4;
				for (int i = av; i < av + bv; ++i) {
					int g = a.order[i];
					++seen4[g];
					for (int j = 0; j < 3; ++j)
						if (wf(it.node, k, j) > boxes[g].lo[j] || wf(it.node, k, 4 + j) < boxes[g].hi[j]) { std::puts("FAIL wide leaf box"); return 1; }
				}
			} else {
				work.push_back({ av, { wf(it.node, k, 0), wf(it.node, k, 1), wf(it.node, k, 2) },
					{ wf(it.node, k, 4), wf(it.node, k, 5), wf(it.node, k, 6) } });
			}
		}
		if (used < 2) { std::puts("FAIL wide node with fewer than two children"); return 1; }
	}
	for (int g = 0; g < n; ++g)
		if (seen4[g] != 1) { std::puts("FAIL wide primitive coverage"); return 1; }
	for (int i = 0; i < nw; ++i)
		if (visits[i] != 1) { std::puts("FAIL wide node unreachable"); return 1; }

	// the device's 4-wide walk (traverse.cuh closest_hit4, no primitive tests, no culling by a best hit)
	// on random rays: it ends within n_nodes4 steps and reaches exactly the leaves whose own box the ray
	// enters (every ancestor box contains it), unused slots included as empty leaves
	std::uniform_real_distribution<double> D(-1.0, 1.0);
	auto slab = [](const float *lo, const float *hi, const float o[3], const float inv[3]) {
		float tl = 0.0f, th = INFINITY;
		for (int j = 0; j < 3; ++j) {
			float t0 = std::fma(lo[j], inv[j], -o[j] * inv[j]), t1 = std::fma(hi[j], inv[j], -o[j] * inv[j]);
			tl = std::fmax(tl, std::fmin(t0, t1));
			th = std::fmin(th, std::fmax(t0, t1));
		}
		return tl <= th;
	};
	for (int r = 0; r < 2000; ++r) {
		float o[3], dv[3], inv[3];
		for (int j = 0; j < 3; ++j) o[j] = (float)(1.5 * U(rng)), dv[j] = (float)D(rng);
		for (int j = 0; j < 3; ++j) inv[j] = 1.0f / (dv[j] != 0.0f ? dv[j] : 1e-20f);
		std::vector<int> st{ 0 };
		std::vector<int> got, want;
		int steps = 0;
		while (!st.empty()) {
			int node = st.back();
			st.pop_back();
			if (++steps > nw) { std::puts("FAIL wide walk does not end"); return 1; }
			for (int k = 0; k < 4; ++k) {
				float lo[3] = { wf(node, k, 0), wf(node, k, 1), wf(node, k, 2) };
				float hi[3] = { wf(node, k, 4), wf(node, k, 5), wf(node, k, 6) };
				if (!slab(lo, hi, o, inv)) continue;
				const int av = wi(node, k, 3), bv = wi(node, k, 7);
				if (bv == 0) {
					if (av <= 0 || av >= nw) { std::puts("FAIL wide walk reference"); return 1; }
					st.push_back(av);
				} else if (bv > 0) {
					got.push_back(av);
				}
			}
		}
		// leaves of the binary tree whose box the ray enters
		std::vector<int> bs{ 0 };
		while (!bs.empty()) {
			int node = bs.back();
			bs.pop_back();
			float lo[3] = { f(node, 0), f(node, 1), f(node, 2) }, hi[3] = { f(node, 4), f(node, 5), f(node, 6) };
			if (!slab(lo, hi, o, inv)) continue;
			if (ii(node, 7) > 0) {
				want.push_back(ii(node, 3));
			} else {
				bs.push_back(ii(node, 3));
				bs.push_back(ii(node, 3) + 1);
			}
		}
		std::sort(got.begin(), got.end());
		std::sort(want.begin(), want.end());
		// the wide walk skips collapsed levels, so it may enter a leaf whose binary ancestor it did not test
		if (!std::includes(got.begin(), got.end(), want.begin(), want.end())) { std::puts("FAIL wide walk misses a leaf"); return 1; }
	}
	std::printf("OK nodes %d depth %d max_leaf %d wide %d leaves %d fingerprint %016llx\n", a.n_nodes, a.depth, a.max_leaf,
		nw, leaves4, fingerprint(a, w));
	return 0;
}
