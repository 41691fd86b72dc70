// bvh.cpp — binned SAH build (host), then a layout pass that places the top
// levels breadth-first (so the first nodes can be staged in shared memory)
// and every deeper subtree depth-first, with each sibling pair on one
// 64-byte line.
#include "bvh.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <deque>
#include <limits>
#include <numeric>
#include <atomic>
#include <thread>

#include "core.h"

namespace are_core {
namespace {

struct TmpNode {
	double lo[3], hi[3];
	int32_t left = -1, right = -1;  // children in tmp, -1 for leaves
	int32_t first = 0, count = 0;   // range in `idx`
	int32_t depth = 0;
};

// a range's box and its centroids' box; known once the parent's binning has them
struct Bounds {
	double lo[3], hi[3], clo[3], chi[3];
	bool known = false;
};

constexpr int NBINS = 16;
constexpr int32_t SEQUENTIAL_BUILD_MAX = 1 << 15;  // primitives below which one thread builds the tree

inline double area(const double lo[3], const double hi[3]) {
	double dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
	if (dx < 0 || dy < 0 || dz < 0) return 0.0;
	return 2.0 * (dx * dy + dy * dz + dz * dx);
}

struct Builder {
	const std::vector<PrimBox> &boxes;
	std::vector<double> cen;  // 3 per prim
	std::vector<int32_t> idx;
	std::vector<TmpNode> nodes;
	int leaf_size;
	int max_depth = 0;

	Builder(const std::vector<PrimBox> &b, int leaf) : boxes(b), leaf_size(leaf) {}

	// Splits [first, first + count) into chunks run on threads when the range
	// is large (the top levels of the tree); fn(begin, end, chunk) fills
	// chunk-local results that the caller merges with order-free operations
	// (min, max, sums of integers), so the result does not depend on timing.
	static constexpr int32_t PAR_RANGE = 1 << 17;
	// set on pool threads that each take whole jobs: their passes run inline
	static bool &inline_passes() {
		static thread_local bool v = false;
		return v;
	}
	template <class F>
	static int chunked(int32_t first, int32_t count, F fn) {
		if (count < PAR_RANGE || inline_passes()) {
			fn(first, first + count, 0);
			return 1;
		}
		static const int hw = (int)hw_threads();
		const int nc = std::min(hw, (int)(count / (PAR_RANGE / 4)));
		if (nc <= 1) {
			fn(first, first + count, 0);
			return 1;
		}
		std::vector<std::thread> pool;
		for (int c = 1; c < nc; ++c)
			pool.emplace_back(fn, first + (int32_t)((int64_t)count * c / nc), first + (int32_t)((int64_t)count * (c + 1) / nc), c);
		fn(first, first + (int32_t)(count / nc), 0);
		for (std::thread &t : pool) t.join();
		return nc;
	}

	// Order-preserving partition of idx[first, first + count) by `left` on the
	// chunks of chunked(): each chunk counts its left elements, then scatters
	// both sides to their offsets in a copy.  Returns the first right index.
	// The chunks are fixed by the range alone, so the result does not depend
	// on timing.
	template <class Pred>
	int32_t partition_parallel(int32_t first, int32_t count, Pred left) {
		int32_t nleft[32] = { 0 };
		const int nc = chunked(first, count, [&](int32_t b0, int32_t b1, int c) {
			int32_t k = 0;
			for (int32_t i = b0; i < b1; ++i) k += left(idx[i]) ? 1 : 0;
			nleft[c] = k;
		});
		// chunk c covers [first + count c / nc, first + count (c + 1) / nc)
		int32_t lofs[32], rofs[32];
		int32_t total_left = 0;
		for (int c = 0; c < nc; ++c) total_left += nleft[c];
		int32_t l = first, r = first + total_left;
		for (int c = 0; c < nc; ++c) {
			const int32_t b0 = first + (int32_t)((int64_t)count * c / nc), b1 = first + (int32_t)((int64_t)count * (c + 1) / nc);
			lofs[c] = l, rofs[c] = r;
			l += nleft[c];
			r += (b1 - b0) - nleft[c];
		}
		std::vector<int32_t> out((size_t)count);
		chunked(first, count, [&](int32_t b0, int32_t b1, int c) {
			int32_t lo_ = lofs[c] - first, ro_ = rofs[c] - first;
			for (int32_t i = b0; i < b1; ++i) {
				const int32_t p = idx[i];
				if (left(p))
					out[lo_++] = p;
				else
					out[ro_++] = p;
			}
		});
		std::copy(out.begin(), out.end(), idx.begin() + first);
		return first + total_left;
	}

	void bounds(int32_t first, int32_t count, double lo[3], double hi[3], double clo[3], double chi[3]) const {
		struct Part {
			double lo[3], hi[3], clo[3], chi[3];
		};
		Part part[32];
		const int nc = chunked(first, count, [&](int32_t b0, int32_t b1, int c) {
			Part &q = part[c];
			for (int k = 0; k < 3; ++k) {
				q.lo[k] = q.clo[k] = std::numeric_limits<double>::infinity();
				q.hi[k] = q.chi[k] = -std::numeric_limits<double>::infinity();
			}
			for (int32_t i = b0; i < b1; ++i) {
				const PrimBox &b = boxes[idx[i]];
				for (int k = 0; k < 3; ++k) {
					q.lo[k] = std::min(q.lo[k], b.lo[k]);
					q.hi[k] = std::max(q.hi[k], b.hi[k]);
					double cc = cen[3 * idx[i] + k];
					q.clo[k] = std::min(q.clo[k], cc);
					q.chi[k] = std::max(q.chi[k], cc);
				}
			}
		});
		for (int k = 0; k < 3; ++k) {
			lo[k] = clo[k] = std::numeric_limits<double>::infinity();
			hi[k] = chi[k] = -std::numeric_limits<double>::infinity();
		}
		for (int c = 0; c < nc; ++c)
			for (int k = 0; k < 3; ++k) {
				lo[k] = std::min(lo[k], part[c].lo[k]), hi[k] = std::max(hi[k], part[c].hi[k]);
				clo[k] = std::min(clo[k], part[c].clo[k]), chi[k] = std::max(chi[k], part[c].chi[k]);
			}
	}

	// returns the split position (index in [first, first+count)) or -1 for a
	// leaf; kid[0], kid[1] get the two sides' bounds when the binned split
	// is taken (unions of the bins': min and max are exact, so they equal
	// a pass over the sides' primitives)
	int32_t split(int32_t first, int32_t count, int depth, const double lo[3], const double hi[3],
		const double clo[3], const double chi[3], Bounds kid[2]) {
		kid[0].known = kid[1].known = false;
		if (count <= 1) return -1;
		int axis = 0;
		for (int k = 1; k < 3; ++k)
			if (chi[k] - clo[k] > chi[axis] - clo[axis]) axis = k;
		double ext = chi[axis] - clo[axis];
		auto median = [&]() {
			int32_t mid = first + count / 2;
			std::nth_element(idx.begin() + first, idx.begin() + mid, idx.begin() + first + count,
				[&](int32_t a, int32_t b) {
					double ca = cen[3 * a + axis], cb = cen[3 * b + axis];
					return ca < cb || (ca == cb && a < b);
				});
			return mid;
		};
		if (depth >= MAX_BVH_DEPTH - 2) return count <= leaf_size ? -1 : median();
		if (!(ext > 0)) return count <= leaf_size ? -1 : median();
		// binned SAH along the widest centroid axis
		struct Bin {
			double lo[3], hi[3], clo[3], chi[3];
			int32_t n;
		};
		// the bins in use (bit b of `used`), each set by its first primitive:
		// min and max of one value are the value, and empty bins change no
		// union, so only used bins are visited
		struct BinSet {
			Bin bin[NBINS];
			uint32_t used = 0;
			void add(int b, const double *lo, const double *hi, const double *cc) {
				Bin &x = bin[b];
				if (!(used >> b & 1u)) {
					used |= 1u << b;
					for (int k = 0; k < 3; ++k) x.lo[k] = lo[k], x.hi[k] = hi[k], x.clo[k] = x.chi[k] = cc[k];
					x.n = 1;
					return;
				}
				for (int k = 0; k < 3; ++k) {
					x.lo[k] = std::min(x.lo[k], lo[k]), x.hi[k] = std::max(x.hi[k], hi[k]);
					x.clo[k] = std::min(x.clo[k], cc[k]), x.chi[k] = std::max(x.chi[k], cc[k]);
				}
				++x.n;
			}
			void merge(const BinSet &o) {
				for (uint32_t m = o.used; m; m &= m - 1) {
					const int b = __builtin_ctz(m);
					const Bin &y = o.bin[b];
					if (!(used >> b & 1u)) {
						used |= 1u << b;
						bin[b] = y;
						continue;
					}
					Bin &x = bin[b];
					for (int k = 0; k < 3; ++k) {
						x.lo[k] = std::min(x.lo[k], y.lo[k]), x.hi[k] = std::max(x.hi[k], y.hi[k]);
						x.clo[k] = std::min(x.clo[k], y.clo[k]), x.chi[k] = std::max(x.chi[k], y.chi[k]);
					}
					x.n += y.n;
				}
			}
		};
		double scale = NBINS / ext;
		auto bin_of = [&](int32_t p) {
			int b = (int)((cen[3 * p + axis] - clo[axis]) * scale);
			return std::min(std::max(b, 0), NBINS - 1);
		};
		// one range: binned straight into `bins`; the few large ranges: chunk-local bins on the heap, merged
		BinSet bins;
		std::vector<BinSet> heap_bins(count >= PAR_RANGE ? 32 : 0);
		auto bins_of = [&](int c) -> BinSet & { return heap_bins.empty() ? bins : heap_bins[c]; };
		const int nc = chunked(first, count, [&](int32_t b0, int32_t b1, int c) {
			BinSet &lb = bins_of(c);
			lb.used = 0;
			for (int32_t i = b0; i < b1; ++i) {
				const int32_t p = idx[i];
				lb.add(bin_of(p), boxes[p].lo, boxes[p].hi, &cen[3 * (size_t)p]);
			}
		});
		if (!heap_bins.empty())
			for (int c = 0; c < nc; ++c) bins.merge(heap_bins[c]);
		// SAH sweep over the used bins.  Candidate i splits between used bins
		// occ[i - 1] and occ[i]; every split position in that gap gives the same
		// two sides, and the first, occ[i - 1] + 1, is the one a sweep over all
		// positions keeps (the first minimum wins).
		int occ[NBINS], m = 0;
		for (uint32_t u = bins.used; u; u &= u - 1) occ[m++] = __builtin_ctz(u);
		double right_area[NBINS];
		int32_t right_n[NBINS];
		double rlo[3], rhi[3];
		for (int k = 0; k < 3; ++k) rlo[k] = std::numeric_limits<double>::infinity(), rhi[k] = -rlo[k];
		int32_t rn = 0;
		for (int i = m - 1; i > 0; --i) {
			const Bin &x = bins.bin[occ[i]];
			for (int k = 0; k < 3; ++k) rlo[k] = std::min(rlo[k], x.lo[k]), rhi[k] = std::max(rhi[k], x.hi[k]);
			rn += x.n;
			right_area[i] = area(rlo, rhi);
			right_n[i] = rn;
		}
		double llo[3], lhi[3];
		for (int k = 0; k < 3; ++k) llo[k] = std::numeric_limits<double>::infinity(), lhi[k] = -llo[k];
		int32_t ln = 0;
		double best = std::numeric_limits<double>::infinity();
		int best_b = -1;
		for (int i = 1; i < m; ++i) {
			const Bin &x = bins.bin[occ[i - 1]];
			for (int k = 0; k < 3; ++k) llo[k] = std::min(llo[k], x.lo[k]), lhi[k] = std::max(lhi[k], x.hi[k]);
			ln += x.n;
			double c = area(llo, lhi) * ln + right_area[i] * right_n[i];
			if (c < best) best = c, best_b = occ[i - 1] + 1;
		}
		double parent = area(lo, hi);
		double leaf_cost = (double)count;
		double split_cost = parent > 0 ? 0.5 + best / parent : std::numeric_limits<double>::infinity();
		if (best_b < 0) return count <= leaf_size ? -1 : median();
		if (count <= leaf_size && split_cost >= leaf_cost) return -1;
		int32_t mid;
		if (count >= PAR_RANGE) {
			mid = partition_parallel(first, count, [&](int32_t p) { return bin_of(p) < best_b; });
		} else {
			auto it = std::partition(idx.begin() + first, idx.begin() + first + count,
				[&](int32_t p) { return bin_of(p) < best_b; });
			mid = (int32_t)(it - idx.begin());
		}
		if (mid == first || mid == first + count) return median();
		for (int side = 0; side < 2; ++side) {
			Bounds &w = kid[side];
			for (int k = 0; k < 3; ++k)
				w.lo[k] = w.clo[k] = std::numeric_limits<double>::infinity(), w.hi[k] = w.chi[k] = -w.lo[k];
		}
		for (int i = 0; i < m; ++i) {
			const Bin &x = bins.bin[occ[i]];
			Bounds &w = kid[occ[i] < best_b ? 0 : 1];
			for (int k = 0; k < 3; ++k) {
				w.lo[k] = std::min(w.lo[k], x.lo[k]), w.hi[k] = std::max(w.hi[k], x.hi[k]);
				w.clo[k] = std::min(w.clo[k], x.clo[k]), w.chi[k] = std::max(w.chi[k], x.chi[k]);
			}
		}
		kid[0].known = kid[1].known = true;
		return mid;
	}

	void build() {
		int32_t n = (int32_t)boxes.size();
		cen.resize(3 * (size_t)n);
		idx.resize(n);
		std::iota(idx.begin(), idx.end(), 0);
		for (int32_t i = 0; i < n; ++i)
			for (int k = 0; k < 3; ++k) cen[3 * i + k] = 0.5 * (boxes[i].lo[k] + boxes[i].hi[k]);
		nodes.reserve(2 * (size_t)n);
		struct Job {
			int32_t node, first, count, depth;
			Bounds bounds;  // of [first, first + count), when the parent's split knew them
		};
		if (n < SEQUENTIAL_BUILD_MAX) {
			// small scenes: the whole tree on this thread (starting threads would cost more)
			std::vector<Job> st{ { 0, 0, n, 0, {} } };
			nodes.push_back(TmpNode{});
			while (!st.empty()) {
				Job j = st.back();
				st.pop_back();
				expand(j, nodes, st, max_depth);
			}
			return;
		}
		// The top of the tree is split level by level.  A level's jobs (disjoint
		// ranges of idx) are split in parallel, whole jobs per thread, once there
		// are enough of them; before that one at a time with chunk-parallel
		// passes.  Children are then allocated in job order.  Subtrees below
		// par_min primitives are set aside and built by worker threads, each into
		// its own node list, then appended.  Every split depends only on the
		// subtree's own primitives, so the tree is the one a single thread builds.
		static const int n_hw = (int)hw_threads();
		const int32_t par_min = std::max<int32_t>(4096, n / (4 * n_hw));
		std::vector<Job> deferred;
		std::vector<Job> level{ { 0, 0, n, 0, {} } };
		nodes.push_back(TmpNode{});
		while (!level.empty()) {
			std::vector<int32_t> mids(level.size());
			std::vector<std::array<Bounds, 2>> kid_bounds(level.size());
			auto split_job = [&](size_t k) {
				const Job &j = level[k];
				Bounds bb = j.bounds;
				if (!bb.known) bounds(j.first, j.count, bb.lo, bb.hi, bb.clo, bb.chi);
				TmpNode &t = nodes[j.node];
				std::memcpy(t.lo, bb.lo, sizeof bb.lo);
				std::memcpy(t.hi, bb.hi, sizeof bb.hi);
				t.depth = j.depth;
				mids[k] = split(j.first, j.count, j.depth, bb.lo, bb.hi, bb.clo, bb.chi, kid_bounds[k].data());
			};
			if ((int)level.size() >= n_hw) {
				std::atomic<size_t> next{ 0 };
				auto worker = [&]() {
					inline_passes() = true;
					for (size_t k; (k = next.fetch_add(1)) < level.size();) split_job(k);
					inline_passes() = false;
				};
				std::vector<std::thread> pool;
				for (int t = 1; t < n_hw; ++t) pool.emplace_back(worker);
				worker();
				for (std::thread &t : pool) t.join();
			} else {
				for (size_t k = 0; k < level.size(); ++k) split_job(k);
			}
			std::vector<Job> below;
			for (size_t k = 0; k < level.size(); ++k) {
				const Job &j = level[k];
				max_depth = std::max(max_depth, j.depth);
				const int32_t mid = mids[k];
				if (mid < 0) {
					nodes[j.node].first = j.first;
					nodes[j.node].count = j.count;
					continue;
				}
				const int32_t l = (int32_t)nodes.size();
				nodes.push_back(TmpNode{});
				nodes.push_back(TmpNode{});
				nodes[j.node].left = l;
				nodes[j.node].right = l + 1;
				const Job kids[2] = { { l, j.first, mid - j.first, j.depth + 1, kid_bounds[k][0] },
					{ l + 1, mid, j.first + j.count - mid, j.depth + 1, kid_bounds[k][1] } };
				for (const Job &c : kids) {
					if (c.count < par_min && c.count > leaf_size)
						deferred.push_back(c);
					else
						below.push_back(c);
				}
			}
			level.swap(below);
		}
		if (deferred.empty()) return;
		std::vector<std::vector<TmpNode>> local(deferred.size());
		std::vector<int> local_depth(deferred.size(), 0);
		// largest subtrees first, so no large one starts last (each writes only its own list)
		std::vector<size_t> by_size(deferred.size());
		std::iota(by_size.begin(), by_size.end(), (size_t)0);
		std::stable_sort(by_size.begin(), by_size.end(),
			[&](size_t x, size_t y) { return deferred[x].count > deferred[y].count; });
		std::atomic<size_t> next_job{ 0 };
		auto worker = [&]() {
			inline_passes() = true;  // whole subtrees per thread
			for (size_t q; (q = next_job.fetch_add(1)) < deferred.size();) {
				const size_t k = by_size[q];
				std::vector<TmpNode> &ln = local[k];
				std::vector<Job> st;
				ln.reserve(2 * (size_t)deferred[k].count);  // a binary tree over count primitives, leaves of one or more
				ln.push_back(TmpNode{});
				st.push_back({ 0, deferred[k].first, deferred[k].count, deferred[k].depth, deferred[k].bounds });
				while (!st.empty()) {
					Job j = st.back();
					st.pop_back();
					expand(j, ln, st, local_depth[k]);
				}
			}
			inline_passes() = false;
		};
		const unsigned nthreads = (unsigned)std::min<size_t>(hw_threads(), deferred.size());
		std::vector<std::thread> pool;
		for (unsigned t = 1; t < nthreads; ++t) pool.emplace_back(worker);
		worker();
		for (std::thread &t : pool) t.join();
		// append each subtree (in job order, copied in parallel): local node 0
		// fills the placeholder, the rest shift by base - 1
		std::vector<int32_t> base(deferred.size());
		size_t total = nodes.size();
		for (size_t k = 0; k < deferred.size(); ++k) {
			base[k] = (int32_t)total;
			total += local[k].size() - 1;
			max_depth = std::max(max_depth, local_depth[k]);
		}
		nodes.resize(total);
		run_jobs(deferred.size(), nthreads, [&](size_t k) {
			const std::vector<TmpNode> &ln = local[k];
			const int32_t b0 = base[k];
			auto map = [&](int32_t i) { return i < 0 ? i : b0 + i - 1; };
			TmpNode root = ln[0];
			root.left = map(root.left), root.right = map(root.right);
			nodes[deferred[k].node] = root;
			for (size_t i = 1; i < ln.size(); ++i) {
				TmpNode t = ln[i];
				t.left = map(t.left), t.right = map(t.right);
				nodes[(size_t)b0 + i - 1] = t;
			}
		});
	}

	// one step of the build: bounds and split of job j's range into node j.node of `ns`
	template <class JobT>
	void expand(const JobT &j, std::vector<TmpNode> &ns, std::vector<JobT> &stack, int &depth_max) {
		Bounds bb = j.bounds;
		if (!bb.known) bounds(j.first, j.count, bb.lo, bb.hi, bb.clo, bb.chi);
		TmpNode &t = ns[j.node];
		std::memcpy(t.lo, bb.lo, sizeof bb.lo);
		std::memcpy(t.hi, bb.hi, sizeof bb.hi);
		t.depth = j.depth;
		depth_max = std::max(depth_max, j.depth);
		Bounds kid[2];
		int32_t mid = split(j.first, j.count, j.depth, bb.lo, bb.hi, bb.clo, bb.chi, kid);
		if (mid < 0) {
			ns[j.node].first = j.first;
			ns[j.node].count = j.count;
			return;
		}
		int32_t l = (int32_t)ns.size();
		ns.push_back(TmpNode{});
		ns.push_back(TmpNode{});
		ns[j.node].left = l;
		ns[j.node].right = l + 1;
		stack.push_back({ l + 1, mid, j.first + j.count - mid, j.depth + 1, kid[1] });
		stack.push_back({ l, j.first, mid - j.first, j.depth + 1, kid[0] });
	}
};

}  // namespace

BvhResult build_bvh(const std::vector<PrimBox> &boxes, int leaf_size) {
	BvhResult r;
	if (leaf_size <= 0) leaf_size = 4;
	if (leaf_size > 64) leaf_size = 64;
	if (boxes.empty()) {
		r.n_nodes = 2;
		r.nodes.assign(16, 0.0f);
		// an empty leaf whose box is inverted: nothing is ever hit
		for (int k = 0; k < 3; ++k) r.nodes[k] = 1.0f, r.nodes[4 + k] = -1.0f;
		return r;
	}
	Builder b(boxes, leaf_size);
	b.build();

	double scale = 0.0;
	for (const PrimBox &pb : boxes)
		for (int k = 0; k < 3; ++k) scale = std::max(scale, std::max(std::fabs(pb.lo[k]), std::fabs(pb.hi[k])));
	r.box_pad = (float)(scale * std::ldexp(1.0, -19)) + 1e-30f;

	// layout: root at 0, padding at 1, sibling pairs at even indices; pairs are
	// allocated breadth-first until 1024 nodes exist, depth-first afterwards.
	const size_t ntmp = b.nodes.size();
	const unsigned nthreads = ntmp < ((size_t)1 << 16) ? 1u : hw_threads();
	std::vector<int32_t> slot(ntmp, -1);
	slot[0] = 0;
	int32_t next = 2;
	std::deque<int32_t> work;
	work.push_back(0);
	while (!work.empty() && next < SMEM_NODES) {
		const int32_t t = work.front();
		work.pop_front();
		const TmpNode &tn = b.nodes[t];
		if (tn.left < 0) continue;
		slot[tn.left] = next;
		slot[tn.right] = next + 1;
		next += 2;
		if (next < SMEM_NODES) {
			work.push_back(tn.left);
			work.push_back(tn.right);
		} else {  // depth-first from here: the left child first
			work.push_back(tn.right);
			work.push_back(tn.left);
		}
	}
	// Depth-first, the queued subtrees are laid out one after another, last
	// queued first, each over a contiguous run of slots as long as its node
	// count less one: one parallel pass counts each subtree's nodes, a second
	// lays each out on its own.
	std::vector<std::pair<int32_t, int32_t>> dfs;  // (subtree root, first slot of its descendants)
	for (auto it = work.rbegin(); it != work.rend(); ++it) dfs.push_back({ *it, 0 });
	run_jobs(dfs.size(), nthreads, [&](size_t k) {
		std::vector<int32_t> st{ dfs[k].first };
		int32_t c = 0;
		while (!st.empty()) {
			const TmpNode &tn = b.nodes[st.back()];
			st.pop_back();
			++c;
			if (tn.left >= 0) st.push_back(tn.left), st.push_back(tn.right);
		}
		dfs[k].second = c;
	});
	for (auto &d : dfs) {
		const int32_t c = d.second;
		d.second = next;
		next += c - 1;
	}
	run_jobs(dfs.size(), nthreads, [&](size_t k) {
		std::vector<int32_t> st{ dfs[k].first };
		int32_t nx = dfs[k].second;
		while (!st.empty()) {
			const TmpNode &tn = b.nodes[st.back()];
			st.pop_back();
			if (tn.left < 0) continue;
			slot[tn.left] = nx;
			slot[tn.right] = nx + 1;
			nx += 2;
			st.push_back(tn.right);
			st.push_back(tn.left);
		}
	});
	r.n_nodes = next;
	r.nodes.assign(8 * (size_t)next, 0.0f);
	// padding node 1: inverted box, never hit
	for (int k = 0; k < 3; ++k) r.nodes[8 + k] = 1.0f, r.nodes[12 + k] = -1.0f;

	// leaves keep the primitive ranges of the build order; node records are
	// written in parallel ranges (each node independently)
	r.order = b.idx;
	std::vector<int32_t> part_max_leaf(nthreads, 0);
	auto write_range = [&](unsigned part) {
		int32_t &max_leaf = part_max_leaf[part];
		for (size_t t = ntmp * part / nthreads; t < ntmp * (part + 1) / nthreads; ++t) {
			const TmpNode &tn = b.nodes[t];
			float *o = &r.nodes[8 * (size_t)slot[t]];
			for (int k = 0; k < 3; ++k) {
				float lo = (float)tn.lo[k], hi = (float)tn.hi[k];
				if ((double)lo > tn.lo[k]) lo = std::nextafter(lo, -INFINITY);
				if ((double)hi < tn.hi[k]) hi = std::nextafter(hi, INFINITY);
				o[k] = lo - r.box_pad;
				o[4 + k] = hi + r.box_pad;
			}
			int32_t a, bb;
			if (tn.left < 0) {
				a = tn.first;
				bb = tn.count;
				max_leaf = std::max(max_leaf, tn.count);
			} else {
				a = slot[tn.left];
				bb = 0;
			}
			std::memcpy(&o[3], &a, 4);
			std::memcpy(&o[7], &bb, 4);
		}
	};
	{
		std::vector<std::thread> pool;
		for (unsigned t = 1; t < nthreads; ++t) pool.emplace_back(write_range, t);
		write_range(0);
		for (std::thread &t : pool) t.join();
	}
	r.depth = b.max_depth;
	r.max_leaf = *std::max_element(part_max_leaf.begin(), part_max_leaf.end());
	return r;
}

std::vector<float> collapse_bvh4(const BvhResult &bvh, int bfs_nodes) {
	std::vector<float> out;
	const float *rec = bvh.nodes.data();
	auto is_leaf = [&](int32_t r) {
		int32_t b;
		std::memcpy(&b, &rec[8 * (size_t)r + 7], 4);
		return b != 0;
	};
	auto child = [&](int32_t r) {
		int32_t a;
		std::memcpy(&a, &rec[8 * (size_t)r + 3], 4);
		return a;
	};
	auto area = [&](int32_t r) {
		const float *o = &rec[8 * (size_t)r];
		double dx = (double)o[4] - o[0], dy = (double)o[5] - o[1], dz = (double)o[6] - o[2];
		return dx * dy + dy * dz + dz * dx;
	};
	if (bvh.n_nodes < 4 || is_leaf(0)) return out;
	// children (binary record indices) of the wide node made from binary interior record r
	auto gather = [&](int32_t r, int32_t kids[4]) {
		int n = 2;
		kids[0] = child(r), kids[1] = child(r) + 1;
		while (n < 4) {
			int best = -1;
			double ba = -1.0;
			for (int k = 0; k < n; ++k)
				if (!is_leaf(kids[k]) && area(kids[k]) > ba) ba = area(kids[k]), best = k;
			if (best < 0) break;
			const int32_t c = child(kids[best]);
			kids[best] = c;
			kids[n++] = c + 1;
		}
		return n;
	};
	// wide nodes in order: breadth-first, then depth-first (as the binary layout)
	std::vector<int32_t> src;  // binary interior record of each wide node
	src.push_back(0);
	std::deque<int32_t> work;  // wide node indices whose children are not numbered yet
	work.push_back(0);
	std::vector<std::array<int32_t, 4>> refs;  // per wide node: wide index of each interior child, -1 otherwise
	std::vector<std::array<int32_t, 4>> kids_of;
	std::vector<int> nkids;
	const size_t cap = (size_t)bvh.n_nodes / 2 + 1;  // at most one wide node per binary interior node
	src.reserve(cap), refs.reserve(cap), kids_of.reserve(cap), nkids.reserve(cap);
	refs.push_back({ -1, -1, -1, -1 });
	kids_of.push_back({ -1, -1, -1, -1 });
	nkids.push_back(0);
	// wide node w: its children (records) and the numbers of its interior children,
	// taken from next_index(binary record) in child order
	auto expand = [&](int32_t w, auto &&next_index, int32_t inner[4]) {
		int32_t kids[4];
		const int n = gather(src[w], kids);
		nkids[w] = n;
		int n_inner = 0;
		for (int k = 0; k < n; ++k) {
			kids_of[w][k] = kids[k];
			if (is_leaf(kids[k])) continue;
			const int32_t m = next_index(kids[k]);
			refs[w][k] = m;
			inner[n_inner++] = m;
		}
		return n_inner;
	};
	auto append = [&](int32_t r) {
		src.push_back(r);
		refs.push_back({ -1, -1, -1, -1 });
		kids_of.push_back({ -1, -1, -1, -1 });
		nkids.push_back(0);
		return (int32_t)src.size() - 1;
	};
	while (!work.empty() && (int)src.size() < bfs_nodes) {
		const int32_t w = work.front();
		work.pop_front();
		int32_t inner[4];
		const int n_inner = expand(w, append, inner);
		if ((int)src.size() < bfs_nodes) {
			for (int k = 0; k < n_inner; ++k) work.push_back(inner[k]);
		} else {  // depth-first from here: the first child next
			for (int k = n_inner - 1; k >= 0; --k) work.push_back(inner[k]);
		}
	}
	// Depth-first, the queued wide nodes' subtrees are numbered one after
	// another, last queued first, each over a contiguous run as long as its
	// count of wide descendants: one parallel pass counts them, a second
	// numbers and fills each subtree on its own.
	const unsigned nthreads = bvh.n_nodes < (1 << 16) ? 1u : hw_threads();
	std::vector<int32_t> roots(work.rbegin(), work.rend());
	std::vector<int32_t> first(roots.size());
	run_jobs(roots.size(), nthreads, [&](size_t k) {
		std::vector<int32_t> st{ src[roots[k]] };
		int32_t c = 0;
		while (!st.empty()) {
			int32_t kids[4];
			const int n = gather(st.back(), kids);
			st.pop_back();
			for (int i = 0; i < n; ++i)
				if (!is_leaf(kids[i])) ++c, st.push_back(kids[i]);
		}
		first[k] = c;
	});
	size_t total = src.size();
	for (int32_t &f : first) {
		const int32_t c = f;
		f = (int32_t)total;
		total += c;
	}
	src.resize(total);
	refs.resize(total, { -1, -1, -1, -1 });
	kids_of.resize(total, { -1, -1, -1, -1 });
	nkids.resize(total, 0);
	run_jobs(roots.size(), nthreads, [&](size_t k) {
		std::vector<int32_t> st{ roots[k] };
		int32_t nx = first[k];
		auto take = [&](int32_t r) {
			src[nx] = r;
			return nx++;
		};
		while (!st.empty()) {
			const int32_t w = st.back();
			st.pop_back();
			int32_t inner[4];
			const int n_inner = expand(w, take, inner);
			for (int i = n_inner - 1; i >= 0; --i) st.push_back(inner[i]);
		}
	});
	const size_t nw = src.size();
	out.assign(32 * nw, 0.0f);
	const size_t nparts = nthreads > 1 ? 4 * (size_t)nthreads : 1;
	run_jobs(nparts, nthreads, [&](size_t part) {
		for (size_t w = nw * part / nparts; w < nw * (part + 1) / nparts; ++w) {
			for (int k = 0; k < 4; ++k) {
				float *o = &out[32 * w + 8 * (size_t)k];
				if (k >= nkids[w]) {
					// unused slot: an empty leaf (count -1, no primitives), so entering it does nothing
					// (a min > max box is no guard: the slab test orders each axis's two planes)
					const int32_t a = 0, b = -1;
					for (int j = 0; j < 3; ++j) o[j] = 1.0f, o[4 + j] = -1.0f;
					std::memcpy(&o[3], &a, 4);
					std::memcpy(&o[7], &b, 4);
					continue;
				}
				const int32_t r = kids_of[w][k];
				std::memcpy(o, &rec[8 * (size_t)r], 32);  // box, first / count as in the binary record
				if (!is_leaf(r)) {
					const int32_t a = refs[w][k], b = 0;
					std::memcpy(&o[3], &a, 4);
					std::memcpy(&o[7], &b, 4);
				}
			}
		}
	});
	return out;
}

}  // namespace are_core
