// render.cu — the path tracer (megakernel and wavefront schedules) and the
// batched closest-hit query.
//
// Replaces rt.cpp render() / trace() / intersect() (experiments/rt.cpp:209-374).
// The reference walks pixels one by one and recurses per path on one host
// thread.  Here work items are (pixel, chunk of samples); a path slot runs an
// item's samples in order and keeps their Kahan sums, so the per-item sums -
// and the image - do not depend on scheduling; `resolve` adds the items of
// each pixel in chunk order.  Two schedules run the slots:
//
//   megakernel (default): `tail` as one persistent launch, one slot per
//     resident thread; a thread traces its path to the end, accumulates it,
//     takes its next sample or work item and goes on, the path state and the
//     slot's sums in registers.  One instantiation per closest-hit strategy
//     (warp-cooperative linear scan of a tiny scene; binary or 4-wide BVH).
//   wavefront: a pool of P paths in HBM as 64-byte SoA queue records (the
//     path state travels with its ray), two kernels per iteration over
//     compacted queues, captured K iterations at a time in a CUDA graph:
//       intersect : closest hit of every queued ray
//       shade     : emission + scatter + Russian roulette; a surviving path
//                   appends its next ray, a finished one accumulates and
//                   appends its slot's next camera ray (warp-ballot
//                   compaction, one atomic per warp)
//     and, when every item is taken and few paths remain, `tail` finishes
//     them in one launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "scene.h"
#include "shade.cuh"
#include "mega.cuh"
#include "path.cuh"
#include "traverse.cuh"
#include "wave.cuh"

namespace are_core {

// ---------------------------------------------------------------------------
// batched closest hit (are_intersect)

__device__ __forceinline__ float4 hit_record(const Hit &h) {
	return h.leaf >= 0 ? make_float4(h.t, __int_as_float(h.gid), h.u, h.v)
					   : make_float4(__int_as_float(0x7f800000), __int_as_float(-1), 0.f, 0.f);
}

// Closest hits of this thread's rays i, i + stride, ... (< n) over the 4-wide
// tree with the lanes' walks interleaved: each round steps either the lanes
// at a wide node or those at a leaf (whichever are more), and a lane whose
// walk has ended stores its hit and begins its next ray at once, so no lane
// waits for the longest walk of its warp (Aila and Laine's persistent threads
// with dynamic ray fetch, per lane).  The same hits as closest_hit4.  Every
// lane of the warp calls it (converged).
//   load(i, o, d, tmin, tmax): ray i;  store(i, hit): its closest hit
template <int SHORT, class Load, class Store>
__device__ __forceinline__ void walk_rays4(const DevScene &S, const float4 *__restrict__ snodes, int n_snodes,
	int4 *__restrict__ sstack, int64_t n, uint32_t &err, Load load, Store store) {
	WalkStack<MAX_STACK4 - SHORT> st;
	Walk w;
	const int64_t stride = (int64_t)gridDim.x * blockDim.x;
	int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
	f3 o{}, d{};
	float tmin = 0.f, tmax = 0.f;
	// takes rays until one needs a walk (a ray that misses the root's box gets its miss at once)
	auto fetch = [&]() -> bool {
		for (; i < n; i += stride) {
			load(i, o, d, tmin, tmax);
			if (walk4_begin(S, o, d, tmin, tmax, w)) return true;
			store(i, w.best);
		}
		return false;
	};
	bool walking = fetch();
	while (__any_sync(0xffffffffu, walking)) {
		const unsigned walkers = __ballot_sync(0xffffffffu, walking);
		const unsigned at_leaf = __ballot_sync(0xffffffffu, walking && w.b > 0);
		const bool leaf_round = 2 * __popc(at_leaf) >= __popc(walkers);
		if (walking && (w.b > 0) == leaf_round &&
			!walk4_step<SHORT>(S, snodes, n_snodes, o, d, tmin, tmax, err, sstack, st, w)) {
			store(i, w.best);
			i += stride;
			walking = fetch();
		}
	}
}

// LINEAR: a scene of at most LINEAR_MAX primitives, scanned from shared memory
// (its instantiation holds the staged primitives and the per-warp scratch);
// else the BVH with its top levels in shared memory, walked ray by ray, or
// (WALKS) the 4-wide tree with the lanes' walks interleaved (walk_rays4: 1.3x
// the rays per second on the 2M-triangle mesh; on binary trees it gained
// nothing on the mesh and lost a third on a few dozen quads).
template <bool LINEAR, bool WALKS = false>
__global__ void __launch_bounds__(BLOCK) k_intersect_batch(DevScene S, const float4 *__restrict__ rays, int64_t n,
	float4 *__restrict__ hits, unsigned *err_word) {
	__shared__ float4 snodes[LINEAR ? 6 * LINEAR_MAX : 2 * SMEM_NODES];
	__shared__ WarpHitScratch scratch[LINEAR ? BLOCK / 32 : 1];
	int n_snodes = 0;
	constexpr bool linear = LINEAR;
	if (linear) {
		stage_prims(S, snodes);
		__syncthreads();
	} else {
		stage_bvh(S, snodes, n_snodes);
	}
	uint32_t err = 0;
	if constexpr (WALKS) {
		walk_rays4<0>(S, snodes, n_snodes, nullptr, n, err,
			[&](int64_t i, f3 &o, f3 &d, float &tmin, float &tmax) {
				const float4 r0 = rays[2 * i], r1 = rays[2 * i + 1];
				o = ld3(r0), d = ld3(r1), tmin = r0.w, tmax = r1.w;
			},
			[&](int64_t i, const Hit &h) { hits[i] = hit_record(h); });
		if (err) atomicOr(err_word, err);
		return;
	}
	// whole warps walk the rays together (the linear scan is warp-cooperative)
	for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
		const int64_t i = base + threadIdx.x;
		const bool active = i < n;
		float4 r0 = make_float4(0.f, 0.f, 0.f, 0.f), r1 = r0;
		if (active) r0 = rays[2 * i], r1 = rays[2 * i + 1];
		Hit h;
		// the cooperative scan orders hits by t's bits, which needs t > 0: rays with tmin >= 0
		if (linear && __all_sync(0xffffffffu, !active || r0.w >= 0.0f)) {
			h = closest_hit_linear_warp(snodes, S.n_leaves, S.triangle_test, ld3(r0), ld3(r1), r0.w, r1.w, active,
				scratch[threadIdx.x >> 5]);
		} else if (linear && active) {
			h = closest_hit_linear(snodes, S.n_leaves, S.triangle_test, ld3(r0), ld3(r1), r0.w, r1.w);
		} else if (active) {
			h = closest_hit_any(S, snodes, n_snodes, ld3(r0), ld3(r1), r0.w, r1.w, err);
		}
		if (active) hits[i] = hit_record(h);
	}
	if (err) atomicOr(err_word, err);
}

// ---------------------------------------------------------------------------
// wavefront kernels

__global__ void __launch_bounds__(BLOCK) k_init(Wave W, int n_first) {
	// slot s takes work item s; its first camera ray goes to queue 0 position s
	for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < W.P; s += gridDim.x * blockDim.x) {
		W.acc_s[s] = make_float4(0.f, 0.f, 0.f, 0.f);
		W.acc_c[s] = make_float4(0.f, 0.f, 0.f, 0.f);
		W.acc_q[s] = make_float4(0.f, 0.f, 0.f, 0.f);
		if (s < n_first) put_camera_ray(W, 0, (unsigned)s, s, s, 0);
	}
}

// LINEAR: the warp-cooperative scan of a tiny scene; else the binary tree, or
// the 4-wide tree (WIDE), with the top INTERSECT_SHORT_STACK stack entries of
// each thread in shared memory.
template <bool LINEAR, bool WIDE = false>
__global__ void __launch_bounds__(BLOCK) k_intersect(DevScene S, Wave W, int par) {
	__shared__ float4 snodes[LINEAR ? 6 * LINEAR_MAX : 2 * SMEM_NODES];
	__shared__ WarpHitScratch scratch[LINEAR ? BLOCK / 32 : 1];
	__shared__ int4 sstack[LINEAR ? 1 : INTERSECT_SHORT_STACK * BLOCK];
	int n_snodes = 0;
	const unsigned n = W.cnt[par];
	if (blockIdx.x == 0 && threadIdx.x == 0) {
		W.cnt[par ^ 1] = 0;  // output queue of this iteration
		W.cnt[2] = 0;        // finished list
		atomicAdd(&W.stat[0], (unsigned long long)n);
	}
	if ((unsigned)(blockIdx.x * blockDim.x) >= n) return;
	constexpr bool linear = LINEAR;
	if (linear) {
		stage_prims(S, snodes);
		__syncthreads();
	} else if (WIDE) {
		stage_nodes4(S, snodes, n_snodes);
	} else {
		stage_nodes(S, snodes, n_snodes);
	}
	const float4 *__restrict__ qa = W.qa[par];
	const float4 *__restrict__ qb = W.qb[par];
	uint32_t err = 0;
	const float inf = __int_as_float(0x7f800000);
	if constexpr (WIDE) {
		// the 4-wide tree: the lanes' walks interleaved, each lane taking its next queued ray at once
		walk_rays4<INTERSECT_SHORT_STACK>(S, snodes, n_snodes, sstack + threadIdx.x, (int64_t)n, err,
			[&](int64_t i, f3 &o, f3 &d, float &tmin, float &tmax) {
				o = ld3(qa[i]), d = ld3(qb[i]), tmin = W.t_min, tmax = inf;
			},
			[&](int64_t i, const Hit &h) { W.hit[i] = make_float4(h.t, __int_as_float(h.leaf), h.u, h.v); });
		if (err) atomicOr(&W.cnt[4], err);
		return;
	}
	// whole warps walk the queue together (the linear scan is warp-cooperative)
	for (unsigned base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
		const unsigned i = base + threadIdx.x;
		const bool active = i < n;
		float4 r0 = make_float4(0.f, 0.f, 0.f, 0.f), r1 = r0;
		if (active) r0 = qa[i], r1 = qb[i];
		Hit h;
		if (linear) {
			h = closest_hit_linear_warp(snodes, S.n_leaves, S.triangle_test, ld3(r0), ld3(r1), W.t_min, inf, active,
				scratch[threadIdx.x >> 5]);
		} else if (active) {
			h = WIDE ? closest_hit4<INTERSECT_SHORT_STACK>(S, snodes, n_snodes, ld3(r0), ld3(r1), W.t_min, inf, err,
						   sstack + threadIdx.x)
					 : closest_hit<INTERSECT_SHORT_STACK>(S, snodes, n_snodes, ld3(r0), ld3(r1), W.t_min, inf, err,
						   sstack + threadIdx.x);
		}
		if (active) W.hit[i] = make_float4(h.t, __int_as_float(h.leaf), h.u, h.v);
	}
	if (err) atomicOr(&W.cnt[4], err);
}

// One bounce of path P at hit h (t, leaf bits, u, v): scatter and, when the
// path ends, the accumulate step and the slot's next camera path.  Returns
// true if P holds a ray to trace (the continued path or the new one).  With
// ACC_IN_REGS the slot's sums are the caller's registers (sm, cm, q), else
// they are read and written in device memory.
template <bool ACC_IN_REGS>
__device__ __forceinline__ bool shade_step(const DevScene &S, const Wave &W, PathState &P, float4 h, uint32_t &err,
	unsigned long long &done, float4 &sm, float4 &cm, float4 &q) {
	bool cont = false;
	const int leaf = __float_as_int(h.y);
	if (leaf < 0) {
		P.L = add(P.L, mulv(P.beta, background(S, P.d)));
	} else {
		const uint64_t key = P.key;
		Surface sf = surface_at(S, leaf, P.o, P.d, h.x, h.z, h.w);
		f3 nd;
		cont = scatter(S, sf, P.d, key, P.depth, W.rr_depth, P.beta, P.L, nd);
		if (cont && P.depth + 1 >= W.max_depth) cont = false;
		if (cont) {
			P.o = sf.p;
			P.d = nd;
			++P.depth;
			return true;
		}
	}
	++done;
	int64_t item = P.item;
	int j = P.j;
	const bool more = ACC_IN_REGS ? accumulate(W, P.L, item, j, err, &W.cnt[3], sm, cm, q)
								  : finish_path(W, P.slot, P.L, item, j, err, &W.cnt[3]);
	if (!more) return false;
	camera_path(W, P.slot, item, j, P);
	return true;
}

// One bounce of every queued path, fused with the accumulate and generate
// steps: a path that continues is appended to the next queue; a path that
// ends adds its radiance to its slot (finish_path) and, if the slot has a
// next sample, that sample's camera ray takes its place in the next queue.
// One warp-aggregated append serves both.
__global__ void __launch_bounds__(BLOCK) k_shade(DevScene S, Wave W, int par) {
	const unsigned n = W.cnt[par];
	const int out = par ^ 1;
	uint32_t err = 0;
	unsigned long long done = 0;
	for (unsigned base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
		unsigned i = base + threadIdx.x;
		bool live = false;
		PathState P;
		if (i < n) {
			P = load_path(W, par, i);
			float4 unused;
			live = shade_step<false>(S, W, P, W.hit[i], err, done, unused, unused, unused);
		}
		unsigned pos = warp_append(&W.cnt[out], live);
		if (live) {
			if (pos < (unsigned)W.P)
				store_path(W, out, pos, P);
			else
				err |= ERR_QUEUE_OVERFLOW;
		}
	}
	// one atomic per warp: every lane of the block reaches this point
	for (int o = 16; o > 0; o >>= 1) done += __shfl_down_sync(0xffffffffu, done, o);
	if (lane_id() == 0 && done) atomicAdd(&W.stat[1], done);
	if (err) atomicOr(&W.cnt[4], err);
}

// One thread per queued path traces it to the end, then the rest of its
// slot's samples and, while work items are left, the next ones, with the same
// device functions and in the same sample order as the wavefront, so the image
// is the same bit for bit.  Two uses: the end of a wavefront render, when
// every item has been taken and few paths are left (it replaces the long tail
// of nearly empty iterations: paths that keep bouncing between glass and
// metal), and the whole render under the megakernel schedule (queue 0 then
// holds one camera path per resident thread).
//
// One instantiation per closest-hit strategy (LINEAR: the staged linear scan of
// a scene with at most LINEAR_MAX primitives, else the BVH: WIDE the 4-wide
// tree, INTER the lanes' walks interleaved (mega.cuh) rather than one walk per
// ray and bounce; the 4-wide tree always interleaves, a binary tree does for
// scenes with quads or triangles, measured faster there and slower on sphere
// fields), each with the occupancy that measured fastest for it.
template <bool LINEAR, bool WIDE = false, bool INTER = WIDE>
__global__ void __launch_bounds__(BLOCK, tail_min_blocks(LINEAR, WIDE, INTER))
	k_tail(DevScene S, Wave W, int par) {
	// linear scenes: the staged primitives and leaf boxes (6 float4 per primitive at most) and
	// one closest-hit scratch per warp; BVH scenes: the top BVH levels
	__shared__ float4 snodes[LINEAR ? 6 * LINEAR_MAX : WIDE ? 8 * TAIL_SMEM_NODES4 : 2 * SMEM_NODES];
	__shared__ WarpHitScratch scratch[LINEAR ? BLOCK / 32 : 1];
	// BVH scenes: the top traversal-stack entries of every thread
	constexpr int SHORT = WIDE ? TAIL_SHORT_STACK_WIDE : TAIL_SHORT_STACK;
	__shared__ int4 sstack[LINEAR ? 1 : SHORT * BLOCK];
	int n_snodes = 0;
	const unsigned n = W.cnt[par];
	if ((unsigned)(blockIdx.x * blockDim.x) >= n) return;
	if (LINEAR) {
		stage_prims(S, snodes);
		__syncthreads();
	} else if (WIDE) {
		stage_nodes4(S, snodes, n_snodes, TAIL_SMEM_NODES4);
	} else {
		stage_nodes(S, snodes, n_snodes);
	}
	uint32_t err = 0;
	unsigned long long done = 0, segments = 0;
	const float inf = __int_as_float(0x7f800000);
	if constexpr (LINEAR) {
		// every lane of a warp stays in the loop while any of its lanes has a path, so the
		// warp-cooperative closest hit always runs with the full warp
		WarpHitScratch &ws = scratch[threadIdx.x >> 5];
		for (unsigned base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
			const unsigned i = base + threadIdx.x;
			bool live = i < n;
			PathState P{};
			float4 sm{}, cm{}, q{};
			if (live) {
				P = load_path(W, par, i);
				sm = W.acc_s[P.slot], cm = W.acc_c[P.slot], q = W.acc_q[P.slot];
				sm.w = cm.w = q.w = 0.f;  // unused lanes: constant, so they hold no registers in the loop
			}
			const int slot = P.slot;
			while (__any_sync(0xffffffffu, live)) {
				Hit hh = closest_hit_linear_warp(snodes, S.n_leaves, S.triangle_test, P.o, P.d, W.t_min, inf, live, ws);
				if (live) {
					++segments;
					live = shade_step<true>(S, W, P, make_float4(hh.t, __int_as_float(hh.leaf), hh.u, hh.v), err, done,
						sm, cm, q);
				}
			}
			if (i < n) W.acc_s[slot] = sm, W.acc_c[slot] = cm, W.acc_q[slot] = q;
		}
	} else if constexpr (WIDE || INTER) {
		PathState P{};
		float4 sm{}, cm{}, q{};
		interleaved_walks<SHORT, WIDE>(S, snodes, n_snodes, sstack + threadIdx.x, W.t_min, blockIdx.x * blockDim.x + threadIdx.x,
			n, gridDim.x * blockDim.x, P, err, segments,
			[&](unsigned i) {
				P = load_path(W, par, i);
				// the slot's sums stay in registers while this thread owns the slot
				sm = W.acc_s[P.slot], cm = W.acc_c[P.slot], q = W.acc_q[P.slot];
				sm.w = cm.w = q.w = 0.f;
			},
			[&](float4 h) { return shade_step<true>(S, W, P, h, err, done, sm, cm, q); },
			[&]() { W.acc_s[P.slot] = sm, W.acc_c[P.slot] = cm, W.acc_q[P.slot] = q; });
	} else {
		for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
			PathState P = load_path(W, par, i);
			const int slot = P.slot;
			// the slot's sums stay in registers while this thread owns the slot
			float4 sm = W.acc_s[slot], cm = W.acc_c[slot], q = W.acc_q[slot];
			sm.w = cm.w = q.w = 0.f;
			bool live = true;
			while (live) {
				Hit hh = closest_hit<SHORT>(S, snodes, n_snodes, P.o, P.d, W.t_min, inf, err, sstack + threadIdx.x);
				++segments;
				live = shade_step<true>(S, W, P, make_float4(hh.t, __int_as_float(hh.leaf), hh.u, hh.v), err, done, sm,
					cm, q);
			}
			W.acc_s[slot] = sm, W.acc_c[slot] = cm, W.acc_q[slot] = q;
		}
	}
	for (int o = 16; o > 0; o >>= 1) {
		done += __shfl_down_sync(0xffffffffu, done, o);
		segments += __shfl_down_sync(0xffffffffu, segments, o);
	}
	if (lane_id() == 0) {
		if (done) atomicAdd(&W.stat[1], done);
		if (segments) atomicAdd(&W.stat[0], segments), atomicAdd(&W.stat[2], segments);
	}
	if (err) atomicOr(&W.cnt[4], err);
}

// mean and variance of the mean per pixel from the per-item sums, in chunk order
__global__ void k_resolve(Wave W, float *__restrict__ rgb, float *__restrict__ var, int clamp) {
	for (int px = blockIdx.x * blockDim.x + threadIdx.x; px < W.npix; px += gridDim.x * blockDim.x) {
		float s[3] = { 0.f, 0.f, 0.f }, c[3] = { 0.f, 0.f, 0.f }, q[3] = { 0.f, 0.f, 0.f };
		for (int ch = 0; ch < W.nchunk; ++ch) {
			int64_t it = (int64_t)ch * W.npix + px;
			const float4 a = W.item_s[it];
			// one-sample items store no square: fl(a a) is the value accumulate computed (fma(L, L, 0))
			const float4 b = W.item_q ? W.item_q[it]
									  : make_float4(__fmul_rn(a.x, a.x), __fmul_rn(a.y, a.y), __fmul_rn(a.z, a.z), 0.f);
			float v[3] = { a.x, a.y, a.z }, w[3] = { b.x, b.y, b.z };
			for (int k = 0; k < 3; ++k) {
				float y = v[k] - c[k];
				float t = s[k] + y;
				c[k] = (t - s[k]) - y;
				s[k] = t;
				q[k] += w[k];
			}
		}
		float n = (float)W.spp;
		for (int k = 0; k < 3; ++k) {
			float m = s[k] / n;
			if (var) {
				float v = W.spp > 1 ? (q[k] - n * m * m) / (n - 1.f) / n : 0.f;
				var[3 * (size_t)px + k] = v > 0.f ? v : 0.f;
			}
			if (clamp) m = fminf(fmaxf(m, 0.f), 1.f);
			rgb[3 * (size_t)px + k] = m;
		}
	}
}

// ---------------------------------------------------------------------------
// host side

namespace {

are_status bad(const std::string &m) {
	set_error(m);
	return ARE_ERR_INVALID_ARGUMENT;
}

// Resident blocks per SM of each kernel, looked up once per (kernel, shared memory, device): the
// occupancy query costs microseconds, and a frame rendered end to end (scene created, rendered,
// destroyed) would otherwise pay it several times.
struct OccKey {
	const void *kernel;
	size_t smem;
	int device;
};
std::mutex g_occ_mu;
std::vector<std::pair<OccKey, int>> g_occ;

int grid_for(const void *kernel, int n_sms, size_t smem = 0) {
	int device = 0;
	cudaGetDevice(&device);
	{
		std::lock_guard<std::mutex> lk(g_occ_mu);
		for (const auto &e : g_occ)
			if (e.first.kernel == kernel && e.first.smem == smem && e.first.device == device) return e.second * n_sms;
	}
	int per_sm = 0;
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, BLOCK, smem) != cudaSuccess) {
		cudaGetLastError();
		per_sm = 0;
	}
	per_sm = std::max(1, per_sm);
	std::lock_guard<std::mutex> lk(g_occ_mu);
	g_occ.push_back({ OccKey{ kernel, smem, device }, per_sm });
	return per_sm * n_sms;
}

template <class T>
T *carve(char *&p, size_t count) {
	T *r = (T *)p;
	p += (count * sizeof(T) + 255) & ~(size_t)255;
	return r;
}

}  // namespace

void camera_frame(const are_camera &c, int w, int h, int flags, CameraFrame &f) {
	// rt.cpp:339-343: forward, right = forward x up, up' = right x forward
	float fw[3] = { c.lookat[0] - c.lookfrom[0], c.lookat[1] - c.lookfrom[1], c.lookat[2] - c.lookfrom[2] };
	auto nrm = [](float *v) {
		float l = 1.0f / std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
		v[0] *= l, v[1] *= l, v[2] *= l;
	};
	nrm(fw);
	float rt[3] = { fw[1] * c.vup[2] - fw[2] * c.vup[1], fw[2] * c.vup[0] - fw[0] * c.vup[2],
		fw[0] * c.vup[1] - fw[1] * c.vup[0] };
	nrm(rt);
	float up[3] = { rt[1] * fw[2] - rt[2] * fw[1], rt[2] * fw[0] - rt[0] * fw[2], rt[0] * fw[1] - rt[1] * fw[0] };
	for (int k = 0; k < 3; ++k) f.pos[k] = c.lookfrom[k], f.fwd[k] = fw[k], f.right[k] = rt[k], f.up[k] = up[k];
	f.aspect = (float)w / (float)h;
	f.scale = std::tan(c.vfov_deg * 0.5f * (float)3.14159265358979323846 / 180.f);
	f.lens = c.aperture > 0.0f;
	f.lens_r = c.aperture * 0.5f;
	f.focus = c.focus_dist;
	f.jitter = !(flags & ARE_FLAG_NO_JITTER);
	f.width = w;
	f.height = h;
}

// the megakernel instantiation for scene S: linear scan, 4-wide tree, or binary tree with interleaved
// or per-ray walks
static const void *tail_fn(bool linear, const DevScene &S) {
	if (linear) return (const void *)k_tail<true>;
	if (S.n_nodes4 > 0) return (const void *)k_tail<false, true>;
	return S.interleave ? (const void *)k_tail<false, false, true> : (const void *)k_tail<false, false, false>;
}

void launch_tail(bool linear, int grid, cudaStream_t s, const DevScene &S, const Wave &W) {
	if (linear)
		k_tail<true><<<grid, BLOCK, 0, s>>>(S, W, 0);
	else if (S.n_nodes4 > 0)
		k_tail<false, true><<<grid, BLOCK, 0, s>>>(S, W, 0);
	else if (S.interleave)
		k_tail<false, false, true><<<grid, BLOCK, 0, s>>>(S, W, 0);
	else
		k_tail<false, false, false><<<grid, BLOCK, 0, s>>>(S, W, 0);
}

int tail_grid(bool linear, const DevScene &S, int n_sms) { return grid_for(tail_fn(linear, S), n_sms); }

void launch_intersect(bool linear, int grid, cudaStream_t s, const DevScene &S, const Wave &W, int par) {
	if (linear)
		k_intersect<true><<<grid, BLOCK, 0, s>>>(S, W, par);
	else if (S.n_nodes4 > 0)
		k_intersect<false, true><<<grid, BLOCK, 0, s>>>(S, W, par);
	else
		k_intersect<false, false><<<grid, BLOCK, 0, s>>>(S, W, par);
}

int intersect_grid(bool linear, const DevScene &S, int n_sms) {
	const void *fn = linear ? (const void *)k_intersect<true>
							: S.n_nodes4 > 0 ? (const void *)k_intersect<false, true> : (const void *)k_intersect<false, false>;
	return grid_for(fn, n_sms);
}

are_status render(are_scene *sc, const are_camera *cam, const are_render_params *prm, float *rgb, float *var,
	are_render_stats *stats) {
	if (!sc || !cam || !prm || !rgb) return bad("null scene, camera, params or output");
	const are_render_params &p = *prm;
	if (p.width <= 0 || p.height <= 0 || p.spp <= 0 || p.max_depth <= 0 || p.max_depth > 255)
		return bad("width, height, spp must be > 0 and max_depth in [1, 255]");
	if ((int64_t)p.width * p.height > (1 << 26)) return bad("image too large (max 2^26 pixels)");
	if (!(cam->vfov_deg > 0.0f && cam->vfov_deg < 180.0f)) return bad("vfov must be in (0, 180)");
	if (!(p.t_min >= 0.0f) || !std::isfinite(p.t_min)) return bad("t_min must be finite and >= 0");
	cudaSetDevice(sc->device);
	if (p.estimator == ARE_EST_LEGACY_RT) return render_legacy(sc, cam, p, rgb, stats);
	if (p.estimator != ARE_EST_PATH) return bad("unknown estimator");

	if (p.schedule < ARE_SCHEDULE_AUTO || p.schedule > ARE_SCHEDULE_MEGAKERNEL) return bad("unknown schedule");
	// measured on GB300, the megakernel is the faster schedule on every workload scene (the path
	// state stays in registers; no queue records go through memory between bounces)
	const bool mega = p.schedule != ARE_SCHEDULE_WAVEFRONT;
	const bool linear = sc->linear;
	const int g_int = mega ? 0 : intersect_grid(linear, sc->dev, sc->n_sms);  // wavefront kernels only
	const int g_sh = mega ? 0 : grid_for((const void *)k_shade, sc->n_sms);
	const int g_tail = tail_grid(linear, sc->dev, sc->n_sms);

	Wave W{};
	W.npix = p.width * p.height;
	W.spp = p.spp;
	int64_t total = (int64_t)W.npix * p.spp;
	// megakernel: one path per resident thread of the persistent launch
	int P = p.pool_size > 0 ? p.pool_size : mega ? g_tail * BLOCK : (1 << 20);
	if (P > (1 << 24)) return bad("pool_size too large (max 2^24)");
	int chunk = p.chunk;
	// wavefront: small work items keep the end-of-frame tail short (a slot finishes its item before
	// going idle), large ones take fewer atomics on the next-item counter.  Megakernel: one sample per
	// item measured fastest on every workload (mesh 967 -> 1201, spheres at 256 spp 1908 -> 2525
	// Msamples/s against 16-sample items); its items cost 16 bytes each, so larger items only when the
	// item sums of one-sample items would pass MEGA_ITEM_BUDGET bytes
	if (chunk <= 0) {
		if (mega && total * 16 <= MEGA_ITEM_BUDGET)
			chunk = 1;
		else if (mega)
			chunk = (int)std::min<int64_t>(p.spp, (total * 32 + MEGA_ITEM_BUDGET - 1) / MEGA_ITEM_BUDGET);
		else
			chunk = (int)std::min<int64_t>(16, std::max<int64_t>(1, total / (16 * (int64_t)P)));
	}
	chunk = std::min(chunk, p.spp);
	W.chunk = chunk;
	W.nchunk = (p.spp + chunk - 1) / chunk;
	W.n_items = (int64_t)W.npix * W.nchunk;
	if (W.n_items >= (int64_t)UINT32_MAX - (int64_t)P) return bad("too many work items; raise chunk");
	P = (int)std::min<int64_t>(P, W.n_items);
	P = (P + 31) & ~31;
	W.P = P;
	W.max_depth = p.max_depth;
	W.rr_depth = p.rr_depth;
	W.t_min = p.t_min;
	W.seed = p.seed;
	camera_frame(*cam, p.width, p.height, p.flags, W.cam);

	// workspace
	size_t need = 0;
	{
		char *z = nullptr;
		for (int q = 0; q < 2; ++q)
			carve<float4>(z, P), carve<float4>(z, P), carve<float4>(z, P), carve<float4>(z, P);
		carve<float4>(z, P);                      // hit
		carve<float4>(z, P), carve<float4>(z, P), carve<float4>(z, P);
		carve<unsigned>(z, 64);
		carve<unsigned long long>(z, 8);
		need = (size_t)z;
	}
	cudaStream_t s = sc->stream;
	if (need > sc->ws_bytes) {
		pool_free(sc, sc->ws);
		sc->ws = nullptr;
		sc->ws_bytes = 0;
		if (are_status st = pool_alloc(sc, need, &sc->ws)) return st;
		sc->ws_bytes = need;
	}
	const bool one_sample_items = W.chunk == 1;  // no per-item sum of squares (see k_resolve)
	size_t item_need = (size_t)W.n_items * (one_sample_items ? 1 : 2) * sizeof(float4) +
		2 * (size_t)W.npix * 3 * sizeof(float);
	if (item_need > sc->items_bytes) {
		pool_free(sc, sc->items);
		sc->items = nullptr;
		sc->items_bytes = 0;
		if (are_status st = pool_alloc(sc, item_need, &sc->items)) return st;
		sc->items_bytes = item_need;
	}
	{
		char *z = (char *)sc->ws;
		for (int q = 0; q < 2; ++q)
			W.qa[q] = carve<float4>(z, P), W.qb[q] = carve<float4>(z, P), W.qc[q] = carve<float4>(z, P),
			W.qd[q] = carve<float4>(z, P);
		W.hit = carve<float4>(z, P);
		W.acc_s = carve<float4>(z, P), W.acc_c = carve<float4>(z, P), W.acc_q = carve<float4>(z, P);
		W.cnt = carve<unsigned>(z, 64);
		W.stat = carve<unsigned long long>(z, 8);
		W.item_s = (float4 *)sc->items;
		W.item_q = one_sample_items ? nullptr : W.item_s + W.n_items;
	}
	float *d_rgb = (float *)(W.item_s + W.n_items * (one_sample_items ? 1 : 2));
	float *d_var = d_rgb + 3 * (size_t)W.npix;
	const bool dev_out = (p.flags & ARE_FLAG_DEVICE_OUTPUT) != 0;

	// timing events: ev0, ev1 around the render, then 4 per graph iteration (created once per scene)
	// the megakernel times two spans (render, launch), the wavefront four per graph iteration
	const size_t n_events = mega ? 4 : 2 + 4 * GRAPH_ITERS;
	while (sc->render_events.size() < n_events) {
		cudaEvent_t e = nullptr;
		cudaEventCreate(&e);
		sc->render_events.push_back(e);
	}
	cudaEvent_t ev0 = sc->render_events[0], ev1 = sc->render_events[1];
	cudaEvent_t *kev = sc->render_events.data() + 2;
	cudaGraph_t graph = nullptr;
	cudaGraphExec_t exec = nullptr;
	are_status st = ARE_OK;
	int64_t iterations = 0;
	int64_t launches[4] = { 0, 0, 0, 0 };
	double kms[4] = { 0.0, 0.0, 0.0, 0.0 };

	// queued paths below which the tail kernel takes over (once every item is taken): its time is set
	// by the longest remaining path, not by how many paths are left, so it can start early
	const unsigned tail_max = (unsigned)std::max<int64_t>(8192, P / 4);
	const DevScene S = sc->dev;

	// the initial counters go up from the scene's pinned block (an asynchronous copy; the host does not
	// touch words 0..7 again before the stream's next synchronisation)
	unsigned *init = sc->host_counters;
	for (int k = 0; k < 8; ++k) init[k] = 0u;
	init[0] = init[3] = (unsigned)std::min<int64_t>(P, W.n_items);
	cudaEventRecord(ev0, s);
	st = cuda_status(cudaMemcpyAsync(W.cnt, init, 8 * sizeof(unsigned), cudaMemcpyHostToDevice, s),
		"cudaMemcpyAsync(counters)");
	if (!st) st = cuda_status(cudaMemsetAsync(W.stat, 0, 8 * sizeof(unsigned long long), s), "cudaMemsetAsync(stats)");
	if (!st) {
		k_init<<<grid_for((const void *)k_init, sc->n_sms), BLOCK, 0, s>>>(W, (int)init[0]);
		++launches[ARE_KERNEL_OTHER];
		st = cuda_status(cudaGetLastError(), "k_init launch");
	}
	if (!st && mega) {
		// the whole render in one persistent launch (queue 0 holds one camera path per thread)
		cudaEventRecord(kev[0], s);
		launch_tail(linear, g_tail, s, S, W);
		cudaEventRecord(kev[1], s);
		++launches[ARE_KERNEL_OTHER];
		st = cuda_status(cudaGetLastError(), "k_tail launch");
		// no synchronisation here: the resolve and the read-back follow in stream order, and the
		// launch's time is read from its events after the render's one synchronisation
	}
	// capture GRAPH_ITERS iterations, each bracketed by timing events
	if (!st && !mega) st = cuda_status(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
	if (!st && !mega) {
		for (int it = 0; it < GRAPH_ITERS; ++it) {
			int par = it & 1;
			// external event nodes: the events are recorded each time the graph runs
			cudaEventRecordWithFlags(kev[4 * it + 0], s, cudaEventRecordExternal);
			launch_intersect(linear, g_int, s, S, W, par);
			cudaEventRecordWithFlags(kev[4 * it + 1], s, cudaEventRecordExternal);
			k_shade<<<g_sh, BLOCK, 0, s>>>(S, W, par);
			cudaEventRecordWithFlags(kev[4 * it + 2], s, cudaEventRecordExternal);
		}
		st = cuda_status(cudaStreamEndCapture(s, &graph), "cudaStreamEndCapture");
	}
	if (!st && !mega && sc->render_exec) {
		// same kernels and events as the cached graph: update its parameters in place
		cudaGraphExecUpdateResultInfo info;
		if (cudaGraphExecUpdate(sc->render_exec, graph, &info) == cudaSuccess) {
			exec = sc->render_exec;
		} else {
			cudaGetLastError();
			cudaGraphExecDestroy(sc->render_exec);
			sc->render_exec = nullptr;
		}
	}
	if (!st && !mega && !exec) {
		st = cuda_status(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate");
		if (!st) sc->render_exec = exec;
	}
	// run until no ray is queued; counters are read back one launch behind
	const int64_t max_launches = (int64_t)(W.n_items / std::max(1, P) + 2) * (int64_t)p.max_depth * W.chunk + 16;
	int64_t g = 0;
	while (!st && !mega) {
		st = cuda_status(cudaGraphLaunch(exec, s), "cudaGraphLaunch");
		if (st) break;
		cudaMemcpyAsync(sc->host_counters, W.cnt, 8 * sizeof(unsigned), cudaMemcpyDeviceToHost, s);
		st = cuda_status(cudaStreamSynchronize(s), "render iteration");
		if (st) break;
		++g;
		iterations += GRAPH_ITERS;
		for (int it = 0; it < GRAPH_ITERS; ++it) {
			for (int k = 0; k < 2; ++k) {  // intersect; shade (with accumulate and generate)
				float ms = 0.f;
				if (cudaEventElapsedTime(&ms, kev[4 * it + k], kev[4 * it + k + 1]) == cudaSuccess) kms[k] += ms;
				++launches[k];
			}
		}
		if (sc->host_counters[0] == 0) break;  // next iteration's input queue is empty
		if (sc->host_counters[3] >= W.n_items && sc->host_counters[0] <= tail_max) {
			// every work item is taken and few paths are left: finish them in one launch
			cudaEventRecord(kev[0], s);
			launch_tail(linear, g_tail, s, S, W);
			cudaEventRecord(kev[1], s);
			st = cuda_status(cudaGetLastError(), "k_tail launch");
			if (!st) st = cuda_status(cudaStreamSynchronize(s), "render tail");
			float ms = 0.f;
			if (!st && cudaEventElapsedTime(&ms, kev[0], kev[1]) == cudaSuccess) kms[ARE_KERNEL_OTHER] += ms;
			++launches[ARE_KERNEL_OTHER];
			break;
		}
		if (g > max_launches) {
			set_error("render did not converge");
			st = ARE_ERR_INTERNAL;
		}
	}
	cudaGetLastError();
	if (!st) {
		k_resolve<<<std::max(1, std::min(4096, (W.npix + BLOCK - 1) / BLOCK)), BLOCK, 0, s>>>(
			W, dev_out ? rgb : d_rgb, var ? (dev_out ? var : d_var) : nullptr, (p.flags & ARE_FLAG_CLAMP_OUTPUT) != 0);
		++launches[ARE_KERNEL_OTHER];
		st = cuda_status(cudaGetLastError(), "k_resolve launch");
	}
	cudaEventRecord(ev1, s);
	unsigned long long hstat[3] = { 0, 0, 0 };
	unsigned herr = 0;
	if (!st) {
		// statistics and the error word come back through the pinned block (words 16..23 and 24)
		unsigned long long *pstat = (unsigned long long *)(sc->host_counters + 16);
		cudaMemcpyAsync(pstat, W.stat, sizeof hstat, cudaMemcpyDeviceToHost, s);
		cudaMemcpyAsync(sc->host_counters + 24, W.cnt + 4, sizeof herr, cudaMemcpyDeviceToHost, s);
		if (!dev_out) {
			cudaMemcpyAsync(rgb, d_rgb, 3 * sizeof(float) * W.npix, cudaMemcpyDeviceToHost, s);
			if (var) cudaMemcpyAsync(var, d_var, 3 * sizeof(float) * W.npix, cudaMemcpyDeviceToHost, s);
		}
		st = cuda_status(cudaStreamSynchronize(s), "render");
		if (!st) {
			for (int k = 0; k < 3; ++k) hstat[k] = pstat[k];
			herr = sc->host_counters[24];
		}
	}
	if (st) cudaStreamSynchronize(s);  // nothing of this render (the counter upload) is left in flight
	if (mega && !st) {
		float ms = 0.f;
		if (cudaEventElapsedTime(&ms, kev[0], kev[1]) == cudaSuccess) kms[ARE_KERNEL_OTHER] += ms;
	}
	float total_ms = 0.f;
	cudaEventElapsedTime(&total_ms, ev0, ev1);
	if (graph) cudaGraphDestroy(graph);  // the instantiated graph stays with the scene
	if (!st && herr) {
		set_error("device error word " + std::to_string(herr));
		st = ARE_ERR_INTERNAL;
	}
	if (stats) {
		stats->samples = (int64_t)hstat[1];
		stats->segments = (int64_t)hstat[0];
		stats->iterations = iterations;
		stats->device_ms = total_ms;
		for (int k = 0; k < 4; ++k) stats->kernel_ms[k] = kms[k], stats->kernel_launches[k] = launches[k];
		stats->error_word = (int32_t)herr;
		stats->aux[0] = (double)hstat[2];  // segments traced by the tail kernel (kernel_ms[ARE_KERNEL_OTHER])
	}
	return st;
}

are_status intersect(are_scene *sc, const float *rays, int64_t n, float *hits, int32_t device_ptrs, float *ms) {
	if (!sc) return bad("null scene");
	if (n < 0) return bad("negative ray count");
	if (n == 0) {
		if (ms) *ms = 0.f;
		return ARE_OK;
	}
	if (!rays || !hits) return bad("null rays or hits");
	cudaSetDevice(sc->device);
	cudaStream_t s = sc->stream;
	const float4 *d_rays = (const float4 *)rays;
	float4 *d_hits = (float4 *)hits;
	// the error word (and, for host pointers, the rays and hits) in one block of the device's
	// stream-ordered pool on the scene's stream; the timing events are the scene's own
	void *tmp = nullptr;
	const size_t io_bytes = device_ptrs ? 0 : (size_t)n * 48;
	are_status st = pool_alloc(sc, 256 + io_bytes, &tmp);
	if (st) return st;
	unsigned *err_word = (unsigned *)tmp;
	if (!device_ptrs) {
		d_rays = (const float4 *)((char *)tmp + 256);
		d_hits = (float4 *)((char *)tmp + 256 + (size_t)n * 32);
		st = cuda_status(cudaMemcpyAsync((void *)d_rays, rays, (size_t)n * 32, cudaMemcpyHostToDevice, s), "H2D rays");
	}
	if (!st) st = cuda_status(cudaMemsetAsync(err_word, 0, sizeof(unsigned), s), "memset");
	while (sc->render_events.size() < 2) {
		cudaEvent_t e = nullptr;
		cudaEventCreate(&e);
		sc->render_events.push_back(e);
	}
	cudaEvent_t e0 = sc->render_events[0], e1 = sc->render_events[1];
	if (!st) {
		const bool linear = sc->linear, walks = !linear && sc->dev.n_nodes4 > 0;
		const void *fn = linear ? (const void *)k_intersect_batch<true>
						 : walks ? (const void *)k_intersect_batch<false, true>
								 : (const void *)k_intersect_batch<false>;
		int grid = grid_for(fn, sc->n_sms);
		grid = (int)std::min<int64_t>(grid, (n + BLOCK - 1) / BLOCK);
		cudaEventRecord(e0, s);
		if (linear)
			k_intersect_batch<true><<<grid, BLOCK, 0, s>>>(sc->dev, d_rays, n, d_hits, err_word);
		else if (walks)
			k_intersect_batch<false, true><<<grid, BLOCK, 0, s>>>(sc->dev, d_rays, n, d_hits, err_word);
		else
			k_intersect_batch<false><<<grid, BLOCK, 0, s>>>(sc->dev, d_rays, n, d_hits, err_word);
		cudaEventRecord(e1, s);
		st = cuda_status(cudaGetLastError(), "k_intersect_batch launch");
	}
	unsigned herr = 0;
	if (!st) {
		if (!device_ptrs)
			st = cuda_status(cudaMemcpyAsync(hits, d_hits, (size_t)n * 16, cudaMemcpyDeviceToHost, s), "D2H hits");
		cudaMemcpyAsync(sc->host_counters + 24, err_word, sizeof herr, cudaMemcpyDeviceToHost, s);
		if (!st) st = cuda_status(cudaStreamSynchronize(s), "intersect");
		if (!st) herr = sc->host_counters[24];
	}
	if (st) cudaStreamSynchronize(s);
	if (ms) {
		float t = 0.f;
		if (!st) cudaEventElapsedTime(&t, e0, e1);
		*ms = t;
	}
	pool_free(sc, tmp);
	if (!st && herr) {
		set_error("device error word " + std::to_string(herr));
		st = ARE_ERR_INTERNAL;
	}
	return st;
}

}  // namespace are_core
