// path.cuh — per-path pieces shared by the renderers (render.cu: megakernel
// and wavefront; guided.cu): warp-aggregated appends, work-item coordinates,
// the 64-byte queue record of a path, camera paths and the accumulate step.
#pragma once

#include "shade.cuh"
#include "wave.cuh"

namespace are_core {

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Warp-aggregated append: every lane of the (converged) warp calls this.
__device__ __forceinline__ unsigned warp_append(unsigned *counter, bool pred) {
	unsigned m = __ballot_sync(0xffffffffu, pred);
	unsigned base = 0;
	if (m) {
		if (lane_id() == (unsigned)(__ffs(m) - 1)) base = atomicAdd(counter, (unsigned)__popc(m));
		base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
	}
	return base + (unsigned)__popc(m & ((1u << lane_id()) - 1u));
}

__device__ __forceinline__ void item_coords(const Wave &W, int64_t item, int j, int &pixel, int &sample) {
	const uint32_t it = (uint32_t)item, np = (uint32_t)W.npix;  // n_items < 2^32 (checked on the host)
	const uint32_t chunk = it / np;
	pixel = (int)(it - chunk * np);
	sample = (int)chunk * W.chunk + j;
}

// queue record of a fresh camera path for (item, j) in `slot`
__device__ __forceinline__ void put_camera_ray(const Wave &W, int q, unsigned pos, int slot, int64_t item, int j) {
	int pixel, sample;
	item_coords(W, item, j, pixel, sample);
	uint64_t key = path_key(W.seed, (uint32_t)pixel, (uint32_t)sample);
	f3 o, d;
	camera_ray(W.cam, pixel % W.cam.width, pixel / W.cam.width, key, o, d);
	W.qa[q][pos] = make_float4(o.x, o.y, o.z, __int_as_float(slot));
	W.qb[q][pos] = make_float4(d.x, d.y, d.z, __int_as_float(j << 8));
	W.qc[q][pos] = make_float4(1.f, 1.f, 1.f, __int_as_float((int)item));
	W.qd[q][pos] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Kahan accumulation of a finished path's radiance L into a slot's sums (sm,
// compensation cm, sum of squares q), in sample order; when the slot's work
// item is complete its sums are published and the slot takes the next item
// from *next_item.  Returns whether the slot has a next sample (item, j).
__device__ __forceinline__ bool accumulate(const Wave &W, f3 L, int64_t &item, int &j, uint32_t &err,
	unsigned *next_item, float4 &sm, float4 &cm, float4 &q) {
	if (!(isfinite(L.x) && isfinite(L.y) && isfinite(L.z))) {
		err |= ERR_NONFINITE;
		L = f3{ 0.f, 0.f, 0.f };
	}
	if (W.chunk == 1) {
		// one-sample items: the Kahan sum of one sample is the sample (sm = L, cm = 0, q = fl(L L)),
		// published as is, without the bookkeeping
		W.item_s[item] = make_float4(L.x, L.y, L.z, 0.f);
		if (W.item_q) W.item_q[item] = make_float4(L.x * L.x, L.y * L.y, L.z * L.z, 0.f);
		item = (int64_t)atomicAdd(next_item, 1u);
		j = 0;
		return item < W.n_items;
	}
	float ys[3] = { L.x - cm.x, L.y - cm.y, L.z - cm.z };
	float ts[3] = { sm.x + ys[0], sm.y + ys[1], sm.z + ys[2] };
	cm = make_float4((ts[0] - sm.x) - ys[0], (ts[1] - sm.y) - ys[1], (ts[2] - sm.z) - ys[2], 0.f);
	sm = make_float4(ts[0], ts[1], ts[2], 0.f);
	q = make_float4(q.x + L.x * L.x, q.y + L.y * L.y, q.z + L.z * L.z, 0.f);
	++j;
	int chunk_len = min(W.chunk, W.spp - (int)((uint32_t)item / (uint32_t)W.npix) * W.chunk);
	if (j >= chunk_len) {
		// item complete: publish its sums, take the next item
		W.item_s[item] = make_float4(sm.x - cm.x, sm.y - cm.y, sm.z - cm.z, 0.f);
		if (W.item_q) W.item_q[item] = q;  // one-sample items: q is fl(L L), which resolve recomputes
		sm = cm = q = make_float4(0.f, 0.f, 0.f, 0.f);
		item = (int64_t)atomicAdd(next_item, 1u);
		j = 0;
	}
	return item < W.n_items;
}

// accumulate() on the slot's sums in device memory
__device__ __forceinline__ bool finish_path(const Wave &W, int slot, f3 L, int64_t &item, int &j, uint32_t &err,
	unsigned *next_item) {
	float4 sm = W.acc_s[slot], cm = W.acc_c[slot], q = W.acc_q[slot];
	const bool more = accumulate(W, L, item, j, err, next_item, sm, cm, q);
	W.acc_s[slot] = sm;
	W.acc_c[slot] = cm;
	W.acc_q[slot] = q;
	return more;
}

// A path between bounces: its ray and the state that travels with it.
struct PathState {
	f3 o, d, beta, L;
	int slot, depth, j;
	uint32_t item;  // work item (fewer than 2^32, checked on the host)
	uint64_t key;   // the sample's random-number key, path_key(seed, pixel, sample)
};

__device__ __forceinline__ PathState load_path(const Wave &W, int q, unsigned i) {
	const float4 ra = W.qa[q][i], rb = W.qb[q][i], rc = W.qc[q][i], rd = W.qd[q][i];
	PathState P;
	P.o = ld3(ra), P.d = ld3(rb), P.beta = ld3(rc), P.L = ld3(rd);
	P.slot = __float_as_int(ra.w);
	const int meta = __float_as_int(rb.w);
	P.depth = meta & 0xff, P.j = meta >> 8;
	P.item = (uint32_t)__float_as_int(rc.w);
	int pixel, sample;
	item_coords(W, P.item, P.j, pixel, sample);
	P.key = path_key(W.seed, (uint32_t)pixel, (uint32_t)sample);
	return P;
}

__device__ __forceinline__ void store_path(const Wave &W, int q, unsigned pos, const PathState &P) {
	W.qa[q][pos] = make_float4(P.o.x, P.o.y, P.o.z, __int_as_float(P.slot));
	W.qb[q][pos] = make_float4(P.d.x, P.d.y, P.d.z, __int_as_float(P.depth | (P.j << 8)));
	W.qc[q][pos] = make_float4(P.beta.x, P.beta.y, P.beta.z, __int_as_float((int)P.item));
	W.qd[q][pos] = make_float4(P.L.x, P.L.y, P.L.z, 0.f);
}

// The first ray of sample j of work item `item`, as put_camera_ray writes it.
__device__ __forceinline__ void camera_path(const Wave &W, int slot, int64_t item, int j, PathState &P) {
	int pixel, sample;
	item_coords(W, item, j, pixel, sample);
	uint64_t key = path_key(W.seed, (uint32_t)pixel, (uint32_t)sample);
	camera_ray(W.cam, pixel % W.cam.width, pixel / W.cam.width, key, P.o, P.d);
	P.beta = f3{ 1.f, 1.f, 1.f };
	P.L = f3{ 0.f, 0.f, 0.f };
	P.slot = slot, P.depth = 0, P.j = j, P.item = (uint32_t)item;
	P.key = key;
}

}  // namespace are_core
