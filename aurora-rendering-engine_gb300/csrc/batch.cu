// batch.cu — many scenes of uneven size in one persistent kernel launch.
//
// The work of all scenes is one flat list of items (scene, pixel, chunk of
// samples), scene after scene.  Every warp of a persistent grid (one wave of
// resident blocks) takes `fetch` x 32 items per atomic on one shared counter
// and each lane traces its item's samples to the end (the path estimator of
// the wavefront core: same camera, BVH queries, scatter and random numbers),
// then adds the item's sums to its pixel.  The last item of a scene stamps
// the scene's completion time (%globaltimer).  The launch, its clears and the
// per-scene resolves are one CUDA graph.  Nothing waits on other blocks:
// the only shared state is atomics.
//
// are_batch_autotune times the launch on a calibration run for each BVH
// leaf size x block size x items-per-fetch and returns the fastest.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <string>
#include <vector>

#include "scene.h"
#include "shade.cuh"
#include "traverse.cuh"
#include "wave.cuh"

namespace are_core {

namespace {

struct BatchScene {
	DevScene S;
	CameraFrame cam;
	int32_t npix, spp, chunk, max_depth, rr_depth;
	float t_min;
	uint64_t seed;
	unsigned long long item_begin, n_items;
	float4 *acc;  // per pixel: (sum, 0), (sum of squares, 0)
};

struct BatchCtl {
	unsigned long long *next;   // next unclaimed item
	unsigned long long total;
	unsigned *left;             // items not yet finished, per scene
	unsigned long long *done;   // per scene completion time (ns, %globaltimer)
	unsigned long long *start;  // earliest block start (ns)
	unsigned long long *segments;
	unsigned *err;
};

__device__ __forceinline__ unsigned long long gtimer() {
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

// ANY_WIDE: some scene of the batch has a 4-wide tree (each query then picks its scene's tree);
// otherwise every query walks the binary tree
template <bool ANY_WIDE>
__global__ void k_batch(const BatchScene *__restrict__ T, int n_scenes, BatchCtl C, int fetch) {
	if (threadIdx.x == 0) atomicMin(C.start, gtimer());
	const unsigned lane = threadIdx.x & 31u;
	uint32_t err = 0;
	unsigned long long segs = 0;
	const float inf = __int_as_float(0x7f800000);
	while (true) {
		unsigned long long base = 0;
		if (lane == 0) base = atomicAdd(C.next, 32ull * (unsigned long long)fetch);
		base = __shfl_sync(0xffffffffu, base, 0);
		if (base >= C.total) break;
		for (int k = 0; k < fetch; ++k) {
			unsigned long long item = base + (unsigned long long)k * 32ull + lane;
			if (item >= C.total) break;
			int lo = 0, hi = n_scenes - 1;
			while (lo < hi) {
				int mid = (lo + hi + 1) >> 1;
				if (T[mid].item_begin <= item)
					lo = mid;
				else
					hi = mid - 1;
			}
			const BatchScene &B = T[lo];
			const unsigned long long local = item - B.item_begin;
			const int npix = B.npix;
			const int pixel = (int)(local % (unsigned long long)npix);
			const int s0 = (int)(local / (unsigned long long)npix) * B.chunk;
			const int s1 = min(s0 + B.chunk, B.spp);
			f3 sum{ 0.f, 0.f, 0.f }, sq{ 0.f, 0.f, 0.f };
			for (int smp = s0; smp < s1; ++smp) {
				uint64_t key = path_key(B.seed, (uint32_t)pixel, (uint32_t)smp);
				f3 o, d;
				camera_ray(B.cam, pixel % B.cam.width, pixel / B.cam.width, key, o, d);
				f3 beta{ 1.f, 1.f, 1.f }, L{ 0.f, 0.f, 0.f };
				for (int depth = 0; depth < B.max_depth; ++depth) {
					++segs;
					Hit h = ANY_WIDE ? closest_hit_any(B.S, nullptr, 0, o, d, B.t_min, inf, err)
									 : closest_hit(B.S, nullptr, 0, o, d, B.t_min, inf, err);
					if (h.leaf < 0) {
						L = add(L, mulv(beta, background(B.S, d)));
						break;
					}
					Surface sf = surface_at(B.S, h.leaf, o, d, h.t, h.u, h.v);
					f3 nd;
					if (!scatter(B.S, sf, d, key, depth, B.rr_depth, beta, L, nd)) break;
					o = sf.p;
					d = nd;
				}
				if (!(isfinite(L.x) && isfinite(L.y) && isfinite(L.z))) {
					err |= ERR_NONFINITE;
					L = f3{ 0.f, 0.f, 0.f };
				}
				sum = add(sum, L);
				sq = add(sq, mulv(L, L));
			}
			float *a = reinterpret_cast<float *>(B.acc + 2 * (size_t)pixel);
			atomicAdd(a + 0, sum.x), atomicAdd(a + 1, sum.y), atomicAdd(a + 2, sum.z);
			atomicAdd(a + 4, sq.x), atomicAdd(a + 5, sq.y), atomicAdd(a + 6, sq.z);
			__threadfence();
			if (atomicSub(&C.left[lo], 1u) == 1u) C.done[lo] = gtimer();
		}
	}
	for (int o = 16; o > 0; o >>= 1) segs += __shfl_down_sync(0xffffffffu, segs, o);
	if (lane == 0) atomicAdd(C.segments, segs);
	if (err) atomicOr(C.err, err);
}

__global__ void k_batch_init(const BatchScene *__restrict__ T, int n_scenes, BatchCtl C) {
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i == 0) {
		*C.next = 0ull;
		*C.start = ~0ull;
		*C.segments = 0ull;
		*C.err = 0u;
	}
	if (i < n_scenes) {
		C.left[i] = (unsigned)T[i].n_items;
		C.done[i] = 0ull;
	}
}

__global__ void k_batch_resolve(const float4 *__restrict__ acc, int npix, int spp, float *__restrict__ rgb,
	float *__restrict__ var) {
	for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
		float4 s = acc[2 * (size_t)p], q = acc[2 * (size_t)p + 1];
		float n = (float)spp;
		float sv[3] = { s.x, s.y, s.z }, qv[3] = { q.x, q.y, q.z };
		for (int k = 0; k < 3; ++k) {
			float m = sv[k] / n;
			rgb[3 * (size_t)p + k] = m;
			if (var) {
				float v = spp > 1 ? (qv[k] - n * m * m) / (n - 1.f) / n : 0.f;
				var[3 * (size_t)p + k] = v > 0.f ? v : 0.f;
			}
		}
	}
}

are_status bad(const std::string &m) {
	set_error(m);
	return ARE_ERR_INVALID_ARGUMENT;
}

}  // namespace

// Renders n scenes in one persistent launch.  rgb_out[i] (host, width*height*3)
// may be null to skip the copy; scene_ms[i] gets each scene's completion time
// from the launch's start; total_ms the launch + resolves (CUDA events).
are_status render_batch(are_scene *const *scenes, const are_camera *cams, const are_render_params *params, int n,
	const are_batch_options *opt, float *const *rgb_out, double *scene_ms, are_render_stats *stats) {
	if (!scenes || !cams || !params || n <= 0 || n > 4096) return bad("need 1..4096 scenes with cameras and params");
	int block = opt && opt->block_size > 0 ? opt->block_size : 256;
	int fetch = opt && opt->fetch > 0 ? opt->fetch : 4;
	if (block % 32 || block < 32 || block > 1024) return bad("block_size must be a multiple of 32 in [32, 1024]");
	if (fetch > 1024) return bad("fetch must be in [1, 1024]");
	int device = -1;
	std::vector<BatchScene> table((size_t)n);
	unsigned long long total = 0;
	size_t acc_bytes = 0, out_bytes = 0;
	for (int i = 0; i < n; ++i) {
		const are_render_params &p = params[i];
		if (!scenes[i]) return bad("null scene " + std::to_string(i));
		if (p.width <= 0 || p.height <= 0 || p.spp <= 0 || p.max_depth <= 0 || p.max_depth > 255 || !(p.t_min >= 0.f))
			return bad("bad render params for scene " + std::to_string(i));
		if (!(cams[i].vfov_deg > 0.0f && cams[i].vfov_deg < 180.0f)) return bad("bad camera for scene " + std::to_string(i));
		if (device < 0) device = scenes[i]->device;
		if (scenes[i]->device != device) return bad("all scenes of a batch must live on one device");
		BatchScene &B = table[i];
		B.S = scenes[i]->dev;
		camera_frame(cams[i], p.width, p.height, p.flags, B.cam);
		B.npix = p.width * p.height;
		B.spp = p.spp;
		B.chunk = p.chunk > 0 ? std::min(p.chunk, p.spp) : std::min(p.spp, 16);
		B.max_depth = p.max_depth;
		B.rr_depth = p.rr_depth;
		B.t_min = p.t_min;
		B.seed = p.seed;
		B.item_begin = total;
		B.n_items = (unsigned long long)B.npix * (unsigned long long)((p.spp + B.chunk - 1) / B.chunk);
		if (B.n_items >= 0xffffffffull) return bad("too many work items in scene " + std::to_string(i));
		total += B.n_items;
		acc_bytes += ((size_t)B.npix * 32 + 255) & ~(size_t)255;
		out_bytes += ((size_t)B.npix * 12 + 255) & ~(size_t)255;
	}
	cudaSetDevice(device);
	int n_sms = scenes[0]->n_sms;
	size_t ctl_bytes = 4096 + (size_t)n * 16;
	// the accumulators, images and control block come from the device's stream-ordered pool on the
	// first scene's stream (the stream the batch runs on), and go back to it when the call ends
	void *mem = nullptr;
	are_status st = pool_alloc(scenes[0], acc_bytes + out_bytes + ctl_bytes + sizeof(BatchScene) * n + 256, &mem);
	if (st) return st;
	struct Free {
		are_scene *sc;
		void *p;
		~Free() { pool_free(sc, p); }
	} release{ scenes[0], mem };
	char *z = (char *)mem;
	std::vector<float *> d_out((size_t)n);
	for (int i = 0; i < n; ++i) {
		table[i].acc = (float4 *)z;
		z += ((size_t)table[i].npix * 32 + 255) & ~(size_t)255;
	}
	for (int i = 0; i < n; ++i) {
		d_out[i] = (float *)z;
		z += ((size_t)table[i].npix * 12 + 255) & ~(size_t)255;
	}
	BatchCtl C{};
	C.next = (unsigned long long *)z;
	C.start = C.next + 1;
	C.segments = C.next + 2;
	C.err = (unsigned *)(C.next + 3);
	C.done = C.next + 8;
	C.left = (unsigned *)(C.done + n);
	C.total = total;
	char *ctl_base = z;
	z += ctl_bytes;
	BatchScene *d_table = (BatchScene *)(((uintptr_t)z + 255) & ~(uintptr_t)255);

	cudaStream_t s = scenes[0]->stream;
	cudaGetLastError();
	// every scene's upload (asynchronous, on its own stream) has landed before the launch reads it
	for (int i = 1; i < n && !st; ++i)
		if (scenes[i]->stream != s) st = cuda_status(cudaStreamSynchronize(scenes[i]->stream), "scene upload");
	if (!st) st = cuda_status(cudaMemcpyAsync(d_table, table.data(), sizeof(BatchScene) * n, cudaMemcpyHostToDevice, s), "table");
	if (!st) st = cuda_status(cudaStreamSynchronize(s), "table");
	cudaGraph_t graph = nullptr;
	cudaGraphExec_t exec = nullptr;
	if (!st) st = cuda_status(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "capture");
	bool any_wide = false;
	for (int i = 0; i < n; ++i) any_wide = any_wide || table[i].S.n_nodes4 > 0;
	const void *batch_fn = any_wide ? (const void *)k_batch<true> : (const void *)k_batch<false>;
	int per_sm = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_fn, block, 0);
	const int grid = std::max(1, per_sm) * n_sms;
	if (!st) {
		k_batch_init<<<(n + 255) / 256, 256, 0, s>>>(d_table, n, C);
		cudaMemsetAsync(mem, 0, acc_bytes, s);
		if (any_wide)
			k_batch<true><<<grid, block, 0, s>>>(d_table, n, C, fetch);
		else
			k_batch<false><<<grid, block, 0, s>>>(d_table, n, C, fetch);
		for (int i = 0; i < n; ++i)
			k_batch_resolve<<<std::max(1, std::min(1024, (table[i].npix + 255) / 256)), 256, 0, s>>>(table[i].acc,
				table[i].npix, table[i].spp, d_out[i], nullptr);
		st = cuda_status(cudaStreamEndCapture(s, &graph), "capture end");
	}
	if (!st) st = cuda_status(cudaGraphInstantiate(&exec, graph, 0), "instantiate");
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	if (!st) {
		cudaEventRecord(e0, s);
		st = cuda_status(cudaGraphLaunch(exec, s), "graph launch");
		cudaEventRecord(e1, s);
	}
	std::vector<unsigned long long> ctl(8 + (size_t)n);
	if (!st) {
		cudaMemcpyAsync(ctl.data(), ctl_base, ctl.size() * 8, cudaMemcpyDeviceToHost, s);
		for (int i = 0; i < n && rgb_out; ++i)
			if (rgb_out[i]) cudaMemcpyAsync(rgb_out[i], d_out[i], (size_t)table[i].npix * 12, cudaMemcpyDeviceToHost, s);
		st = cuda_status(cudaStreamSynchronize(s), "batch render");
	}
	float ms = 0.f;
	if (!st) cudaEventElapsedTime(&ms, e0, e1);
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	if (exec) cudaGraphExecDestroy(exec);
	if (graph) cudaGraphDestroy(graph);
	if (st) return st;
	unsigned err = (unsigned)(ctl[3] & 0xffffffffu);
	if (scene_ms)
		for (int i = 0; i < n; ++i) scene_ms[i] = ctl[8 + i] >= ctl[1] ? (double)(ctl[8 + i] - ctl[1]) * 1e-6 : -1.0;
	if (stats) {
		*stats = are_render_stats{};
		int64_t smp = 0;
		for (int i = 0; i < n; ++i) smp += (int64_t)table[i].npix * table[i].spp;
		stats->samples = smp;
		stats->segments = (int64_t)ctl[2];
		stats->iterations = 1;
		stats->device_ms = ms;
		stats->kernel_ms[ARE_KERNEL_OTHER] = ms;
		stats->kernel_launches[ARE_KERNEL_OTHER] = 1 + n;
		stats->error_word = (int32_t)err;
	}
	if (err) {
		set_error("device error word " + std::to_string(err));
		return ARE_ERR_INTERNAL;
	}
	return ARE_OK;
}

are_status batch_autotune(const are_scene_desc *const *descs, const are_camera *cams, const are_render_params *params,
	int n, int calib_spp, are_batch_options *best, double *best_ms) {
	if (!descs || !cams || !params || !best || n <= 0) return bad("bad autotune arguments");
	static const int leafs[] = { 2, 4, 8 };
	static const int blocks[] = { 128, 256, 512 };
	static const int fetches[] = { 1, 4, 16 };
	double best_t = 1e300;
	std::vector<are_render_params> cal(params, params + n);
	for (auto &p : cal) p.spp = std::max(1, std::min(p.spp, calib_spp));
	// stage 1: leaf size x block x fetch on the binary tree; stage 2: the node layout (binary or
	// 4-wide tree) x leaf size at the best block and fetch of stage 1
	auto calibrate = [&](int width, int leaf, const int *bs, int nb, const int *fs, int nf) -> are_status {
		std::vector<are_scene *> sc((size_t)n, nullptr);
		are_status st = ARE_OK;
		for (int i = 0; i < n && !st; ++i) {
			are_scene_desc d = *descs[i];
			d.bvh_leaf_size = leaf;
			d.bvh_width = width;
			if (width == 4) d.bvh_build = ARE_BVH_HOST_SAH;  // the 4-wide collapse is made by the host build
			st = scene_create(&d, &sc[i]);
		}
		for (int bi = 0; bi < nb && !st; ++bi)
			for (int fi = 0; fi < nf && !st; ++fi) {
				are_batch_options o{ bs[bi], fs[fi], leaf, width };
				are_render_stats rs{};
				// one warm-up, then the timed calibration launch
				st = render_batch(sc.data(), cams, cal.data(), n, &o, nullptr, nullptr, &rs);
				if (!st) st = render_batch(sc.data(), cams, cal.data(), n, &o, nullptr, nullptr, &rs);
				if (!st && rs.device_ms < best_t) {
					best_t = rs.device_ms;
					*best = o;
				}
			}
		for (are_scene *p : sc) delete p;
		return st;
	};
	for (int leaf : leafs)
		if (are_status st = calibrate(2, leaf, blocks, 3, fetches, 3)) return st;
	const int b1 = best->block_size, f1 = best->fetch;
	for (int leaf : leafs)
		if (are_status st = calibrate(4, leaf, &b1, 1, &f1, 1)) return st;
	if (best_ms) *best_ms = best_t;
	return ARE_OK;
}

}  // namespace are_core
