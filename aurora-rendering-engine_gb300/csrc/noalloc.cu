// noalloc.cu — are_render_noalloc: the wavefront render with its scratch in
// a fixed, statically sized device array instead of allocated memory.
//
// Who needs it: code that renders where it may not allocate device memory —
// a plugin host that hands a plugin a fixed device-memory budget and forbids
// it from allocating on its own, or an application that owns all device
// memory through its own allocator and must not meet the device-wide
// synchronisation of a cudaMalloc/cudaFree in the middle of a frame.  Such a
// caller creates the scene beforehand (scene creation does allocate) and then
// renders with this entry point, which calls no cudaMalloc, no cudaFree, no
// allocating library routine, and creates no events, streams or graphs.  The
// render runs on the scene's own stream and the call returns when it is done.
//
// The scratch — the path pool, its queues and accumulators, and the work
// items (pixel x chunk of samples) — lives in g_noalloc_scratch below
// (ARE_NOALLOC_SCRATCH_BYTES).  Both schedules of are_render run here
// (params->schedule; the megakernel is one launch of k_tail with at most
// ARE_NOALLOC_MAX_PATHS paths).
// The array belongs to the library's device module: every GPU that loads the
// library holds it until the process exits.  Kernels receive its address; host
// code never dereferences the symbol (on the host, the name is only a
// stand-in for the device array), so the address is looked up once per device
// with cudaGetSymbolAddress, with that device current, on the first call made
// on that device, and kept for the life of the process (a cudaDeviceReset of
// that device invalidates it; calls after one are not supported).  That first
// call should therefore come before any stream capture.  All calls share the
// one array and it keeps the last call's contents; everything that must start
// at zero is cleared by each call, and calls whose work overlaps on the GPU
// (two streams, two host threads) race on it: serialise them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>

#include "scene.h"
#include "wave.cuh"

namespace are_core {

namespace {

constexpr size_t NA_SLOT_BYTES = WAVE_SLOT_BYTES;  // queues, hit, accumulators
constexpr size_t NA_ITEM_BYTES = 2 * sizeof(float4);                  // per-pixel sum and sum of squares
constexpr size_t NA_SCRATCH = (size_t)ARE_NOALLOC_MAX_PATHS * NA_SLOT_BYTES + (size_t)ARE_NOALLOC_MAX_PIXELS * NA_ITEM_BYTES +
	64 * sizeof(unsigned) + 8 * sizeof(unsigned long long) + 18 * 256;  // 18 arrays, each padded to 256 bytes
static_assert(NA_SCRATCH <= (size_t)ARE_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the stated size");

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[ARE_NOALLOC_SCRATCH_BYTES];

namespace {

std::mutex g_mu;
void *g_scratch_addr[256];  // per device ordinal, filled on first use

are_status scratch_address(int device, unsigned char **out) {
	std::lock_guard<std::mutex> lk(g_mu);
	if (device < 0 || device >= 256) {
		set_error("device ordinal out of range");
		return ARE_ERR_INVALID_ARGUMENT;
	}
	if (!g_scratch_addr[device]) {
		void *p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
		if (e != cudaSuccess || !p) return cuda_status(e != cudaSuccess ? e : cudaErrorInvalidSymbol, "cudaGetSymbolAddress");
		g_scratch_addr[device] = p;
	}
	*out = (unsigned char *)g_scratch_addr[device];
	return ARE_OK;
}

template <class T>
T *take(unsigned char *&p, size_t count) {
	T *r = (T *)p;
	p += (count * sizeof(T) + 255) & ~(size_t)255;
	return r;
}

int blocks_for(const void *kernel, int n_sms) {
	int per_sm = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, BLOCK, 0);
	return std::max(1, per_sm) * n_sms;
}

are_status bad(const std::string &m) {
	set_error(m);
	return ARE_ERR_INVALID_ARGUMENT;
}

}  // namespace

are_status render_noalloc(are_scene *sc, const are_camera *cam, const are_render_params *prm, float *rgb, float *var,
	are_render_stats *stats) {
	if (!sc || !cam || !prm || !rgb) return bad("null scene, camera, params or output");
	const are_render_params &p = *prm;
	if (!(p.flags & ARE_FLAG_DEVICE_OUTPUT))
		return bad("are_render_noalloc writes device buffers only: set ARE_FLAG_DEVICE_OUTPUT and pass device pointers");
	if (p.estimator != ARE_EST_PATH) return bad("are_render_noalloc renders the path estimator only");
	if (p.width <= 0 || p.height <= 0 || p.spp <= 0 || p.max_depth <= 0 || p.max_depth > 255)
		return bad("width, height, spp must be > 0 and max_depth in [1, 255]");
	if ((int64_t)p.width * p.height > ARE_NOALLOC_MAX_PIXELS)
		return bad("image has " + std::to_string((int64_t)p.width * p.height) + " pixels; are_render_noalloc handles at most " +
			std::to_string(ARE_NOALLOC_MAX_PIXELS) + " (its scratch is a fixed static array)");
	if (p.pool_size > ARE_NOALLOC_MAX_PATHS)
		return bad("pool_size above ARE_NOALLOC_MAX_PATHS (" + std::to_string(ARE_NOALLOC_MAX_PATHS) + ")");
	if (!(cam->vfov_deg > 0.0f && cam->vfov_deg < 180.0f)) return bad("vfov must be in (0, 180)");
	if (!(p.t_min >= 0.0f) || !std::isfinite(p.t_min)) return bad("t_min must be finite and >= 0");
	if (p.schedule < ARE_SCHEDULE_AUTO || p.schedule > ARE_SCHEDULE_MEGAKERNEL) return bad("unknown schedule");
	if (cudaSetDevice(sc->device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
	const bool mega = p.schedule != ARE_SCHEDULE_WAVEFRONT;
	const bool linear = sc->linear;
	const int g_tail = tail_grid(linear, sc->dev, sc->n_sms);
	unsigned char *base = nullptr;
	if (are_status st = scratch_address(sc->device, &base)) return st;

	// work items are (pixel, chunk of samples), as in are_render; the automatic chunk is the smallest
	// whose items fit the array, so small images still spread over many paths
	Wave W{};
	W.npix = p.width * p.height;
	W.spp = p.spp;
	const int64_t max_chunks = ARE_NOALLOC_MAX_PIXELS / W.npix;  // >= 1: the pixel count was checked above
	W.chunk = p.chunk > 0 ? std::min(p.chunk, p.spp) : (int)((p.spp + max_chunks - 1) / max_chunks);
	W.nchunk = (p.spp + W.chunk - 1) / W.chunk;
	W.n_items = (int64_t)W.npix * W.nchunk;
	if (W.n_items > ARE_NOALLOC_MAX_PIXELS)
		return bad("chunk " + std::to_string(W.chunk) + " gives " + std::to_string(W.n_items) +
			" work items; are_render_noalloc handles at most " + std::to_string(ARE_NOALLOC_MAX_PIXELS));
	// megakernel: at most one path per resident thread of its persistent grid
	int P = p.pool_size > 0 ? p.pool_size : mega ? std::min(ARE_NOALLOC_MAX_PATHS, g_tail * BLOCK) : ARE_NOALLOC_MAX_PATHS;
	P = (int)std::min<int64_t>(P, W.n_items);
	P = std::min((P + 31) & ~31, ARE_NOALLOC_MAX_PATHS);
	W.P = P;
	W.max_depth = p.max_depth;
	W.rr_depth = p.rr_depth;
	W.t_min = p.t_min;
	W.seed = p.seed;
	camera_frame(*cam, p.width, p.height, p.flags, W.cam);
	unsigned char *z = base;
	for (int q = 0; q < 2; ++q)
		W.qa[q] = take<float4>(z, ARE_NOALLOC_MAX_PATHS), W.qb[q] = take<float4>(z, ARE_NOALLOC_MAX_PATHS),
		W.qc[q] = take<float4>(z, ARE_NOALLOC_MAX_PATHS), W.qd[q] = take<float4>(z, ARE_NOALLOC_MAX_PATHS);
	W.hit = take<float4>(z, ARE_NOALLOC_MAX_PATHS);
	W.acc_s = take<float4>(z, ARE_NOALLOC_MAX_PATHS), W.acc_c = take<float4>(z, ARE_NOALLOC_MAX_PATHS);
	W.acc_q = take<float4>(z, ARE_NOALLOC_MAX_PATHS);
	W.item_s = take<float4>(z, ARE_NOALLOC_MAX_PIXELS);
	W.item_q = take<float4>(z, ARE_NOALLOC_MAX_PIXELS);
	W.cnt = take<unsigned>(z, 64);
	W.stat = take<unsigned long long>(z, 8);
	if ((size_t)(z - base) > (size_t)ARE_NOALLOC_SCRATCH_BYTES) {
		set_error("scratch layout exceeds ARE_NOALLOC_SCRATCH_BYTES");
		return ARE_ERR_INTERNAL;
	}
	const int n_first = (int)std::min<int64_t>(P, W.n_items);

	cudaStream_t s = sc->stream;
	unsigned *hc = sc->host_counters;  // pinned, allocated with the scene
	// counters: queue 0 holds the first camera rays; next work item follows them
	for (int k = 0; k < 8; ++k) hc[k] = 0;
	hc[0] = hc[3] = (unsigned)n_first;
	cudaGetLastError();
	are_status st = cuda_status(cudaMemcpyAsync(W.cnt, hc, 8 * sizeof(unsigned), cudaMemcpyHostToDevice, s), "counters");
	if (!st) st = cuda_status(cudaMemsetAsync(W.stat, 0, 8 * sizeof(unsigned long long), s), "stats");
	if (!st) st = cuda_status(cudaStreamSynchronize(s), "counters");  // hc is reused for read-back below
	int64_t launches[4] = { 0, 0, 0, 0 }, iterations = 0;
	if (!st) {
		k_init<<<blocks_for((const void *)k_init, sc->n_sms), BLOCK, 0, s>>>(W, n_first);
		++launches[ARE_KERNEL_OTHER];
		st = cuda_status(cudaGetLastError(), "k_init launch");
	}
	if (!st && mega) {
		// the whole render in one persistent launch (queue 0 holds one camera path per thread)
		launch_tail(linear, g_tail, s, sc->dev, W);
		++launches[ARE_KERNEL_OTHER];
		st = cuda_status(cudaGetLastError(), "k_tail launch");
	}
	const int g_int = intersect_grid(linear, sc->dev, sc->n_sms);
	const int g_sh = blocks_for((const void *)k_shade, sc->n_sms);
	const int64_t max_rounds = (W.n_items / std::max(1, P) + 2) * (int64_t)p.max_depth * W.chunk / GRAPH_ITERS + 16;
	for (int64_t round = 0; !st && !mega; ++round) {
		for (int it = 0; it < GRAPH_ITERS; ++it) {
			int par = it & 1;
			launch_intersect(linear, g_int, s, sc->dev, W, par);
			k_shade<<<g_sh, BLOCK, 0, s>>>(sc->dev, W, par);
		}
		iterations += GRAPH_ITERS;
		for (int k = 0; k < 2; ++k) launches[k] += GRAPH_ITERS;
		st = cuda_status(cudaGetLastError(), "wavefront launch");
		if (st) break;
		st = cuda_status(cudaMemcpyAsync(hc, W.cnt, 8 * sizeof(unsigned), cudaMemcpyDeviceToHost, s), "counters");
		if (!st) st = cuda_status(cudaStreamSynchronize(s), "render iteration");
		if (st || hc[0] == 0) break;
		if (round > max_rounds) {
			set_error("render did not converge");
			st = ARE_ERR_INTERNAL;
		}
	}
	if (!st) {
		k_resolve<<<std::max(1, std::min(4096, (W.npix + BLOCK - 1) / BLOCK)), BLOCK, 0, s>>>(W, rgb, var,
			(p.flags & ARE_FLAG_CLAMP_OUTPUT) != 0);
		++launches[ARE_KERNEL_OTHER];
		st = cuda_status(cudaGetLastError(), "k_resolve launch");
	}
	unsigned long long hstat[2] = { 0, 0 };
	unsigned herr = 0;
	if (!st) {
		st = cuda_status(cudaMemcpyAsync(hc, W.stat, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s), "stats");
		if (!st) st = cuda_status(cudaMemcpyAsync(hc + 4, W.cnt + 4, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "error");
		if (!st) st = cuda_status(cudaStreamSynchronize(s), "render");
		if (!st) {
			hstat[0] = ((unsigned long long)hc[1] << 32) | hc[0];
			hstat[1] = ((unsigned long long)hc[3] << 32) | hc[2];
			herr = hc[4];
		}
	}
	if (!st && herr) {
		set_error("device error word " + std::to_string(herr));
		st = ARE_ERR_INTERNAL;
	}
	if (stats) {
		*stats = are_render_stats{};
		stats->samples = (int64_t)hstat[1];
		stats->segments = (int64_t)hstat[0];
		stats->iterations = iterations;
		for (int k = 0; k < 4; ++k) stats->kernel_launches[k] = launches[k];
		stats->error_word = (int32_t)herr;
	}
	return st;
}

}  // namespace are_core
