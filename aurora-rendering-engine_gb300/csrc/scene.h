// scene.h — host-side owner of a device-resident scene and its render
// workspace (the opaque are_scene of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "core.h"

struct are_scene {
	are_core::DevScene dev{};
	int device = 0;
	int n_sms = 0;
	int64_t n_prims = 0, n_nodes = 0;
	bool linear = false;  // closest hits by the linear scan of staged primitives (else the BVH)
	int32_t n_spheres = 0, n_quads = 0, n_triangles = 0;
	int32_t max_leaf = 0, depth = 0;
	float box_lo[3] = { 0, 0, 0 }, box_hi[3] = { 0, 0, 0 };  // bounds of all primitives
	std::vector<void *> allocations;       // device buffers owned by the scene (cudaMalloc)
	std::vector<void *> pool_allocations;  // device buffers from the device's pool (freed on `stream`)
	cudaStream_t stream = nullptr;

	// cached wavefront workspace (grown on demand)
	void *ws = nullptr;
	size_t ws_bytes = 0;
	void *items = nullptr;
	size_t items_bytes = 0;
	unsigned *host_counters = nullptr;  // pinned (a block of the process-wide slab)

	// the render's CUDA graph and timing events, kept between renders: a new
	// render updates the instantiated graph in place (same topology, new
	// kernel parameters) instead of instantiating it again
	cudaGraphExec_t render_exec = nullptr;
	std::vector<cudaEvent_t> render_events;

	~are_scene();
};

namespace are_core {

// thread-local last error message for are_last_error()
void set_error(const std::string &msg);
const char *last_error();

// CUDA call guard: records a message and returns ARE_ERR_CUDA / ARE_ERR_OUT_OF_MEMORY
are_status cuda_status(cudaError_t e, const char *what);

// Memory.  Scene arrays and render workspaces come from one stream-ordered
// pool per device (cudaMemPool) that keeps up to an eighth of the device's
// memory (at least 1 GiB) cached after frees, so a
// caller that creates, renders and destroys a scene per frame does not pay
// cudaMalloc and cudaFree (each a device-wide synchronisation) every time.
// Allocations are ordered on the scene's stream; pool_free releases on it.
are_status pool_alloc(are_scene *sc, size_t bytes, void **p);
void pool_free(are_scene *sc, void *p);
// releases the cached (unused) memory of device's pool, or of every pool for -1
are_status pool_trim(int device);
// 256-byte pinned host blocks (read-back counters) from a process-wide slab
unsigned *pinned_block_acquire();
void pinned_block_release(unsigned *p);

are_status scene_create(const are_scene_desc *desc, are_scene **out);
are_status render(are_scene *sc, const are_camera *cam, const are_render_params *p, float *rgb, float *var,
	are_render_stats *stats);
are_status render_noalloc(are_scene *sc, const are_camera *cam, const are_render_params *p, float *rgb, float *var,
	are_render_stats *stats);
are_status render_batch(are_scene *const *scenes, const are_camera *cams, const are_render_params *params, int n,
	const are_batch_options *opt, float *const *rgb_out, double *scene_ms, are_render_stats *stats);
are_status batch_autotune(const are_scene_desc *const *descs, const are_camera *cams, const are_render_params *params,
	int n, int calib_spp, are_batch_options *best, double *best_ms);
are_status render_legacy(are_scene *sc, const are_camera *cam, const are_render_params &p, float *rgb,
	are_render_stats *stats);
are_status intersect(are_scene *sc, const float *rays, int64_t n, float *hits, int32_t device_ptrs, float *ms);
are_status tonemap(const float *rgb, int64_t n, const are_tonemap_params *p, uint8_t *out);
are_status write_ppm(const char *path, const uint8_t *rgb8, int w, int h);
are_status write_pfm(const char *path, const float *rgb, int w, int h);
are_status read_ppm(const char *path, int *w, int *h, float *texels);

}  // namespace are_core
