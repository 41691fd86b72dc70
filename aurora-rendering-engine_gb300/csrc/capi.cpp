// capi.cpp — the extern "C" entry points of include/aurora_gb300.h.
// Every entry point converts C++ exceptions into status codes; nothing is
// thrown across the ABI.
#include <cuda_runtime.h>

#include <new>
#include <string>

#include "aurora_gb300.h"
#include "scene.h"

namespace are_core {
are_status config_build(int32_t config, uint64_t seed, int32_t freq, are_config **out);
}

namespace {

template <class F>
are_status guarded(F &&f) {
	try {
		are_core::set_error("");
		return f();
	} catch (const std::bad_alloc &) {
		are_core::set_error("out of host memory");
		return ARE_ERR_OUT_OF_MEMORY;
	} catch (const std::exception &e) {
		are_core::set_error(e.what());
		return ARE_ERR_INTERNAL;
	} catch (...) {
		are_core::set_error("unknown exception");
		return ARE_ERR_INTERNAL;
	}
}

}  // namespace

extern "C" {

ARE_API const char *are_status_string(are_status s) {
	switch (s) {
	case ARE_OK: return "ok";
	case ARE_ERR_INVALID_ARGUMENT: return "invalid argument";
	case ARE_ERR_CUDA: return "CUDA error";
	case ARE_ERR_OUT_OF_MEMORY: return "out of memory";
	case ARE_ERR_NO_DEVICE: return "no device";
	case ARE_ERR_KERNEL_TIMEOUT: return "kernel timeout";
	case ARE_ERR_INTERNAL: return "internal error";
	case ARE_ERR_IO: return "file error";
	}
	return "unknown status";
}

ARE_API const char *are_last_error(void) { return are_core::last_error(); }

ARE_API int32_t are_version(void) { return 10000; }

ARE_API int32_t are_device_count(void) {
	int n = 0;
	if (cudaGetDeviceCount(&n) != cudaSuccess) {
		cudaGetLastError();
		return 0;
	}
	return n;
}

ARE_API are_status are_trim_memory(int32_t device) {
	return guarded([&] { return are_core::pool_trim(device); });
}

ARE_API are_status are_scene_create(const are_scene_desc *desc, are_scene **out) {
	return guarded([&] { return are_core::scene_create(desc, out); });
}

ARE_API are_status are_scene_destroy(are_scene *scene) {
	return guarded([&] {
		delete scene;
		return ARE_OK;
	});
}

ARE_API are_status are_scene_info(const are_scene *scene, int64_t *n_prims, int64_t *n_nodes, int32_t *max_leaf,
	int32_t *depth) {
	if (!scene) {
		are_core::set_error("null scene");
		return ARE_ERR_INVALID_ARGUMENT;
	}
	if (n_prims) *n_prims = scene->n_prims;
	if (n_nodes) *n_nodes = scene->n_nodes;
	if (max_leaf) *max_leaf = scene->max_leaf;
	if (depth) *depth = scene->depth;
	return ARE_OK;
}

ARE_API are_status are_render(are_scene *scene, const are_camera *camera, const are_render_params *params,
	float *rgb_out, float *var_out, are_render_stats *stats) {
	return guarded([&] { return are_core::render(scene, camera, params, rgb_out, var_out, stats); });
}

ARE_API are_status are_render_noalloc(are_scene *scene, const are_camera *camera, const are_render_params *params,
	float *rgb_out, float *var_out, are_render_stats *stats) {
	return guarded([&] { return are_core::render_noalloc(scene, camera, params, rgb_out, var_out, stats); });
}

ARE_API are_status are_render_batch(are_scene *const *scenes, const are_camera *cameras,
	const are_render_params *params, int32_t n, const are_batch_options *options, float *const *rgb_out,
	double *scene_ms, are_render_stats *stats) {
	return guarded([&] { return are_core::render_batch(scenes, cameras, params, n, options, rgb_out, scene_ms, stats); });
}

ARE_API are_status are_batch_autotune(const are_scene_desc *const *descs, const are_camera *cameras,
	const are_render_params *params, int32_t n, int32_t calib_spp, are_batch_options *best, double *best_ms) {
	return guarded([&] { return are_core::batch_autotune(descs, cameras, params, n, calib_spp, best, best_ms); });
}

ARE_API are_status are_intersect(are_scene *scene, const float *rays, int64_t n, float *hits, int32_t device_ptrs,
	float *ms_out) {
	return guarded([&] { return are_core::intersect(scene, rays, n, hits, device_ptrs, ms_out); });
}

ARE_API are_status are_tonemap(const float *rgb, int64_t n_values, const are_tonemap_params *params, uint8_t *out) {
	return guarded([&] { return are_core::tonemap(rgb, n_values, params, out); });
}

ARE_API are_status are_write_ppm(const char *path, const uint8_t *rgb8, int32_t width, int32_t height) {
	return guarded([&] { return are_core::write_ppm(path, rgb8, width, height); });
}

ARE_API are_status are_write_pfm(const char *path, const float *rgb, int32_t width, int32_t height) {
	return guarded([&] { return are_core::write_pfm(path, rgb, width, height); });
}

ARE_API are_status are_read_ppm(const char *path, int32_t *width, int32_t *height, float *texels) {
	return guarded([&] { return are_core::read_ppm(path, width, height, texels); });
}

ARE_API are_status are_config_build(int32_t config, uint64_t seed, int32_t mesh_frequency, are_config **out) {
	return guarded([&] { return are_core::config_build(config, seed, mesh_frequency, out); });
}

}  // extern "C"
