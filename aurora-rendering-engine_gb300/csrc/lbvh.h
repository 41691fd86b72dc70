// lbvh.h — the device BVH build (lbvh.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "aurora_gb300.h"

struct are_scene;

namespace are_core {

struct LbvhResult {
	float4 *nodes = nullptr;    // 2 float4 per node, core.h layout
	float4 *prims = nullptr;    // records in leaf order
	int32_t *gid = nullptr, *mat = nullptr;
	float *uv = nullptr;
	int64_t n_nodes = 0;
	int depth = 0, max_leaf = 0;
	float box_pad = 0.0f;
	float lo[3] = { 0, 0, 0 }, hi[3] = { 0, 0, 0 };  // bounds of all primitives
};

are_status build_bvh_device(are_scene *sc, const float4 *rec, const int32_t *mat_in, const float *uv_in, int n,
	int leaf_size, LbvhResult &res, cudaStream_t s);

}  // namespace are_core
