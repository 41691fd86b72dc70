// core.h — internal types shared by the host side and the CUDA kernels.
//
// Device layout (all in HBM, built once per scene by scene.cpp):
//   prims    : 3 x float4 per primitive, in BVH leaf order.
//              sphere   [0] = (centre, radius > 0)
//              quad     [0] = (Q, -1), [1] = (u, 0), [2] = (v, 0)
//              triangle [0] = (v0, -2), [1] = (v1, 0), [2] = (v2, 0)
//   prim_gid : leaf order -> global id (spheres, then quads, then triangles)
//   prim_mat : leaf order -> material index
//   tri_uv   : leaf order -> 6 floats of per-vertex uv (triangles only, optional)
//   nodes    : 2 x float4 (32 B) per BVH node:
//              [0] = (bmin, a), [1] = (bmax, b) with a, b int bits;
//              b == 0: interior, children a and a+1 (a is even, so a child
//              pair is one aligned 64-byte line); b > 0: leaf of b prims
//              starting at a.  Node 0 is the root, node 1 is padding.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "aurora_gb300.h"

namespace are_core {

constexpr float PRIM_TAG_QUAD = -1.0f;
constexpr float PRIM_TAG_TRI = -2.0f;
constexpr int MAX_STACK = 64;      // traversal stack entries per ray
constexpr int MAX_BVH_DEPTH = 60;  // the builder never exceeds this
constexpr int SMEM_NODES = 1024;   // top BVH nodes staged in shared memory (32 KB)
constexpr int SMEM_NODES4 = 256;   // the same 32 KB as 4-wide nodes (128 bytes each)
constexpr int MAX_STACK4 = 96;     // 4-wide traversal: up to 3 entries per level
constexpr int WIDE_BVH_MIN_PRIMS = 1 << 19;  // automatic bvh_width: 4-wide above this many primitives
// scenes with at most this many primitives are scanned linearly from shared
// memory (4 float4 per primitive) instead of traversing the BVH
constexpr int LINEAR_MAX = 48;
static_assert(6 * LINEAR_MAX <= 2 * SMEM_NODES, "staged primitives must fit the node buffer");

// error bits of the device error word
enum : uint32_t {
	ERR_STACK_OVERFLOW = 1u,
	ERR_QUEUE_OVERFLOW = 2u,
	ERR_BAD_INDEX = 4u,
	ERR_NONFINITE = 8u,
	ERR_TENSOR_TIMEOUT = 16u,  // a bounded wait for tensor-core work or a bulk copy gave up
	ERR_BVH_WALK = 32u,        // a traversal visited more nodes than the tree has (malformed tree): stopped
};

struct DevMaterial {  // mirrors are_material (48 B)
	int32_t type, texture;
	float fuzz, ior;
	float emit[3];
	float reflect_ratio;
	float tint[3];
	float pad_;
};

struct DevTexture {  // mirrors are_texture (64 B)
	int32_t type, mapping;
	float scale;
	int32_t width, height, texel_offset;
	float a[3], b[3], center[3];
	int32_t filter;
};

struct DevScene {
	const float4 *prims;
	const int32_t *prim_gid;
	const int32_t *prim_mat;
	const float *tri_uv;       // null if the scene has no per-vertex uv
	const float4 *nodes;
	const float4 *nodes4;      // 4-wide tree (8 float4 per node), null if not built
	int32_t n_nodes4;
	const float4 *leaves;      // leaf boxes (node format) when n_prims <= LINEAR_MAX
	int32_t n_leaves;
	const DevMaterial *mats;
	const DevTexture *texs;
	const float *texels;
	int32_t n_prims, n_nodes;
	int32_t n_materials, n_textures;
	int32_t background, triangle_test;
	float bg_a[3], bg_b[3];
	float box_pad;             // absolute padding applied to every node box
	int32_t interleave;        // megakernels interleave the lanes' binary-tree walks (scenes with quads or triangles)
};

}  // namespace are_core
