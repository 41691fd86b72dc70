// lbvh.cu — the BVH built on the device (are_scene_desc.bvh_build =
// ARE_BVH_DEVICE): a linear BVH over Morton codes (Karras, "Maximizing
// Parallelism in the Construction of BVHs, Octrees, and k-d Trees", HPG
// 2012), collapsed to the leaf size and laid out in the same 32-byte node
// format as the host SAH build (core.h), so traversal and results do not
// change: the tree changes the cost of a closest-hit query, never its answer.
//
//   k_lbvh_boxes     per primitive: bounds computed in FP64 and rounded
//                    outward to FP32 (as the host build), centroid, and block
//                    reductions of the centroid bounds and coordinate scale
//   k_lbvh_morton    30-bit Morton code of the centroid, key = code << 32 | index
//   (radix sort of the 64-bit keys: CUB, the one library call of the build)
//   k_lbvh_tree      one thread per internal node: range and split from the
//                    longest common prefixes of neighbouring keys
//   k_lbvh_bounds    one thread per leaf walks to the root; the second thread
//                    to reach a node merges its children's boxes
//   k_lbvh_depth     interior nodes that stay interior after collapsing
//                    (more than leaf_size primitives) and their depths
//   k_lbvh_top_rank  breadth-first ranks of the interior nodes of depth < 9:
//                    their child pairs take nodes 2 .. 1023, the ones the
//                    traversal stages in shared memory
//   k_lbvh_emit      the node records: child pairs at even indices, leaves
//                    as (first, count) ranges of the sorted primitives
//   k_lbvh_gather    primitive records, ids, materials and uvs in leaf order
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>

#include "core.h"
#include "lbvh.h"
#include "scene.h"

namespace are_core {

namespace {

constexpr int LB = 256;
constexpr int TOP_DEPTH = 9;  // interior nodes above this depth: at most 511, their pairs fill nodes 2 .. 1023
constexpr uint32_t LEAF_BIT = 0x80000000u;

// float order-preserving integer encoding (for atomic min/max of floats)
__device__ __forceinline__ uint32_t f2o(float f) {
	uint32_t u = __float_as_uint(f);
	return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t u) { return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u); }

struct Reduce {
	uint32_t cmin[3], cmax[3];  // centroid bounds (ordered ints)
	uint32_t scale;             // max |coordinate| of the primitive boxes (ordered int of a non-negative float)
};

// bounds of record j (3 float4: sphere c,r / quad Q,u,v / triangle v0,v1,v2), in double
__device__ __forceinline__ void record_bounds(const float4 *P, double lo[3], double hi[3]) {
	const float4 p0 = P[0], p1 = P[1], p2 = P[2];
	const double a[3] = { p0.x, p0.y, p0.z }, b[3] = { p1.x, p1.y, p1.z }, c[3] = { p2.x, p2.y, p2.z };
	if (p0.w > 0.0f) {  // sphere: centre, radius in .w
		for (int k = 0; k < 3; ++k) lo[k] = a[k] - p0.w, hi[k] = a[k] + p0.w;
	} else if (p0.w == PRIM_TAG_QUAD) {
		for (int k = 0; k < 3; ++k) {
			const double c1 = a[k] + b[k], c2 = a[k] + c[k], c3 = c1 + c[k];
			lo[k] = fmin(fmin(a[k], c1), fmin(c2, c3));
			hi[k] = fmax(fmax(a[k], c1), fmax(c2, c3));
		}
	} else {
		for (int k = 0; k < 3; ++k) lo[k] = fmin(fmin(a[k], b[k]), c[k]), hi[k] = fmax(fmax(a[k], b[k]), c[k]);
	}
}

__global__ void __launch_bounds__(LB) k_lbvh_boxes(const float4 *__restrict__ rec, int n, float4 *__restrict__ box,
	float4 *__restrict__ cen, Reduce *red) {
	__shared__ uint32_t s[7];
	if (threadIdx.x < 7) s[threadIdx.x] = threadIdx.x < 3 ? 0xffffffffu : 0u;
	__syncthreads();
	uint32_t lmin[3] = { 0xffffffffu, 0xffffffffu, 0xffffffffu }, lmax[3] = { 0u, 0u, 0u }, lscale = f2o(0.0f);
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		double lo[3], hi[3];
		record_bounds(rec + 3 * (size_t)i, lo, hi);
		float flo[3], fhi[3], c[3];
		for (int k = 0; k < 3; ++k) {
			flo[k] = __double2float_rd(lo[k]);
			fhi[k] = __double2float_ru(hi[k]);
			c[k] = (float)(0.5 * (lo[k] + hi[k]));
			lmin[k] = min(lmin[k], f2o(c[k]));
			lmax[k] = max(lmax[k], f2o(c[k]));
			lscale = max(lscale, f2o(fmaxf(fabsf(flo[k]), fabsf(fhi[k]))));
		}
		box[2 * (size_t)i] = make_float4(flo[0], flo[1], flo[2], 0.f);
		box[2 * (size_t)i + 1] = make_float4(fhi[0], fhi[1], fhi[2], 0.f);
		cen[i] = make_float4(c[0], c[1], c[2], 0.f);
	}
	for (int k = 0; k < 3; ++k) atomicMin(&s[k], lmin[k]), atomicMax(&s[3 + k], lmax[k]);
	atomicMax(&s[6], lscale);
	__syncthreads();
	if (threadIdx.x == 0) {
		for (int k = 0; k < 3; ++k) atomicMin(&red->cmin[k], s[k]), atomicMax(&red->cmax[k], s[3 + k]);
		atomicMax(&red->scale, s[6]);
	}
}

__device__ __forceinline__ uint32_t spread10(uint32_t v) {  // 10 bits -> every third bit
	v = (v * 0x00010001u) & 0xFF0000FFu;
	v = (v * 0x00000101u) & 0x0F00F00Fu;
	v = (v * 0x00000011u) & 0xC30C30C3u;
	v = (v * 0x00000005u) & 0x49249249u;
	return v;
}

__global__ void __launch_bounds__(LB) k_lbvh_morton(const float4 *__restrict__ cen, int n, const Reduce *red,
	unsigned long long *__restrict__ keys) {
	float lo[3], inv[3];
	for (int k = 0; k < 3; ++k) {
		lo[k] = o2f(red->cmin[k]);
		const float ext = o2f(red->cmax[k]) - lo[k];
		inv[k] = ext > 0.f ? 1023.0f / ext : 0.f;
	}
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const float4 c = cen[i];
		const float v[3] = { c.x, c.y, c.z };
		uint32_t q[3];
		for (int k = 0; k < 3; ++k) q[k] = (uint32_t)fminf(fmaxf((v[k] - lo[k]) * inv[k], 0.f), 1023.f);
		const uint32_t code = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
		keys[i] = ((unsigned long long)code << 32) | (uint32_t)i;
	}
}

// length of the common prefix of keys i and j; -1 outside [0, n)
__device__ __forceinline__ int delta(const unsigned long long *k, int n, int i, int j) {
	if (j < 0 || j >= n) return -1;
	return __clzll(k[i] ^ k[j]);  // keys are distinct
}

// child reference: internal node index, or LEAF_BIT | sorted primitive index
__global__ void __launch_bounds__(LB) k_lbvh_tree(const unsigned long long *__restrict__ k, int n, uint2 *__restrict__ child,
	int2 *__restrict__ range, int *__restrict__ parent, int *__restrict__ leaf_parent) {
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x) {
		const int d = delta(k, n, i, i + 1) > delta(k, n, i, i - 1) ? 1 : -1;
		const int dmin = delta(k, n, i, i - d);
		int lmax = 2;
		while (delta(k, n, i, i + lmax * d) > dmin) lmax <<= 1;
		int l = 0;
		for (int t = lmax >> 1; t >= 1; t >>= 1)
			if (delta(k, n, i, i + (l + t) * d) > dmin) l += t;
		const int j = i + l * d;
		const int dnode = delta(k, n, i, j);
		int s = 0;
		for (int t = (l + 1) >> 1;; t = (t + 1) >> 1) {
			if (delta(k, n, i, i + (s + t) * d) > dnode) s += t;
			if (t == 1) break;
		}
		const int g = i + s * d + min(d, 0);
		const int first = min(i, j), last = max(i, j);
		const uint32_t left = first == g ? (LEAF_BIT | (uint32_t)g) : (uint32_t)g;
		const uint32_t right = last == g + 1 ? (LEAF_BIT | (uint32_t)(g + 1)) : (uint32_t)(g + 1);
		child[i] = make_uint2(left, right);
		range[i] = make_int2(first, last);
		if (left & LEAF_BIT) leaf_parent[g] = i; else parent[g] = i;
		if (right & LEAF_BIT) leaf_parent[g + 1] = i; else parent[g + 1] = i;
	}
}

// bottom-up boxes of the internal nodes (nbox: 2 float4 per node)
__global__ void __launch_bounds__(LB) k_lbvh_bounds(const float4 *__restrict__ pbox, const unsigned *__restrict__ sorted_idx,
	int n, const uint2 *__restrict__ child, const int *__restrict__ parent, const int *__restrict__ leaf_parent,
	unsigned *__restrict__ visits, float4 *__restrict__ nbox) {
	for (int li = blockIdx.x * blockDim.x + threadIdx.x; li < n; li += gridDim.x * blockDim.x) {
		int node = leaf_parent[li];
		while (node >= 0) {
			__threadfence();
			if (atomicAdd(&visits[node], 1u) == 0) break;  // the sibling's thread finishes this node
			__threadfence();
			const uint2 c = child[node];
			float4 lo = make_float4(INFINITY, INFINITY, INFINITY, 0.f), hi = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.f);
			for (int h = 0; h < 2; ++h) {
				const uint32_t r = h ? c.y : c.x;
				float4 a, b;
				if (r & LEAF_BIT) {
					const unsigned p = sorted_idx[r & ~LEAF_BIT];
					a = pbox[2 * (size_t)p], b = pbox[2 * (size_t)p + 1];
				} else {
					a = __ldcg(&nbox[2 * (size_t)r]), b = __ldcg(&nbox[2 * (size_t)r + 1]);
				}
				lo = make_float4(fminf(lo.x, a.x), fminf(lo.y, a.y), fminf(lo.z, a.z), 0.f);
				hi = make_float4(fmaxf(hi.x, b.x), fmaxf(hi.y, b.y), fmaxf(hi.z, b.z), 0.f);
			}
			__stcg(&nbox[2 * (size_t)node], lo);
			__stcg(&nbox[2 * (size_t)node + 1], hi);
			node = node == 0 ? -1 : parent[node];
		}
	}
}

// interior after collapsing: more than leaf_size primitives below
__global__ void __launch_bounds__(LB) k_lbvh_depth(const int2 *__restrict__ range, const int *__restrict__ parent, int n,
	int leaf_size, int *__restrict__ kept, int *__restrict__ depth, unsigned *__restrict__ top_list, unsigned *top_count,
	unsigned *max_depth) {
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x) {
		const int2 r = range[i];
		const int keep = (r.y - r.x + 1) > leaf_size;
		kept[i] = keep;
		int d = 0;
		if (keep) {
			for (int p = i; p > 0 && d < 1024; p = parent[p]) ++d;  // parents are set for every node but the root
			if (d < TOP_DEPTH) top_list[atomicAdd(top_count, 1u)] = ((unsigned)d << 27) | (unsigned)i;
			atomicMax(max_depth, (unsigned)d);
		}
		depth[i] = d;
	}
}

// rank of each listed node by (depth, index); at most 511 nodes, one block
__global__ void k_lbvh_top_rank(const unsigned *__restrict__ top_list, const unsigned *top_count, int *__restrict__ top_rank) {
	const unsigned t = *top_count;
	for (unsigned a = threadIdx.x; a < t; a += blockDim.x) {
		const unsigned ka = top_list[a];
		unsigned r = 0;
		for (unsigned b = 0; b < t; ++b) r += top_list[b] < ka;
		top_rank[ka & 0x07ffffffu] = (int)r;
	}
}

// pair index of a kept interior node: breadth-first for the top ones, index order after
__device__ __forceinline__ int pair_of(int i, const int *depth, const int *top_rank, const int *rest_scan, int n_top) {
	return depth[i] < TOP_DEPTH ? top_rank[i] : n_top + rest_scan[i];
}

__global__ void __launch_bounds__(LB) k_lbvh_emit(int n, int leaf_size, const uint2 *__restrict__ child,
	const int2 *__restrict__ range, const int *__restrict__ kept, const int *__restrict__ depth,
	const int *__restrict__ top_rank, const int *__restrict__ rest_scan, const unsigned *top_count,
	const float4 *__restrict__ nbox, const float4 *__restrict__ pbox, const unsigned *__restrict__ sorted_idx, float pad,
	float4 *__restrict__ out, unsigned *max_leaf) {
	const int n_top = (int)*top_count;
	auto put = [&](int slot, float4 lo, float4 hi, int a, int b) {
		out[2 * (size_t)slot] = make_float4(lo.x - pad, lo.y - pad, lo.z - pad, __int_as_float(a));
		out[2 * (size_t)slot + 1] = make_float4(hi.x + pad, hi.y + pad, hi.z + pad, __int_as_float(b));
	};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x) {
		if (!kept[i]) continue;
		const int base = 2 + 2 * pair_of(i, depth, top_rank, rest_scan, n_top);
		if (i == 0) put(0, nbox[0], nbox[1], base, 0);  // root
		const uint2 c = child[i];
		for (int h = 0; h < 2; ++h) {
			const uint32_t r = h ? c.y : c.x;
			if (r & LEAF_BIT) {
				const int s = (int)(r & ~LEAF_BIT);
				const unsigned p = sorted_idx[s];
				put(base + h, pbox[2 * (size_t)p], pbox[2 * (size_t)p + 1], s, 1);
				atomicMax(max_leaf, 1u);
			} else if (kept[r]) {
				put(base + h, nbox[2 * (size_t)r], nbox[2 * (size_t)r + 1], 2 + 2 * pair_of((int)r, depth, top_rank, rest_scan, n_top), 0);
			} else {
				const int2 rg = range[r];
				put(base + h, nbox[2 * (size_t)r], nbox[2 * (size_t)r + 1], rg.x, rg.y - rg.x + 1);
				atomicMax(max_leaf, (unsigned)(rg.y - rg.x + 1));
			}
		}
	}
}

__global__ void __launch_bounds__(LB) k_lbvh_gather(const float4 *__restrict__ rec, const int32_t *__restrict__ mat_in,
	const float *__restrict__ uv_in, const unsigned *__restrict__ sorted_idx, int n, float4 *__restrict__ prims,
	int32_t *__restrict__ gid, int32_t *__restrict__ mat, float *__restrict__ uv) {
	for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
		const unsigned p = sorted_idx[j];
		prims[3 * (size_t)j] = rec[3 * (size_t)p];
		prims[3 * (size_t)j + 1] = rec[3 * (size_t)p + 1];
		prims[3 * (size_t)j + 2] = rec[3 * (size_t)p + 2];
		gid[j] = (int32_t)p;
		mat[j] = mat_in[p];
		if (uv)
			for (int k = 0; k < 6; ++k) uv[6 * (size_t)j + k] = uv_in[6 * (size_t)p + k];
	}
}

__global__ void k_lowbits(const unsigned long long *__restrict__ keys, int n, unsigned *__restrict__ idx) {
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) idx[i] = (unsigned)keys[i];
}

__global__ void k_lbvh_rest_flags(const int *__restrict__ kept, const int *__restrict__ depth, int m, int *__restrict__ flags) {
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
		flags[i] = kept[i] && depth[i] >= TOP_DEPTH;
}

}  // namespace

// rec/mat_in/uv_in: device records in input order (3 float4 per primitive as
// in DevScene::prims, global id = position).  The outputs (nodes, records in
// leaf order, ids, materials, uvs) are allocated here and owned by the scene.
are_status build_bvh_device(are_scene *sc, const float4 *rec, const int32_t *mat_in, const float *uv_in, int n,
	int leaf_size, LbvhResult &res, cudaStream_t s) {
	if (leaf_size <= 0) leaf_size = 4;
	if (leaf_size > 64) leaf_size = 64;
	if (n <= leaf_size || n >= (1 << 27)) {
		set_error("device BVH build: primitive count out of range");
		return ARE_ERR_INVALID_ARGUMENT;
	}
	const int m = n - 1;  // internal nodes of the radix tree
	const int grid = std::max(1, std::min(sc->n_sms * 8, (n + LB - 1) / LB));
	size_t cub_sort = 0, cub_scan = 0;
	cub::DeviceRadixSort::SortKeys(nullptr, cub_sort, (unsigned long long *)nullptr, (unsigned long long *)nullptr, n, 0,
		62, s);
	cub::DeviceScan::ExclusiveSum(nullptr, cub_scan, (int *)nullptr, (int *)nullptr, m, s);
	const size_t cub_bytes = std::max(cub_sort, cub_scan);
	auto layout = [&](char *z, bool assign, float4 **pbox, float4 **cen, Reduce **red, unsigned long long **keys,
					  unsigned long long **keys_sorted, unsigned **sorted_idx, uint2 **child, int2 **range, int **parent,
					  int **leaf_parent, unsigned **visits, float4 **nbox, int **kept, int **depth, unsigned **top_list,
					  int **top_rank, int **flags, int **rest_scan, unsigned **counters, void **cub_tmp) {
		auto take = [&](auto **dst, size_t bytes) {
			if (assign) *dst = reinterpret_cast<std::remove_reference_t<decltype(**dst)> *>(z);
			z += (bytes + 255) & ~(size_t)255;
		};
		take(pbox, 32 * (size_t)n), take(cen, 16 * (size_t)n), take(red, sizeof(Reduce)), take(keys, 8 * (size_t)n),
			take(keys_sorted, 8 * (size_t)n), take(sorted_idx, 4 * (size_t)n), take(child, 8 * (size_t)n),
			take(range, 8 * (size_t)n), take(parent, 4 * (size_t)n), take(leaf_parent, 4 * (size_t)n),
			take(visits, 4 * (size_t)n), take(nbox, 32 * (size_t)n), take(kept, 4 * (size_t)n), take(depth, 4 * (size_t)n),
			take(top_list, 4 * 512), take(top_rank, 4 * (size_t)n), take(flags, 4 * (size_t)n),
			take(rest_scan, 4 * (size_t)n), take(counters, 32);
		if (assign) *cub_tmp = z;
		z += cub_bytes;
		return (size_t)z;
	};
	float4 *pbox, *cen, *nbox;
	Reduce *red;
	unsigned long long *keys, *keys_sorted;
	unsigned *sorted_idx, *visits, *top_list, *counters;
	uint2 *child;
	int2 *range;
	int *parent, *leaf_parent, *kept, *depth, *top_rank, *flags, *rest_scan;
	void *cub_tmp;
	const size_t need = layout(nullptr, false, &pbox, &cen, &red, &keys, &keys_sorted, &sorted_idx, &child, &range, &parent,
		&leaf_parent, &visits, &nbox, &kept, &depth, &top_list, &top_rank, &flags, &rest_scan, &counters, &cub_tmp);
	void *scratch = nullptr;
	if (are_status st = cuda_status(cudaMalloc(&scratch, need), "cudaMalloc(BVH build)")) return st;
	struct Free {
		void *p;
		~Free() { cudaFree(p); }
	} release{ scratch };
	layout((char *)scratch, true, &pbox, &cen, &red, &keys, &keys_sorted, &sorted_idx, &child, &range, &parent,
		&leaf_parent, &visits, &nbox, &kept, &depth, &top_list, &top_rank, &flags, &rest_scan, &counters, &cub_tmp);

	auto alloc = [&](void **p, size_t bytes) -> are_status {
		if (are_status st = cuda_status(cudaMalloc(p, bytes), "cudaMalloc(scene)")) return st;
		sc->allocations.push_back(*p);
		return ARE_OK;
	};
	float4 *prims = nullptr, *nodes = nullptr;
	int32_t *gid = nullptr, *mat = nullptr;
	float *uv = nullptr;
	if (are_status st = alloc((void **)&prims, 48 * (size_t)n)) return st;
	if (are_status st = alloc((void **)&gid, 4 * (size_t)n)) return st;
	if (are_status st = alloc((void **)&mat, 4 * (size_t)n)) return st;
	if (uv_in)
		if (are_status st = alloc((void **)&uv, 24 * (size_t)n)) return st;

	cudaGetLastError();
	Reduce init;
	for (int k = 0; k < 3; ++k) init.cmin[k] = 0xffffffffu, init.cmax[k] = 0u;
	init.scale = 0x80000000u;  // ordered encoding of +0
	cudaMemcpyAsync(red, &init, sizeof init, cudaMemcpyHostToDevice, s);
	cudaMemsetAsync(visits, 0, 4 * (size_t)n, s);
	cudaMemsetAsync(counters, 0, 32, s);
	cudaMemsetAsync(parent, 0xff, 4 * (size_t)n, s);
	k_lbvh_boxes<<<grid, LB, 0, s>>>(rec, n, pbox, cen, red);
	k_lbvh_morton<<<grid, LB, 0, s>>>(cen, n, red, keys);
	size_t tb = cub_sort;
	if (are_status st = cuda_status(cub::DeviceRadixSort::SortKeys(cub_tmp, tb, keys, keys_sorted, n, 0, 62, s), "radix sort"))
		return st;
	k_lowbits<<<grid, LB, 0, s>>>(keys_sorted, n, sorted_idx);
	k_lbvh_tree<<<grid, LB, 0, s>>>(keys_sorted, n, child, range, parent, leaf_parent);
	k_lbvh_bounds<<<grid, LB, 0, s>>>(pbox, sorted_idx, n, child, parent, leaf_parent, visits, nbox);
	k_lbvh_depth<<<grid, LB, 0, s>>>(range, parent, n, leaf_size, kept, depth, top_list, counters, counters + 1);
	k_lbvh_top_rank<<<1, 512, 0, s>>>(top_list, counters, top_rank);
	k_lbvh_rest_flags<<<grid, LB, 0, s>>>(kept, depth, m, flags);
	tb = cub_scan;
	if (are_status st = cuda_status(cub::DeviceScan::ExclusiveSum(cub_tmp, tb, flags, rest_scan, m, s), "scan"))
		return st;
	k_lbvh_gather<<<grid, LB, 0, s>>>(rec, mat_in, uv_in, sorted_idx, n, prims, gid, mat, uv);
	if (are_status st = cuda_status(cudaGetLastError(), "device BVH build kernels")) return st;
	// sizes: kept nodes = top ones + the scanned rest
	unsigned hc[2] = { 0, 0 };
	int last_scan = 0, last_flag = 0;
	uint32_t scale_o = 0;
	float4 root[2];
	cudaMemcpyAsync(hc, counters, 8, cudaMemcpyDeviceToHost, s);
	cudaMemcpyAsync(&last_scan, rest_scan + (m - 1), 4, cudaMemcpyDeviceToHost, s);
	cudaMemcpyAsync(&last_flag, flags + (m - 1), 4, cudaMemcpyDeviceToHost, s);
	cudaMemcpyAsync(&scale_o, &red->scale, 4, cudaMemcpyDeviceToHost, s);
	cudaMemcpyAsync(root, nbox, sizeof root, cudaMemcpyDeviceToHost, s);
	if (are_status st = cuda_status(cudaStreamSynchronize(s), "device BVH build")) return st;
	const int n_top = (int)hc[0];
	const int64_t kept_total = (int64_t)n_top + last_scan + last_flag;
	const int64_t n_nodes = 2 + 2 * kept_total;
	float scale;
	{
		uint32_t u = (scale_o & 0x80000000u) ? (scale_o & 0x7fffffffu) : ~scale_o;
		std::memcpy(&scale, &u, 4);
	}
	const float pad = (float)((double)scale * std::ldexp(1.0, -19)) + 1e-30f;
	if (are_status st = alloc((void **)&nodes, 32 * (size_t)n_nodes)) return st;
	// node 1: the padding node of the first pair, an inverted box that is never hit
	const float4 padnode[2] = { make_float4(1.f, 1.f, 1.f, 0.f), make_float4(-1.f, -1.f, -1.f, 0.f) };
	cudaMemcpyAsync(nodes + 2, padnode, sizeof padnode, cudaMemcpyHostToDevice, s);
	k_lbvh_emit<<<grid, LB, 0, s>>>(n, leaf_size, child, range, kept, depth, top_rank, rest_scan, counters, nbox, pbox,
		sorted_idx, pad, nodes, counters + 2);
	unsigned max_leaf = 0;
	cudaMemcpyAsync(&max_leaf, counters + 2, 4, cudaMemcpyDeviceToHost, s);
	if (are_status st = cuda_status(cudaGetLastError(), "k_lbvh_emit")) return st;
	if (are_status st = cuda_status(cudaStreamSynchronize(s), "device BVH build")) return st;
	res = LbvhResult{};
	res.nodes = nodes;
	res.prims = prims;
	res.gid = gid;
	res.mat = mat;
	res.uv = uv;
	res.n_nodes = n_nodes;
	res.depth = (int)hc[1] + 1;
	res.max_leaf = (int)max_leaf;
	res.box_pad = pad;
	for (int k = 0; k < 3; ++k) {
		res.lo[k] = (&root[0].x)[k];
		res.hi[k] = (&root[1].x)[k];
	}
	return ARE_OK;
}

}  // namespace are_core
