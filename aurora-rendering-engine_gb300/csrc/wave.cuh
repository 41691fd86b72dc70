// wave.cuh — the wavefront's device-side state (one struct passed by value
// to every kernel) and the kernels' declarations, shared by the render entry
// points.
#pragma once

#include <cuda_runtime.h>

#include "core.h"
#include "shade.cuh"

namespace are_core {

constexpr int GRAPH_ITERS = 8;  // iterations per graph launch (even)
constexpr int BLOCK = 256;
// resident blocks per SM requested for the tail / megakernel (registers per thread follow):
// linear-scan scenes run best at 4 (64 registers); binary trees walked ray by ray at 2 (104
// registers, no spill); binary trees whose walks interleave (mega.cuh) at 3 (80 registers; four
// blocks' shared memory does not fit beside their 256 staged nodes); 4-wide trees, whose walks
// always interleave, at 4 (64 registers: more warps to cover the node loads of incoherent rays
// outweigh the spills)
constexpr int TAIL_MIN_BLOCKS_LINEAR = 4;
constexpr int TAIL_MIN_BLOCKS_BVH = 2;
constexpr int TAIL_MIN_BLOCKS_BVH_INTERLEAVED = 3;
constexpr int TAIL_MIN_BLOCKS_WIDE = 4;
__host__ __device__ constexpr int tail_min_blocks(bool linear, bool wide, bool interleaved) {
	return linear ? TAIL_MIN_BLOCKS_LINEAR
		 : wide   ? TAIL_MIN_BLOCKS_WIDE
		 : interleaved ? TAIL_MIN_BLOCKS_BVH_INTERLEAVED
					   : TAIL_MIN_BLOCKS_BVH;
}
// wide nodes the megakernel stages in shared memory (16 KB: four blocks per SM fit with their stacks)
constexpr int TAIL_SMEM_NODES4 = 128;
constexpr int64_t MEGA_ITEM_BUDGET = 12ll << 30;  // bytes of per-item sums the megakernel's automatic chunk allows
constexpr int TAIL_SHORT_STACK = 8;       // binary-tree traversal-stack entries per thread in shared memory
constexpr int TAIL_SHORT_STACK_WIDE = 8;  // the same for the 4-wide tree
constexpr int INTERSECT_SHORT_STACK = 4;  // the wavefront's intersect (keeps 4 blocks of 256 per SM)

struct Wave {
	// Ray queues: one 64-byte record per queued path segment, SoA over 4 float4:
	//   qa = (origin, slot bits)  qb = (direction, depth | j << 8)
	//   qc = (throughput, item bits)  qd = (radiance so far, 0)
	// The path state travels with its ray, so every kernel reads and writes
	// its records in queue order; only the per-slot accumulators are gathered.
	float4 *qa[2], *qb[2], *qc[2], *qd[2];
	float4 *hit;      // (t, leaf bits, u, v) per queue position
	float4 *acc_s;    // Kahan sum (xyz) per slot
	float4 *acc_c;    // Kahan compensation per slot
	float4 *acc_q;    // sum of squares per slot
	unsigned *cnt;    // [0],[1] queue sizes, [3] next work item, [4] error word, [6], [7] guided counters
	unsigned long long *stat;  // [0] segments, [1] samples
	float4 *item_s;   // per work item: sum (xyz)
	float4 *item_q;   // per work item: sum of squares; null when every item is one sample (resolve squares the sum)
	int32_t P;
	int32_t npix, spp, chunk, nchunk;
	int64_t n_items;
	int32_t max_depth, rr_depth;
	float t_min;
	uint64_t seed;
	CameraFrame cam;
};

// bytes of wavefront state per path slot (queues x 2, hit, accumulators)
constexpr size_t WAVE_SLOT_BYTES = 2 * 4 * sizeof(float4) + sizeof(float4) + 3 * sizeof(float4);

// rt.cpp:339-343 camera basis (host)
void camera_frame(const are_camera &c, int w, int h, int flags, CameraFrame &f);

__global__ void k_init(Wave W, int n_first);
__global__ void k_shade(DevScene S, Wave W, int par);
__global__ void k_resolve(Wave W, float *__restrict__ rgb, float *__restrict__ var, int clamp);
// k_tail (render.cu) for a scene scanned linearly (linear) or through its BVH, on queue 0;
// tail_grid: its persistent grid (resident blocks x SMs)
void launch_tail(bool linear, int grid, cudaStream_t s, const DevScene &S, const Wave &W);
int tail_grid(bool linear, const DevScene &S, int n_sms);
// k_intersect (render.cu) for a linear-scan or BVH scene on queue par, and its grid
void launch_intersect(bool linear, int grid, cudaStream_t s, const DevScene &S, const Wave &W, int par);
int intersect_grid(bool linear, const DevScene &S, int n_sms);

}  // namespace are_core
