// guide.cu — training and inference kernels of the path-guiding network, and
// the are_guide_* entry points.
//
//   k_guide_pack_tc   FP32 master parameters -> the tcgen05 weight images
//                     (forward, and transposed for the backward pass)
//   k_guide_infer     fused forward of 128-row tiles on the 5th-generation
//                     tensor cores (tcgen05.mma, accumulators in tensor memory)
//   k_guide_fwdbwd_tc the same forward plus loss gradient and backward chain
//                     on the tensor cores; stores each layer's input and
//                     output gradient (FP16)
//   k_guide_wgrad   weight and bias gradients dW = sum_s delta_s h_s^T on the
//                   tensor cores, K = samples, split over blocks, FP32 atomics
//   k_guide_adam    Adam on the FP32 master weights, skipped on FP16 overflow
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "guide.cuh"
#include "guide_host.h"
#include "scene.h"
#include "tc05.cuh"

namespace are_core {

namespace {

constexpr int GT = 256;  // threads per block of the MLP kernels (8 warps)

__global__ void k_guide_pack_tc(const float *__restrict__ P, __half *__restrict__ img) {
	// the backward image (TCB_*) after the forward one
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < TCB_HALVES; i += gridDim.x * blockDim.x) {
		int base, K, off, outs;
		if (i < TCB_W4) base = TCB_W5, K = TCB_K5, off = OFF_W5, outs = 40;
		else if (i < TCB_W3) base = TCB_W4, K = GN_H, off = OFF_W4, outs = GN_H;
		else if (i < TCB_W2) base = TCB_W3, K = GN_H, off = OFF_W3, outs = GN_H;
		else base = TCB_W2, K = GN_H, off = OFF_W2, outs = GN_H;
		const int j = i - base, grp = j / (K * 8), rem = j - grp * (K * 8);
		const int kc = rem >> 6, in = rem & 63;
		const int row = grp * 8 + (in >> 3), k = kc * 8 + (in & 7);  // row: the layer's input, k: its output
		img[TC_HALVES + i] = __float2half_rn(k < outs ? P[off + k * GN_H + row] : 0.0f);
	}
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < TC_HALVES; i += gridDim.x * blockDim.x) {
		// invert tc_index for the layer holding i
		int base, K, off, boff, rows_used;
		if (i < TC_W2) base = TC_W1, K = TC_K1, off = OFF_W1, boff = OFF_B1, rows_used = GN_H;
		else if (i < TC_W3) base = TC_W2, K = TC_KH, off = OFF_W2, boff = OFF_B2, rows_used = GN_H;
		else if (i < TC_W4) base = TC_W3, K = TC_KH, off = OFF_W3, boff = OFF_B3, rows_used = GN_H;
		else if (i < TC_W5) base = TC_W4, K = TC_KH, off = OFF_W4, boff = OFF_B4, rows_used = GN_H;
		else base = TC_W5, K = TC_KH, off = OFF_W5, boff = OFF_B5, rows_used = 40;
		const int j = i - base, grp = j / (K * 8), rem = j - grp * (K * 8);
		const int kc = rem >> 6, in = rem & 63;
		const int row = grp * 8 + (in >> 3), k = kc * 8 + (in & 7);
		const int in_cols = base == TC_W1 ? GN_ENC : GN_H;   // columns of the FP32 matrix
		const int one = base == TC_W1 ? TC_ONE1 : GN_H;       // the bias column
		float v = 0.0f;
		if (row < rows_used) v = k == one ? P[boff + row] : (k < one ? P[off + row * in_cols + k] : 0.0f);
		img[i] = __float2half_rn(v);
	}
}

// ---- inference on the 5th-generation tensor cores ---------------------------
//
// A block is four warpgroups; each warpgroup runs 128-row tiles on its own
// (thread t of the warpgroup owns row t of the tile):
//   layer 1 in two K halves: the thread writes its row's encoding chunks
//   0..15 (K = 128) into the warpgroup's FP16 tile in shared memory
//   (K-major core matrices), one thread issues 8 tcgen05.mma (M = 128,
//   N = 64, K = 16) into the warpgroup's tensor-memory columns and commits
//   them to the warpgroup's mbarrier; after they complete the same tile takes
//   chunks 16..29 (K = 112) and 7 more MMAs accumulate;
//   layers 2..5: every thread reads its row's accumulators (tcgen05.ld),
//   converts them with ReLU to FP16 (one cvt.rn.relu.f16x2 per pair) into the
//   next layer's input tile (K = 80: 64 activations, a constant 1 that
//   carries the bias inside the GEMM, zeros) and the MMAs of that layer run;
//   the 48 outputs of the row go to global memory, raw or as the packed vMF
//   mixture the renderer samples.
// Layer 1's bias rides in encoding column 225, whose input is the constant 1.
// The weights (68 KB) arrive once per block by bulk copy.  Four warpgroups
// keep four tiles in flight per SM, so one warpgroup's encoding and
// epilogues overlap the others' MMAs.  The next tile's features are loaded
// while the current tile runs.  Every wait is bounded: on timeout the error
// word gets ERR_TENSOR_TIMEOUT and the block stops, frees its tensor memory
// and returns.
constexpr int TC_WG = 4;
constexpr int TC_THREADS = 128 * TC_WG;
constexpr int TC_A_BYTES = 128 * 128 * 2;           // one tile of K <= 128
constexpr int TC_SBO_E0 = 128 * 16;                 // bytes between 8-row groups: encoding chunks 0..15
constexpr int TC_SBO_E1 = 112 * 16;                 // encoding chunks 16..29
constexpr int TC_SBO1 = TC_K1 * 16;                 // layer 1's weights (K = 240)
constexpr int TC_SBOH = TC_KH * 16;                 // K = 80
constexpr uint32_t TC_COLS = 512;                   // tensor-memory columns per block: 128 per warpgroup
constexpr uint32_t TC_POLL_LIMIT = 1u << 22;        // polls of a bounded mbarrier wait
constexpr size_t TC_OFF_A = (size_t)TC_HALVES * 2;
constexpr size_t TC_OFF_BAR = TC_OFF_A + (size_t)TC_WG * TC_A_BYTES;
constexpr size_t TC_SMEM = TC_OFF_BAR + 128;
static_assert(TC_OFF_A % 16 == 0 && TC_OFF_BAR % 8 == 0 && (TC_HALVES * 2) % 16 == 0, "bulk copy / mbarrier alignment");
static_assert(TC_SMEM <= 227 * 1024, "shared memory of one block");
static_assert(TC_COLS >= 128u * TC_WG && TC_COLS <= 512u, "tensor memory of one block");

__device__ __forceinline__ uint32_t pack_h2(float a, float b) { return h2u(__floats2half2_rn(a, b)); }
// (max(lo, 0), max(hi, 0)) rounded to FP16, lo in the low half
__device__ __forceinline__ uint32_t pack_relu_h2(float lo, float hi) {
	uint32_t d;
	asm("cvt.rn.relu.f16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
	return d;
}

// Encoding chunk c (8 halves: pairs 4c .. 4c + 3) of a row.  Pair 12 i + k is
// (sin, cos)(pi 2^k x_i): chunk c < 27 is feature i = c / 3 at k = 4j .. 4j + 3
// (j = c % 3), i.e. one evaluation on the special-function unit at k = 4j on
// the argument reduced to [-1, 1] (2^4j x - 2 rint(2^(4j-1) x) is exact;
// absolute error about 4e-7 there) and three angle doublings (sin 2a =
// 2 sin a cos a, cos 2a = (cos a - sin a)(cos a + sin a); error <= 8x).
// Chunk 27 is the raw features 0..7, chunk 28 (x_8, 1: layer 1's bias input,
// 0...), chunk 29 zeros.  c must be a compile-time constant after unrolling.
__device__ __forceinline__ uint4 enc_chunk(const float *x, int c) {
	if (c < 27) {
		const int i = c / 3, j = c % 3;
		const float y = j == 0 ? x[i] : (float)(1 << (4 * j)) * x[i] - 2.0f * rintf((float)(1 << (4 * j - 1)) * x[i]);
		float sn, cs;
		__sincosf(3.14159265358979323846f * y, &sn, &cs);
		uint32_t p[4];
		p[0] = pack_h2(sn, cs);
#pragma unroll
		for (int k = 1; k < 4; ++k) {
			const float s2 = 2.f * sn * cs, c2 = (cs - sn) * (cs + sn);
			sn = s2, cs = c2;
			p[k] = pack_h2(sn, cs);
		}
		return make_uint4(p[0], p[1], p[2], p[3]);
	}
	if (c == 27) return make_uint4(pack_h2(x[0], x[1]), pack_h2(x[2], x[3]), pack_h2(x[4], x[5]), pack_h2(x[6], x[7]));
	if (c == 28) return make_uint4(pack_h2(x[8], 1.0f), 0u, 0u, 0u);
	return make_uint4(0u, 0u, 0u, 0u);
}

// one layer's MMAs: D[tcol] (+)= A (128 x 16 ksteps) x W^T, W rows of stride sbo_w
__device__ __forceinline__ void tc_mmas(uint32_t d_tmem, uint32_t a_addr, uint32_t sbo_a, uint32_t w_addr, uint32_t sbo_w,
	int ksteps, uint32_t idesc, bool accumulate) {
	for (int s = 0; s < ksteps; ++s)
		umma_f16(d_tmem, umma_sdesc(a_addr + 256u * s, 128u, sbo_a), umma_sdesc(w_addr + 256u * s, 128u, sbo_w), idesc,
			(accumulate || s > 0) ? 1u : 0u);
}

// first_limit: polls allowed for each warpgroup's first MMA wait (the others get TC_POLL_LIMIT); a
// caller that wants to see the give-up path taken sets it to 0
__global__ void __launch_bounds__(TC_THREADS, 1) k_guide_infer(const __half *__restrict__ tc_img,
	const float *__restrict__ feat, int n, const unsigned *__restrict__ n_dev, float *__restrict__ out,
	unsigned *__restrict__ err, int mixture_out, uint32_t first_limit) {
	extern __shared__ __align__(16) unsigned char smem[];
	uint64_t *bar = reinterpret_cast<uint64_t *>(smem + TC_OFF_BAR);  // [0] weights, [1 + wg] MMAs of warpgroup wg
	uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar + 1 + TC_WG);
	volatile uint32_t *fail = tmem_slot + 1;  // per warpgroup

	const int tid = threadIdx.x, wg = tid >> 7, lt = tid & 127, warp = tid >> 5;
	if (n_dev) n = min(n, (int)*n_dev);
	const int tiles = (n + 127) / 128;
	if (blockIdx.x * TC_WG >= tiles) return;  // no tile for this block: skip the weight copy and tensor memory
	const bool out_vec = (reinterpret_cast<uintptr_t>(out) & 15) == 0;  // rows are 192 bytes: float4 stores when aligned
	if (tid == 0) {
		for (int b = 0; b < 1 + TC_WG; ++b) mbar_init(&bar[b], 1);
		for (int w = 0; w < TC_WG; ++w) fail[w] = 0;
		mbar_init_fence();
	}
	if (warp == 0) {
		tmem_alloc(tmem_slot, TC_COLS);
		tmem_relinquish();
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tbase = *tmem_slot;
	if (tid == 0) {
		mbar_arrive_expect_tx(&bar[0], (uint32_t)(TC_HALVES * 2));
		bulk_g2s(smem, tc_img, (uint32_t)(TC_HALVES * 2), &bar[0]);
	}
	if (lt == 0 && !mbar_wait(&bar[0], 0, TC_POLL_LIMIT)) fail[wg] = 1;

	unsigned char *A = smem + TC_OFF_A + (size_t)wg * TC_A_BYTES;
	const uint32_t a_addr = smem_addr(A), w_addr = smem_addr(smem);
	const uint32_t tcol = tbase + (uint32_t)wg * 128u;             // this warpgroup's columns
	const uint32_t tlane = (uint32_t)((warp & 3) * 32) << 16;      // this warp's lane quarter
	const uint32_t bar_id = 1 + wg;
	const uint32_t idesc_h = umma_idesc_f16(128, GN_H), idesc_o = umma_idesc_f16(128, GN_OUT);
	uint32_t phase = 0;
	uint64_t *mbar = &bar[1 + wg];
	unsigned char *e0row = A + (lt >> 3) * TC_SBO_E0 + (lt & 7) * 16;
	unsigned char *e1row = A + (lt >> 3) * TC_SBO_E1 + (lt & 7) * 16;
	unsigned char *hrow = A + (lt >> 3) * TC_SBOH + (lt & 7) * 16;
	// issue the MMAs of `stage` after the tile's writes are visible; false once the warpgroup has failed
	auto sync_issue = [&](int stage) -> bool {
		fence_proxy_async_smem();
		tc_fence_before();
		named_bar(bar_id, 128);
		if (fail[wg]) return false;
		if (lt == 0) {
			tc_fence_after();
			if (stage == 0)
				tc_mmas(tcol, a_addr, TC_SBO_E0, w_addr + TC_W1 * 2, TC_SBO1, 8, idesc_h, false);
			else if (stage == 1)
				tc_mmas(tcol, a_addr, TC_SBO_E1, w_addr + TC_W1 * 2 + 256u * 8, TC_SBO1, 7, idesc_h, true);
			else
				tc_mmas(tcol + (stage == 5 ? 64u : 0u), a_addr, TC_SBOH,
					w_addr + (stage == 2 ? TC_W2 : stage == 3 ? TC_W3 : stage == 4 ? TC_W4 : TC_W5) * 2, TC_SBOH, TC_KH / 16,
					stage == 5 ? idesc_o : idesc_h, false);
			umma_commit(mbar);
		}
		return true;
	};
	// one thread polls the mbarrier; the others sleep in the named barrier
	// instead of spending issue slots the other warpgroups could use
	uint32_t limit = min(first_limit, TC_POLL_LIMIT);
	auto wait_mma = [&]() {
		if (lt == 0) {
			if (!mbar_wait(mbar, phase, limit)) fail[wg] = 1;
			tc_fence_before();
		}
		limit = TC_POLL_LIMIT;
		phase ^= 1u;
		named_bar(bar_id, 128);
		tc_fence_after();
	};
	named_bar(bar_id, 128);
	int tile = blockIdx.x * TC_WG + wg;
	const int tstep = gridDim.x * TC_WG;
	float xn[GN_IN];
#pragma unroll
	for (int k = 0; k < GN_IN; ++k) xn[k] = (tile * 128 + lt < n) ? feat[(size_t)(tile * 128 + lt) * GN_IN + k] : 0.0f;
	for (; tile < tiles; tile += tstep) {
		const int row = tile * 128 + lt;
		float x[GN_IN];
#pragma unroll
		for (int k = 0; k < GN_IN; ++k) x[k] = xn[k];
		const int nrow = row + tstep * 128;  // prefetch the next tile's features
#pragma unroll
		for (int k = 0; k < GN_IN; ++k) xn[k] = nrow < n ? feat[(size_t)nrow * GN_IN + k] : 0.0f;
		// layer 1, first K half
#pragma unroll
		for (int c = 0; c < 16; ++c) *reinterpret_cast<uint4 *>(e0row + c * 128) = enc_chunk(x, c);
		if (!sync_issue(0)) break;
		wait_mma();
		// layer 1, second K half (the tile is free again)
#pragma unroll
		for (int c = 16; c < 30; ++c) *reinterpret_cast<uint4 *>(e1row + (c - 16) * 128) = enc_chunk(x, c);
		if (!sync_issue(1)) break;
		wait_mma();
		bool ok = true;
#pragma unroll 1
		for (int layer = 2; layer <= 5 && ok; ++layer) {
			// accumulators of row lt -> ReLU -> FP16 input tile of the next layer, 32 columns at a time
#pragma unroll
			for (int h = 0; h < 2; ++h) {
				uint32_t r[2][16];
				tmem_ld16(tcol + tlane + 32u * h, r[0]);
				tmem_ld16(tcol + tlane + 32u * h + 16u, r[1]);
				tmem_ld_wait();
#pragma unroll
				for (int c = 0; c < 4; ++c) {
					uint32_t w4[4];
#pragma unroll
					for (int e = 0; e < 4; ++e) {
						const int col = 8 * c + 2 * e;
						w4[e] = pack_relu_h2(__uint_as_float(r[col >> 4][col & 15]), __uint_as_float(r[col >> 4][(col & 15) + 1]));
					}
					*reinterpret_cast<uint4 *>(hrow + (4 * h + c) * 128) = make_uint4(w4[0], w4[1], w4[2], w4[3]);
				}
			}
			if (layer == 2) {
				*reinterpret_cast<uint4 *>(hrow + 8 * 128) = make_uint4(pack_h2(1.f, 0.f), 0u, 0u, 0u);
				*reinterpret_cast<uint4 *>(hrow + 9 * 128) = make_uint4(0u, 0u, 0u, 0u);
			}
			ok = sync_issue(layer);
			if (ok) wait_mma();
		}
		if (!ok) break;
		uint32_t r[3][16];
#pragma unroll
		for (int g = 0; g < 3; ++g) tmem_ld16(tcol + 64u + tlane + 16u * g, r[g]);
		tmem_ld_wait();
		if (row < n && mixture_out) {
			// the vMF mixture of the row, packed for the renderer (out is 16-byte aligned there)
			float o[5 * GN_LOBES];
#pragma unroll
			for (int col = 0; col < 5 * GN_LOBES; ++col) o[col] = __uint_as_float(r[col >> 4][col & 15]);
			float pk[GN_OUT];
			pack_mixture_fast(o, pk);
			float4 *dst = reinterpret_cast<float4 *>(out + (size_t)row * GN_OUT);
#pragma unroll
			for (int q = 0; q < GN_OUT / 4; ++q) dst[q] = make_float4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
		} else if (row < n) {
			float *orow = out + (size_t)row * GN_OUT;
			if (out_vec) {
				float4 *o = reinterpret_cast<float4 *>(orow);
#pragma unroll
				for (int q = 0; q < GN_OUT / 4; ++q) {
					const int col = 4 * q;
					o[q] = make_float4(__uint_as_float(r[col >> 4][col & 15]), __uint_as_float(r[col >> 4][(col & 15) + 1]),
						__uint_as_float(r[col >> 4][(col & 15) + 2]), __uint_as_float(r[col >> 4][(col & 15) + 3]));
				}
			} else {
#pragma unroll
				for (int col = 0; col < GN_OUT; ++col) orow[col] = __uint_as_float(r[col >> 4][col & 15]);
			}
		}
		tc_fence_before();
	}
	named_bar(bar_id, 128);
	if (lt == 0 && fail[wg]) {
		atomicOr(err, (unsigned)ERR_TENSOR_TIMEOUT);
		// let work still in flight land before the memory is released
		mbar_wait(&bar[0], 0, TC_POLL_LIMIT);
		mbar_wait(mbar, phase ^ 1u, TC_POLL_LIMIT);
	}
	tc_fence_before();
	__syncthreads();
	if (warp == 0) {
		tc_fence_after();
		tmem_dealloc(tbase, TC_COLS);
	}
}

// d(-log q)/d(outputs) of one sample (as oracle/orc_guide.c out_grad), times wt.
__device__ float sample_out_grad(const float *o, f3 w, float wt, float *g) {
	Mixture m;
	to_mixture(o, m);
	float v[GN_LOBES], q = 0.f;
	for (int l = 0; l < GN_LOBES; ++l) {
		float c = m.mu[l].x * w.x + m.mu[l].y * w.y + m.mu[l].z * w.z;
		v[l] = m.norm[l] * expf(m.kappa[l] * (c - 1.f));
		q += m.pi[l] * v[l];
	}
	q = fmaxf(q, 1e-30f);
	for (int l = 0; l < GN_LOBES; ++l) {
		float r = m.pi[l] * v[l] / q;
		float k = m.kappa[l];
		float c = m.mu[l].x * w.x + m.mu[l].y * w.y + m.mu[l].z * w.z;
		float dlogv = 1.f / k - 2.f / expm1f(2.f * k) + (c - 1.f);
		float sig = 1.f / (1.f + expf(-o[5 * l + 3]));
		g[5 * l + 3] = -r * dlogv * sig * wt;
		float dmu[3] = { -r * k * w.x, -r * k * w.y, -r * k * w.z };
		const float *mm = o + 5 * l;
		float nm = sqrtf(mm[0] * mm[0] + mm[1] * mm[1] + mm[2] * mm[2]);
		float len = nm + 1e-6f;
		float mdot = dmu[0] * mm[0] + dmu[1] * mm[1] + dmu[2] * mm[2];
		for (int j = 0; j < 3; ++j) g[5 * l + j] = (dmu[j] / len - (nm > 0.f ? mm[j] * mdot / (nm * len * len) : 0.f)) * wt;
		g[5 * l + 4] = (m.pi[l] - r) * wt;
	}
	return -wt * logf(q);
}

// ---- forward + backward of a training batch on the 5th-generation tensor cores
//
// k_guide_fwdbwd_tc runs k_guide_infer's forward on 128-row tiles (thread t of
// a warpgroup owns row t) and then, per row: stores its encoding and its four
// hidden activations (FP16, for k_guide_wgrad; the encoding with 0 in the
// bias column, as the master layout has it) and keeps their ReLU masks as bits;
// computes d(-log q)/d(outputs) times the sample's weight and the loss scale
// (sample_out_grad, clipped, FP16) and stores it; then the backward chain on
// the tensor cores: that gradient tile times layer 5's transposed weights
// (K = 48) gives the gradient at h4, which is masked by h4 > 0, clipped,
// rounded to FP16, stored and multiplied by W4^T, and so on down to the
// gradient at h1.  The same numbers as k_guide_fwdbwd up to the order of FP32
// sums and the encoding's last bits.  Waits are bounded as in k_guide_infer;
// a warpgroup that gives up sets ERR_TENSOR_TIMEOUT and the step's overflow
// flag, so the Adam step that follows is skipped.
constexpr size_t TT_OFF_A = (size_t)(TC_HALVES + TCB_HALVES) * 2;
constexpr size_t TT_OFF_BAR = TT_OFF_A + (size_t)TC_WG * TC_A_BYTES;
constexpr size_t TT_SMEM = TT_OFF_BAR + 128;
static_assert(TT_OFF_A % 16 == 0 && TT_OFF_BAR % 8 == 0, "bulk copy / mbarrier alignment");
static_assert(TT_SMEM <= 227 * 1024, "shared memory of one block");
static_assert(TCB_K5 % 16 == 0 && GN_H % 16 == 0, "backward K in 16-element steps");

// the 64 accumulators of row lt at columns [col, col + 64) -> FP16 pairs (ReLU'd when relu, else
// multiplied by the mask bits and clipped), written to the row's input tile (8 chunks) and,
// when g is not null, to g[0..7] (the row's 128 bytes in global memory); relu also returns the
// mask bits (value > 0) of the 64 results
__device__ __forceinline__ uint64_t tt_epilogue(uint32_t taddr, unsigned char *hrow, uint4 *g, bool relu,
	uint64_t mask, float clip) {
	uint64_t bits = 0;
#pragma unroll
	for (int h = 0; h < 2; ++h) {
		uint32_t r[2][16];
		tmem_ld16(taddr + 32u * h, r[0]);
		tmem_ld16(taddr + 32u * h + 16u, r[1]);
		tmem_ld_wait();
#pragma unroll
		for (int c = 0; c < 4; ++c) {
			uint32_t w4[4];
#pragma unroll
			for (int e = 0; e < 4; ++e) {
				const int col = 8 * c + 2 * e, j = 32 * h + col;
				float lo = __uint_as_float(r[col >> 4][col & 15]), hi = __uint_as_float(r[col >> 4][(col & 15) + 1]);
				if (relu) {
					w4[e] = pack_relu_h2(lo, hi);
					bits |= (uint64_t)((w4[e] & 0x7fffu) != 0u) << j;
					bits |= (uint64_t)((w4[e] & 0x7fff0000u) != 0u) << (j + 1);
				} else {
					lo = ((mask >> j) & 1u) ? fminf(fmaxf(lo, -clip), clip) : 0.f;
					hi = ((mask >> (j + 1)) & 1u) ? fminf(fmaxf(hi, -clip), clip) : 0.f;
					w4[e] = pack_h2(lo, hi);
				}
			}
			const uint4 v = make_uint4(w4[0], w4[1], w4[2], w4[3]);
			*reinterpret_cast<uint4 *>(hrow + (4 * h + c) * 128) = v;
			if (g) g[4 * h + c] = v;
		}
	}
	return bits;
}

__global__ void __launch_bounds__(TC_THREADS, 1) k_guide_fwdbwd_tc(const __half *__restrict__ tc_img,
	const float *__restrict__ samples, int n, float wscale, const float *__restrict__ wscale_dev, float wclip,
	float lscale, GuideTrainBufs B, float *__restrict__ loss_sum, unsigned *__restrict__ overflow,
	unsigned *__restrict__ err, uint32_t first_limit) {
	if (wscale_dev) wscale = *wscale_dev > 0.f ? (float)n / *wscale_dev : 0.f;  // device sum of the weights
	extern __shared__ __align__(16) unsigned char smem[];
	uint64_t *bar = reinterpret_cast<uint64_t *>(smem + TT_OFF_BAR);  // [0] weights, [1 + wg] MMAs of warpgroup wg
	uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar + 1 + TC_WG);
	volatile uint32_t *fail = tmem_slot + 1;  // per warpgroup

	const int tid = threadIdx.x, wg = tid >> 7, lt = tid & 127, warp = tid >> 5;
	const int tiles = (n + 127) / 128;
	if (blockIdx.x * TC_WG >= tiles) return;
	if (tid == 0) {
		for (int b = 0; b < 1 + TC_WG; ++b) mbar_init(&bar[b], 1);
		for (int w = 0; w < TC_WG; ++w) fail[w] = 0;
		mbar_init_fence();
	}
	if (warp == 0) {
		tmem_alloc(tmem_slot, TC_COLS);
		tmem_relinquish();
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tbase = *tmem_slot;
	if (tid == 0) {
		mbar_arrive_expect_tx(&bar[0], (uint32_t)((TC_HALVES + TCB_HALVES) * 2));
		bulk_g2s(smem, tc_img, (uint32_t)((TC_HALVES + TCB_HALVES) * 2), &bar[0]);
	}
	if (lt == 0 && !mbar_wait(&bar[0], 0, TC_POLL_LIMIT)) fail[wg] = 1;

	unsigned char *A = smem + TT_OFF_A + (size_t)wg * TC_A_BYTES;
	const uint32_t a_addr = smem_addr(A), w_addr = smem_addr(smem), wt_addr = w_addr + TC_HALVES * 2;
	const uint32_t tcol = tbase + (uint32_t)wg * 128u;
	const uint32_t tlane = (uint32_t)((warp & 3) * 32) << 16;
	const uint32_t bar_id = 1 + wg;
	const uint32_t idesc_h = umma_idesc_f16(128, GN_H), idesc_o = umma_idesc_f16(128, GN_OUT);
	uint32_t phase = 0;
	uint64_t *mbar = &bar[1 + wg];
	unsigned char *e0row = A + (lt >> 3) * TC_SBO_E0 + (lt & 7) * 16;
	unsigned char *e1row = A + (lt >> 3) * TC_SBO_E1 + (lt & 7) * 16;
	unsigned char *hrow = A + (lt >> 3) * TC_SBOH + (lt & 7) * 16;
	// stages 0..5: the forward (as k_guide_infer); 6..9: the backward through layers 5, 4, 3, 2
	auto sync_issue = [&](int stage) -> bool {
		fence_proxy_async_smem();
		tc_fence_before();
		named_bar(bar_id, 128);
		if (fail[wg]) return false;
		if (lt == 0) {
			tc_fence_after();
			if (stage == 0) {
				tc_mmas(tcol, a_addr, TC_SBO_E0, w_addr + TC_W1 * 2, TC_SBO1, 8, idesc_h, false);
			} else if (stage == 1) {
				tc_mmas(tcol, a_addr, TC_SBO_E1, w_addr + TC_W1 * 2 + 256u * 8, TC_SBO1, 7, idesc_h, true);
			} else if (stage <= 5) {
				tc_mmas(tcol + (stage == 5 ? 64u : 0u), a_addr, TC_SBOH,
					w_addr + (stage == 2 ? TC_W2 : stage == 3 ? TC_W3 : stage == 4 ? TC_W4 : TC_W5) * 2, TC_SBOH, TC_KH / 16,
					stage == 5 ? idesc_o : idesc_h, false);
			} else {
				const int K = stage == 6 ? TCB_K5 : GN_H;
				const int off = stage == 6 ? TCB_W5 : stage == 7 ? TCB_W4 : stage == 8 ? TCB_W3 : TCB_W2;
				tc_mmas(tcol, a_addr, TC_SBOH, wt_addr + off * 2, (uint32_t)K * 16u, K / 16, idesc_h, false);
			}
			umma_commit(mbar);
		}
		return true;
	};
	// first_limit: polls allowed for each warpgroup's first MMA wait, as in k_guide_infer
	uint32_t limit = min(first_limit, TC_POLL_LIMIT);
	auto wait_mma = [&]() {
		if (lt == 0) {
			if (!mbar_wait(mbar, phase, limit)) fail[wg] = 1;
			tc_fence_before();
		}
		limit = TC_POLL_LIMIT;
		phase ^= 1u;
		named_bar(bar_id, 128);
		tc_fence_after();
	};
	named_bar(bar_id, 128);
	const float clip = 60000.f;
	float lacc = 0.f;
	for (int tile = blockIdx.x * TC_WG + wg; tile < tiles; tile += gridDim.x * TC_WG) {
		const int row = tile * 128 + lt;
		const bool valid = row < n;
		float x[GN_IN];
#pragma unroll
		for (int k = 0; k < GN_IN; ++k) x[k] = valid ? samples[(size_t)row * 16 + k] : 0.0f;
		uint4 *h0g = valid ? reinterpret_cast<uint4 *>(B.h0 + (size_t)row * GN_ENC) : nullptr;
		// layer 1: the encoding in two K halves, each also stored for the weight gradients
#pragma unroll
		for (int c = 0; c < 16; ++c) {
			const uint4 v = enc_chunk(x, c);
			*reinterpret_cast<uint4 *>(e0row + c * 128) = v;
			if (h0g) h0g[c] = v;
		}
		if (!sync_issue(0)) break;
		wait_mma();
#pragma unroll
		for (int c = 16; c < 30; ++c) {
			const uint4 v = enc_chunk(x, c);
			*reinterpret_cast<uint4 *>(e1row + (c - 16) * 128) = v;
			if (h0g) h0g[c] = c == 28 ? make_uint4(v.x & 0xffffu, 0u, 0u, 0u) : v;  // the master layout's 0 in column 225
		}
		if (h0g) h0g[30] = h0g[31] = make_uint4(0u, 0u, 0u, 0u);
		if (!sync_issue(1)) break;
		wait_mma();
		// layers 2..5: the hidden activations h1..h4 (stored, their masks kept) feed the next layer
		uint64_t mk[4];
		bool ok = true;
#pragma unroll 1
		for (int layer = 2; layer <= 5 && ok; ++layer) {
			uint4 *hg = valid ? reinterpret_cast<uint4 *>(B.h[layer - 2] + (size_t)row * GN_H) : nullptr;
			mk[layer - 2] = tt_epilogue(tcol + tlane, hrow, hg, true, 0ull, clip);
			if (layer == 2) {
				*reinterpret_cast<uint4 *>(hrow + 8 * 128) = make_uint4(pack_h2(1.f, 0.f), 0u, 0u, 0u);
				*reinterpret_cast<uint4 *>(hrow + 9 * 128) = make_uint4(0u, 0u, 0u, 0u);
			}
			ok = sync_issue(layer);
			if (ok) wait_mma();
		}
		if (!ok) break;
		// the output gradient of the row (K = 48 of the next product: 40 used, then zeros)
		{
			uint32_t r[3][16];
#pragma unroll
			for (int g = 0; g < 3; ++g) tmem_ld16(tcol + 64u + tlane + 16u * g, r[g]);
			tmem_ld_wait();
			float o[5 * GN_LOBES], gr[GN_OUT];
#pragma unroll
			for (int col = 0; col < 5 * GN_LOBES; ++col) o[col] = __uint_as_float(r[col >> 4][col & 15]);
#pragma unroll
			for (int j = 0; j < GN_OUT; ++j) gr[j] = 0.f;
			if (valid) {
				const float *s = samples + (size_t)row * 16;
				const float wt = fminf(s[12] * wscale, wclip);
				lacc += sample_out_grad(o, f3{ s[9], s[10], s[11] }, wt, gr);
			}
			uint4 *dg = valid ? reinterpret_cast<uint4 *>(B.d5 + (size_t)row * GN_OUT) : nullptr;
#pragma unroll
			for (int c = 0; c < GN_OUT / 8; ++c) {
				uint32_t w4[4];
#pragma unroll
				for (int e = 0; e < 4; ++e)
					w4[e] = pack_h2(fminf(fmaxf(gr[8 * c + 2 * e] * lscale, -clip), clip),
						fminf(fmaxf(gr[8 * c + 2 * e + 1] * lscale, -clip), clip));
				const uint4 v = make_uint4(w4[0], w4[1], w4[2], w4[3]);
				*reinterpret_cast<uint4 *>(hrow + c * 128) = v;
				if (dg) dg[c] = v;
			}
		}
		// backward: gradients at h4, h3, h2, h1
#pragma unroll 1
		for (int stage = 6; stage <= 9 && ok; ++stage) {
			ok = sync_issue(stage);
			if (!ok) break;
			wait_mma();
			const int L = 9 - stage;  // the gradient at h(L + 1): B.d[L], masked by mk[L]
			uint4 *dg = valid ? reinterpret_cast<uint4 *>(B.d[L] + (size_t)row * GN_H) : nullptr;
			tt_epilogue(tcol + tlane, hrow, dg, false, mk[L], clip);
		}
		if (!ok) break;
		tc_fence_before();
	}
	named_bar(bar_id, 128);
	if (lt == 0 && fail[wg]) {
		atomicOr(err, (unsigned)ERR_TENSOR_TIMEOUT);
		atomicOr(overflow, 1u);
		mbar_wait(&bar[0], 0, TC_POLL_LIMIT);
		mbar_wait(mbar, phase ^ 1u, TC_POLL_LIMIT);
	}
	for (int o = 16; o > 0; o >>= 1) lacc += __shfl_down_sync(0xffffffffu, lacc, o);
	if ((tid & 31) == 0 && lacc != 0.f) atomicAdd(loss_sum, lacc);
	tc_fence_before();
	__syncthreads();
	if (warp == 0) {
		tc_fence_after();
		tmem_dealloc(tbase, TC_COLS);
	}
}

// dW[o][i] += sum over a chunk of samples of delta[s][o] * h[s][i] on the tensor
// cores (mma.sync m16n8k16: M = outputs, N = inputs, K = samples).  The chunk
// is staged in shared memory WG_SUB samples at a time by asynchronous 16-byte
// copies (the per-sample rows are contiguous) into two alternating buffers, so
// the next sub-chunk arrives while this one is multiplied; the fragments are
// transposing ldmatrix loads of the staged rows.  Each warp keeps the accumulators of its
// output x input tiles in registers across the chunk, so the FP32 atomics
// that merge blocks happen once per chunk: a block takes a chunk of
// n / (WG_BLOCKS_PER_SM x SMs) samples, so a step's atomics do not grow with
// its batch.  The bias gradients come out of the same products: each staged
// input row carries a constant 1 in the column after its last input (the
// row's padding), so the extra input tile's first column accumulates
// sum_s delta[s][o].
constexpr int WG_BLOCKS_PER_SM = 2;  // k_guide_wgrad blocks per SM
constexpr int WG_SUB = 64;           // samples staged at a time
constexpr int WG_PAD = 8;      // halves of padding per staged row (bank spread)
// one staging buffer (the output gradients, then the inputs); two of them alternate
constexpr size_t WG_D_HALVES = (size_t)WG_SUB * (GN_H + WG_PAD), WG_H_HALVES = (size_t)WG_SUB * (GN_ENC + WG_PAD);
constexpr size_t WG_SMEM = 2 * (WG_D_HALVES + WG_H_HALVES) * 2;

// four / two 8 x 8 FP16 matrices from shared memory, transposed (ldmatrix .trans): the rows of
// matrix j come from the addresses of lanes 8j .. 8j + 7 (16-byte aligned rows)
__device__ __forceinline__ void ldsm_x4_trans(uint32_t (&r)[4], const __half *p) {
	const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
	asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];\n"
				 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
				 : "r"(a));
}
__device__ __forceinline__ void ldsm_x2_trans(uint32_t (&r)[2], const __half *p) {
	const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
	asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0, %1}, [%2];\n" : "=r"(r[0]), "=r"(r[1]) : "r"(a));
}

// rows [s, s + WG_SUB) of a [samples][width] FP16 matrix -> shared memory with row stride width + WG_PAD,
// as asynchronous 16-byte copies (cp.async) of the calling thread's share
template <int WIDTH>
__device__ __forceinline__ void stage_rows(const __half *__restrict__ src, int s, __half *dst) {
	constexpr int V = WIDTH / 8;  // 16-byte pieces per row
	for (int e = threadIdx.x; e < WG_SUB * V; e += blockDim.x) {
		const int r = e / V, c = e - r * V;
		const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst + r * (WIDTH + WG_PAD) + 8 * c);
		asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src + (size_t)(s + r) * WIDTH + 8 * c)
					 : "memory");
	}
}
__device__ __forceinline__ void stage_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
// every copy but the most recently committed group of this thread has landed
__device__ __forceinline__ void stage_wait_prior() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// sD[2], sH[2]: two staging buffers; sub-chunk i + 1 is copied in while sub-chunk i is multiplied
template <int OUT_TILES, int IN_TILES, int DW, int HW>
__device__ void wgrad_layer(const __half *__restrict__ D, const __half *__restrict__ H, int s0, int s1,
	float *__restrict__ grad, float *__restrict__ bgrad, int out_limit, unsigned *overflow, __half *const *sD,
	__half *const *sH) {
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
	// input tiles 0..IN_TILES-1 are the weights', tile IN_TILES (the padding columns: 1, 0, ..., 0) the bias's
	constexpr int NT = OUT_TILES * (IN_TILES + 1), PER = (NT + GT / 32 - 1) / (GT / 32);
	constexpr int DS = DW + WG_PAD, HS = HW + WG_PAD;
	static_assert(IN_TILES * 8 == HW && WG_PAD == 8, "one padding tile after the inputs");
	float c[PER][4];
#pragma unroll
	for (int k = 0; k < PER; ++k) c[k][0] = c[k][1] = c[k][2] = c[k][3] = 0.f;
	__syncthreads();  // the previous layer's last products have read both buffers
	for (int e = threadIdx.x; e < 2 * WG_SUB * WG_PAD; e += blockDim.x) {
		const int b = e / (WG_SUB * WG_PAD), r = (e / WG_PAD) % WG_SUB, c = e % WG_PAD;
		sH[b][r * HS + HW + c] = __float2half_rn(c == 0 ? 1.f : 0.f);
	}
	stage_rows<DW>(D, s0, sD[0]);
	stage_rows<HW>(H, s0, sH[0]);
	stage_commit();
	int buf = 0;
	for (int s = s0; s < s1; s += WG_SUB, buf ^= 1) {
		if (s + WG_SUB < s1) {
			stage_rows<DW>(D, s + WG_SUB, sD[buf ^ 1]);
			stage_rows<HW>(H, s + WG_SUB, sH[buf ^ 1]);
		}
		stage_commit();
		stage_wait_prior();
		__syncthreads();  // sub-chunk s has landed for every thread
		const __half *sDb = sD[buf], *sHb = sH[buf];
#pragma unroll
		for (int k = 0; k < PER; ++k) {
			const int tile = warp + k * (GT / 32);
			if (tile >= NT) break;
			const int ot = tile / (IN_TILES + 1), it = tile - ot * (IN_TILES + 1);
#pragma unroll
			for (int kk = 0; kk < WG_SUB; kk += 16) {
				// A (outputs x samples) and B (samples x inputs) fragments by transposing 8 x 8 loads of
				// the sample-major staged rows: lane L addresses row L % 8 of matrix L / 8
				uint32_t a[4], b[2];
				ldsm_x4_trans(a, sDb + (kk + (lane & 7) + ((lane >> 4) & 1) * 8) * DS + ot * 16 + ((lane >> 3) & 1) * 8);
				ldsm_x2_trans(b, sHb + (kk + (lane & 7) + ((lane >> 3) & 1) * 8) * HS + it * 8);
				mma16816(c[k], a, b[0], b[1]);
			}
		}
		__syncthreads();  // every product of sub-chunk s has read its buffer before the next copy into it
	}
#pragma unroll
	for (int k = 0; k < PER; ++k) {
		const int tile = warp + k * (GT / 32);
		if (tile >= NT) break;
		const int ot = tile / (IN_TILES + 1), it = tile - ot * (IN_TILES + 1);
		const int o0 = ot * 16 + g, i0 = it * 8 + 2 * t;
		if (!(isfinite(c[k][0]) && isfinite(c[k][1]) && isfinite(c[k][2]) && isfinite(c[k][3]))) atomicOr(overflow, 1u);
		if (it == IN_TILES) {
			// column HW (t == 0, even half of the pair) is the bias's; the rest multiply zeros
			if (t == 0) {
				if (o0 < out_limit) atomicAdd(&bgrad[o0], c[k][0]);
				if (o0 + 8 < out_limit) atomicAdd(&bgrad[o0 + 8], c[k][2]);
			}
			continue;
		}
		if (o0 < out_limit) atomicAdd(&grad[o0 * HW + i0], c[k][0]), atomicAdd(&grad[o0 * HW + i0 + 1], c[k][1]);
		if (o0 + 8 < out_limit)
			atomicAdd(&grad[(o0 + 8) * HW + i0], c[k][2]), atomicAdd(&grad[(o0 + 8) * HW + i0 + 1], c[k][3]);
	}
}

// chunk: samples per block, a multiple of WG_SUB
__global__ void __launch_bounds__(GT) k_guide_wgrad(GuideTrainBufs B, int n, int chunk, float *__restrict__ grad,
	unsigned *overflow) {
	// samples are padded to a multiple of 16 with zero gradients; a partial last
	// sub-chunk reads rows up to the next multiple of WG_SUB, which the training
	// buffers hold (ensure_train rounds their capacity up)
	extern __shared__ __align__(16) unsigned char wsm[];
	__half *const base = reinterpret_cast<__half *>(wsm);
	__half *const sD[2] = { base, base + WG_D_HALVES };
	__half *const sH[2] = { base + 2 * WG_D_HALVES, base + 2 * WG_D_HALVES + WG_H_HALVES };
	const int s0 = blockIdx.x * chunk, s1 = min(s0 + chunk, n);
	if (s0 >= s1) return;
	wgrad_layer<4, 32, GN_H, GN_ENC>(B.d[0], B.h0, s0, s1, grad + OFF_W1, grad + OFF_B1, GN_H, overflow, sD, sH);
	wgrad_layer<4, 8, GN_H, GN_H>(B.d[1], B.h[0], s0, s1, grad + OFF_W2, grad + OFF_B2, GN_H, overflow, sD, sH);
	wgrad_layer<4, 8, GN_H, GN_H>(B.d[2], B.h[1], s0, s1, grad + OFF_W3, grad + OFF_B3, GN_H, overflow, sD, sH);
	wgrad_layer<4, 8, GN_H, GN_H>(B.d[3], B.h[2], s0, s1, grad + OFF_W4, grad + OFF_B4, GN_H, overflow, sD, sH);
	wgrad_layer<3, 8, GN_OUT, GN_H>(B.d5, B.h[3], s0, s1, grad + OFF_W5, grad + OFF_B5, 40, overflow, sD, sH);
}

__global__ void k_guide_adam(float *__restrict__ P, float *__restrict__ m, float *__restrict__ v,
	const float *__restrict__ grad, float gscale, float lr, float b1, float b2, float eps, float c1, float c2,
	const unsigned *overflow) {
	if (*overflow) return;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < GN_PARAMS; i += gridDim.x * blockDim.x) {
		float gi = grad[i] * gscale;
		float mi = b1 * m[i] + (1.f - b1) * gi;
		float vi = b2 * v[i] + (1.f - b2) * gi * gi;
		m[i] = mi;
		v[i] = vi;
		P[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
	}
}

// n / (sum of the batch's weights) -> *out
// sum of the batch's sample weights into *out (zeroed before), many blocks;
// the forward/backward kernel turns it into the mean-weight scale n / sum
__global__ void k_weight_sum(const float *__restrict__ samples, int n, float *__restrict__ out) {
	__shared__ float red[256];
	float acc = 0.f;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		acc += samples[(size_t)i * 16 + 12];
	red[threadIdx.x] = acc;
	__syncthreads();
	for (int w = 128; w > 0; w >>= 1) {
		if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
		__syncthreads();
	}
	if (threadIdx.x == 0) atomicAdd(out, red[0]);
}

are_status bad(const std::string &m) {
	set_error(m);
	return ARE_ERR_INVALID_ARGUMENT;
}

}  // namespace

size_t guide_infer_smem() { return TC_SMEM; }
GuideNet::~GuideNet() {
	if (stream) cudaStreamSynchronize(stream);
	for (void *p : allocs) cudaFree(p);
	if (train_mem) cudaFree(train_mem);
	if (own_stream && stream) cudaStreamDestroy(stream);
}

are_status GuideNet::init(uint64_t seed) {
	cudaGetDevice(&device);
	cudaDeviceGetAttribute(&n_sms, cudaDevAttrMultiProcessorCount, device);
	if (are_status st = cuda_status(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate")) return st;
	own_stream = true;
	auto alloc = [&](void **p, size_t bytes) -> are_status {
		if (are_status st = cuda_status(cudaMalloc(p, bytes), "cudaMalloc(guide)")) return st;
		allocs.push_back(*p);
		return cuda_status(cudaMemset(*p, 0, bytes), "cudaMemset(guide)");
	};
	if (are_status st = alloc((void **)&params, GN_PARAMS * sizeof(float))) return st;
	if (are_status st = alloc((void **)&adam_m, GN_PARAMS * sizeof(float))) return st;
	if (are_status st = alloc((void **)&adam_v, GN_PARAMS * sizeof(float))) return st;
	if (are_status st = alloc((void **)&grad, (GN_PARAMS + 64) * sizeof(float))) return st;
	if (are_status st = alloc((void **)&tc_img, (TC_HALVES + TCB_HALVES) * sizeof(__half))) return st;
	if (are_status st = alloc((void **)&err_word, 16)) return st;
	if (cudaFuncSetAttribute(k_guide_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)guide_infer_smem()) != cudaSuccess ||
		cudaFuncSetAttribute(k_guide_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WG_SMEM) != cudaSuccess ||
		cudaFuncSetAttribute(k_guide_fwdbwd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TT_SMEM) != cudaSuccess)
		return cuda_status(cudaGetLastError(), "cudaFuncSetAttribute(guide)");
	// seeded He-uniform initialisation on the host (SplitMix64 stream)
	std::vector<float> h(GN_PARAMS, 0.0f);
	uint64_t s = seed;
	auto unif = [&]() {
		uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
		z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
		z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
		z ^= z >> 31;
		return (double)(z >> 11) * 0x1.0p-53;
	};
	auto fill = [&](int off, int rows, int cols, double bound) {
		for (int r = 0; r < rows; ++r)
			for (int c = 0; c < cols; ++c) h[off + r * cols + c] = (float)((2.0 * unif() - 1.0) * bound);
	};
	fill(OFF_W1, GN_H, GN_ENC, std::sqrt(6.0 / 225.0));
	fill(OFF_W2, GN_H, GN_H, std::sqrt(6.0 / GN_H));
	fill(OFF_W3, GN_H, GN_H, std::sqrt(6.0 / GN_H));
	fill(OFF_W4, GN_H, GN_H, std::sqrt(6.0 / GN_H));
	fill(OFF_W5, 40, GN_H, 0.1 * std::sqrt(3.0 / GN_H));
	return set_params(h.data());
}

are_status GuideNet::set_params(const float *host) {
	if (are_status st = cuda_status(cudaMemcpyAsync(params, host, GN_PARAMS * sizeof(float), cudaMemcpyHostToDevice, stream), "H2D params"))
		return st;
	cudaMemsetAsync(adam_m, 0, GN_PARAMS * sizeof(float), stream);
	cudaMemsetAsync(adam_v, 0, GN_PARAMS * sizeof(float), stream);
	steps = 0;
	return pack();
}

are_status GuideNet::pack() {
	k_guide_pack_tc<<<68, 256, 0, stream>>>(params, tc_img);
	return cuda_status(cudaGetLastError(), "k_guide_pack_tc");
}

are_status GuideNet::ensure_train(int n) {
	int cap = (n + WG_SUB - 1) / WG_SUB * WG_SUB;  // k_guide_wgrad stages whole WG_SUB-row blocks
	if (cap <= train_cap) return ARE_OK;
	if (train_mem) cudaFree(train_mem);
	train_mem = nullptr;
	train_cap = 0;
	size_t per = (size_t)(GN_ENC + 8 * GN_H + GN_OUT) * sizeof(__half);
	if (are_status st = cuda_status(cudaMalloc(&train_mem, per * cap + 1024), "cudaMalloc(guide training)")) return st;
	__half *p = (__half *)train_mem;
	bufs.h0 = p, p += (size_t)cap * GN_ENC;
	for (int L = 0; L < 4; ++L) bufs.h[L] = p, p += (size_t)cap * GN_H;
	for (int L = 0; L < 4; ++L) bufs.d[L] = p, p += (size_t)cap * GN_H;
	bufs.d5 = p;
	train_cap = cap;
	return ARE_OK;
}

are_status GuideNet::infer(const float *d_feat, int n, float *d_out, cudaStream_t s, const unsigned *n_dev,
	unsigned *d_err, bool mixture_out) {
	if (mixture_out && (reinterpret_cast<uintptr_t>(d_out) & 15)) return bad("mixture output must be 16-byte aligned");
	if (n <= 0) return ARE_OK;
	// one block per SM (its shared memory allows no second); two 128-row tiles per block in flight
	const int tiles = (n + 127) / 128;
	const int grid = std::max(1, std::min(n_sms, (tiles + TC_WG - 1) / TC_WG));
	k_guide_infer<<<grid, TC_THREADS, guide_infer_smem(), s>>>(tc_img, d_feat, n, n_dev, d_out, d_err ? d_err : err_word,
		mixture_out ? 1 : 0, first_wait_limit);
	return cuda_status(cudaGetLastError(), "k_guide_infer");
}

// samples: n x 16 device floats (features 9, direction 3, weight 1, 3 unused).
// Accumulates the gradient (FP32, times the loss scale) in `grad` and the loss in grad[GN_PARAMS].
are_status GuideNet::gradient(const float *d_samples, int n, float wmean, cudaStream_t s, unsigned *d_err) {
	if (are_status st = ensure_train(n)) return st;
	int np = (n + 15) & ~15;
	const int nz = (n + WG_SUB - 1) / WG_SUB * WG_SUB;
	cudaMemsetAsync(grad, 0, (GN_PARAMS + 64) * sizeof(float), s);
	// rows n..nz-1 of the training buffers are zero (no gradient, no activation)
	if (nz > n) {
		for (int L = 0; L < 4; ++L) {
			cudaMemsetAsync(bufs.d[L] + (size_t)n * GN_H, 0, (size_t)(nz - n) * GN_H * 2, s);
			cudaMemsetAsync(bufs.h[L] + (size_t)n * GN_H, 0, (size_t)(nz - n) * GN_H * 2, s);
		}
		cudaMemsetAsync(bufs.d5 + (size_t)n * GN_OUT, 0, (size_t)(nz - n) * GN_OUT * 2, s);
		cudaMemsetAsync(bufs.h0 + (size_t)n * GN_ENC, 0, (size_t)(nz - n) * GN_ENC * 2, s);
	}
	// wmean < 0: the batch's mean weight is computed on the device
	const float *wdev = nullptr;
	float wscale = wmean > 0.f ? 1.0f / wmean : 0.f;
	if (wmean < 0.f) {
		k_weight_sum<<<std::max(1, std::min(n_sms, (n + 255) / 256)), 256, 0, s>>>(d_samples, n, grad + GN_PARAMS + 2);
		wdev = grad + GN_PARAMS + 2;
	}
	// one block (four warpgroups, one 128-row tile each at a time) per SM at most
	const int tiles = (n + 127) / 128;
	const int grid = std::max(1, std::min(n_sms, (tiles + TC_WG - 1) / TC_WG));
	k_guide_fwdbwd_tc<<<grid, TC_THREADS, TT_SMEM, s>>>(tc_img, d_samples, n, wscale, wdev, weight_clip, loss_scale, bufs,
		grad + GN_PARAMS, (unsigned *)(grad + GN_PARAMS + 1), d_err ? d_err : err_word, first_wait_limit);
	const int blocks = WG_BLOCKS_PER_SM * n_sms;
	const int chunk = std::max(WG_SUB, ((np + blocks - 1) / blocks + WG_SUB - 1) / WG_SUB * WG_SUB);
	k_guide_wgrad<<<(np + chunk - 1) / chunk, GT, WG_SMEM, s>>>(bufs, np, chunk, grad, (unsigned *)(grad + GN_PARAMS + 1));
	return cuda_status(cudaGetLastError(), "guide gradient kernels");
}

are_status GuideNet::train_step(const float *d_samples, int n, float wmean, float lr, cudaStream_t s, unsigned *d_err) {
	if (are_status st = gradient(d_samples, n, wmean, s, d_err)) return st;
	++steps;
	float c1 = 1.f - std::pow(0.9f, (float)steps), c2 = 1.f - std::pow(0.99f, (float)steps);
	k_guide_adam<<<64, 256, 0, s>>>(params, adam_m, adam_v, grad, 1.0f / (loss_scale * (float)n), lr, 0.9f, 0.99f, 1e-8f,
		c1, c2, (const unsigned *)(grad + GN_PARAMS + 1));
	k_guide_pack_tc<<<68, 256, 0, s>>>(params, tc_img);
	return cuda_status(cudaGetLastError(), "guide Adam");
}

}  // namespace are_core

// ---------------------------------------------------------------------------
// C ABI

using are_core::GuideNet;

namespace {
template <class F>
are_status guard(F &&f) {
	try {
		are_core::set_error("");
		return f();
	} catch (const std::bad_alloc &) {
		are_core::set_error("out of host memory");
		return ARE_ERR_OUT_OF_MEMORY;
	} catch (...) {
		are_core::set_error("unexpected exception");
		return ARE_ERR_INTERNAL;
	}
}

// host buffer -> device scratch of the net's stream, freed after use
struct DevTmp {
	void *p = nullptr;
	~DevTmp() {
		if (p) cudaFree(p);
	}
};
}  // namespace

extern "C" {

ARE_API int32_t are_guide_param_count(void) { return are_core::GN_PARAMS; }

ARE_API are_status are_guide_create(uint64_t seed, are_guide **out) {
	return guard([&] {
		if (!out) return are_core::bad("null output");
		*out = nullptr;
		int n = 0;
		if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
			cudaGetLastError();
			are_core::set_error("no CUDA device");
			return ARE_ERR_NO_DEVICE;
		}
		GuideNet *g = new GuideNet();
		if (are_status st = g->init(seed)) {
			delete g;
			return st;
		}
		if (are_status st = are_core::cuda_status(cudaStreamSynchronize(g->stream), "guide init")) {
			delete g;
			return st;
		}
		*out = reinterpret_cast<are_guide *>(g);
		return ARE_OK;
	});
}

ARE_API are_status are_guide_destroy(are_guide *g) {
	return guard([&] {
		delete reinterpret_cast<GuideNet *>(g);
		return ARE_OK;
	});
}

ARE_API are_status are_guide_get_params(are_guide *gh, float *out) {
	return guard([&] {
		GuideNet *g = reinterpret_cast<GuideNet *>(gh);
		if (!g || !out) return are_core::bad("null guide or output");
		cudaMemcpyAsync(out, g->params, are_core::GN_PARAMS * sizeof(float), cudaMemcpyDeviceToHost, g->stream);
		return are_core::cuda_status(cudaStreamSynchronize(g->stream), "guide params");
	});
}

ARE_API are_status are_guide_set_params(are_guide *gh, const float *in) {
	return guard([&] {
		GuideNet *g = reinterpret_cast<GuideNet *>(gh);
		if (!g || !in) return are_core::bad("null guide or input");
		if (are_status st = g->set_params(in)) return st;
		return are_core::cuda_status(cudaStreamSynchronize(g->stream), "guide params");
	});
}

ARE_API are_status are_guide_forward(are_guide *gh, const float *features, int64_t n, float *out) {
	return guard([&] {
		GuideNet *g = reinterpret_cast<GuideNet *>(gh);
		if (!g || (n > 0 && (!features || !out)) || n < 0 || n > (1 << 26)) return are_core::bad("bad guide forward arguments");
		if (n == 0) return ARE_OK;
		DevTmp t;
		// outputs start on a 256-byte boundary after the features (the kernel stores rows as float4)
		size_t fb = ((size_t)n * are_core::GN_IN * 4 + 255) & ~(size_t)255, ob = (size_t)n * are_core::GN_OUT * 4;
		if (are_status st = are_core::cuda_status(cudaMalloc(&t.p, fb + ob), "cudaMalloc")) return st;
		cudaMemcpyAsync(t.p, features, (size_t)n * are_core::GN_IN * 4, cudaMemcpyHostToDevice, g->stream);
		cudaMemsetAsync(g->err_word, 0, 4, g->stream);
		if (are_status st = g->infer((const float *)t.p, (int)n, (float *)((char *)t.p + fb), g->stream)) return st;
		cudaMemcpyAsync(out, (char *)t.p + fb, ob, cudaMemcpyDeviceToHost, g->stream);
		unsigned herr = 0;
		cudaMemcpyAsync(&herr, g->err_word, 4, cudaMemcpyDeviceToHost, g->stream);
		if (are_status st = are_core::cuda_status(cudaStreamSynchronize(g->stream), "guide forward")) return st;
		if (herr) {
			are_core::set_error("guide forward: device error word " + std::to_string(herr));
			return ARE_ERR_KERNEL_TIMEOUT;
		}
		return ARE_OK;
	});
}

ARE_API are_status are_guide_mixture(are_guide *gh, const float *features, int64_t n, float *out) {
	return guard([&] {
		GuideNet *g = reinterpret_cast<GuideNet *>(gh);
		if (!g || (n > 0 && (!features || !out)) || n < 0 || n > (1 << 26)) return are_core::bad("bad guide mixture arguments");
		if (n == 0) return ARE_OK;
		DevTmp t;
		size_t fb = ((size_t)n * are_core::GN_IN * 4 + 255) & ~(size_t)255, ob = (size_t)n * are_core::GN_OUT * 4;
		if (are_status st = are_core::cuda_status(cudaMalloc(&t.p, fb + ob), "cudaMalloc")) return st;
		cudaMemcpyAsync(t.p, features, (size_t)n * are_core::GN_IN * 4, cudaMemcpyHostToDevice, g->stream);
		cudaMemsetAsync(g->err_word, 0, 4, g->stream);
		if (are_status st = g->infer((const float *)t.p, (int)n, (float *)((char *)t.p + fb), g->stream, nullptr, nullptr, true))
			return st;
		cudaMemcpyAsync(out, (char *)t.p + fb, ob, cudaMemcpyDeviceToHost, g->stream);
		unsigned herr = 0;
		cudaMemcpyAsync(&herr, g->err_word, 4, cudaMemcpyDeviceToHost, g->stream);
		if (are_status st = are_core::cuda_status(cudaStreamSynchronize(g->stream), "guide mixture")) return st;
		if (herr) {
			are_core::set_error("guide mixture: device error word " + std::to_string(herr));
			return ARE_ERR_KERNEL_TIMEOUT;
		}
		return ARE_OK;
	});
}

// samples: n x 13 host floats (features 9, direction 3, weight 1)
static are_status upload_samples(GuideNet *g, const float *samples, int64_t n, DevTmp &t, float &wmean) {
	std::vector<float> s16((size_t)n * 16, 0.0f);
	double ws = 0.0;
	for (int64_t i = 0; i < n; ++i) {
		std::memcpy(&s16[(size_t)i * 16], samples + 13 * i, 13 * sizeof(float));
		ws += samples[13 * i + 12];
	}
	wmean = n > 0 ? (float)(ws / (double)n) : 0.f;
	if (are_status st = are_core::cuda_status(cudaMalloc(&t.p, s16.size() * 4), "cudaMalloc")) return st;
	cudaMemcpyAsync(t.p, s16.data(), s16.size() * 4, cudaMemcpyHostToDevice, g->stream);
	return are_core::cuda_status(cudaStreamSynchronize(g->stream), "upload samples");
}

ARE_API are_status are_guide_gradient(are_guide *gh, const float *samples, int64_t n, float *loss, float *grad) {
	return guard([&] {
		GuideNet *g = reinterpret_cast<GuideNet *>(gh);
		if (!g || !samples || !grad || n <= 0 || n > (1 << 22)) return are_core::bad("bad guide gradient arguments");
		DevTmp t;
		float wmean = 0.f;
		if (are_status st = upload_samples(g, samples, n, t, wmean)) return st;
		cudaMemsetAsync(g->err_word, 0, 4, g->stream);
		if (are_status st = g->gradient((const float *)t.p, (int)n, wmean, g->stream)) return st;
		std::vector<float> h(are_core::GN_PARAMS + 2);
		cudaMemcpyAsync(h.data(), g->grad, h.size() * 4, cudaMemcpyDeviceToHost, g->stream);
		unsigned herr = 0;
		cudaMemcpyAsync(&herr, g->err_word, 4, cudaMemcpyDeviceToHost, g->stream);
		if (are_status st = are_core::cuda_status(cudaStreamSynchronize(g->stream), "guide gradient")) return st;
		if (herr) {
			are_core::set_error("guide gradient: device error word " + std::to_string(herr));
			return ARE_ERR_KERNEL_TIMEOUT;
		}
		float s = 1.0f / (g->loss_scale * (float)n);
		for (int i = 0; i < are_core::GN_PARAMS; ++i) grad[i] = h[i] * s;
		if (loss) *loss = h[are_core::GN_PARAMS] / (float)n;
		unsigned of;
		std::memcpy(&of, &h[are_core::GN_PARAMS + 1], 4);
		if (of) {
			are_core::set_error("FP16 overflow in the backward pass");
			return ARE_ERR_INTERNAL;
		}
		return ARE_OK;
	});
}

ARE_API are_status are_render_guided(are_scene *scene, are_guide *guide, const are_camera *camera,
	const are_render_params *params, const are_guide_params *guide_params, float *rgb_out, float *var_out,
	are_render_stats *stats) {
	return guard([&] {
		return are_core::render_guided(scene, reinterpret_cast<GuideNet *>(guide), camera, params, guide_params, rgb_out,
			var_out, stats);
	});
}

ARE_API int32_t are_guide_loss_history(are_guide *gh, float *out, int32_t max) {
	GuideNet *g = reinterpret_cast<GuideNet *>(gh);
	if (!g || !out || max <= 0) return 0;
	int32_t n = (int32_t)std::min<size_t>((size_t)max, g->loss_log.size());
	std::memcpy(out, g->loss_log.data() + (g->loss_log.size() - n), n * sizeof(float));
	return n;
}

ARE_API are_status are_guide_set_wait_limit(are_guide *gh, int32_t polls) {
	return guard([&] {
		GuideNet *g = reinterpret_cast<GuideNet *>(gh);
		if (!g) return are_core::bad("null guide");
		g->first_wait_limit = polls < 0 ? 0xffffffffu : (uint32_t)polls;
		return ARE_OK;
	});
}

ARE_API are_status are_guide_train(are_guide *gh, const float *samples, int64_t n, float lr, float *loss) {
	return guard([&] {
		GuideNet *g = reinterpret_cast<GuideNet *>(gh);
		if (!g || !samples || n <= 0 || n > (1 << 22) || !(lr > 0.f)) return are_core::bad("bad guide train arguments");
		DevTmp t;
		float wmean = 0.f;
		if (are_status st = upload_samples(g, samples, n, t, wmean)) return st;
		cudaMemsetAsync(g->err_word, 0, 4, g->stream);
		if (are_status st = g->train_step((const float *)t.p, (int)n, wmean, lr, g->stream)) return st;
		float l = 0.f;
		unsigned herr = 0;
		cudaMemcpyAsync(&l, g->grad + are_core::GN_PARAMS, 4, cudaMemcpyDeviceToHost, g->stream);
		cudaMemcpyAsync(&herr, g->err_word, 4, cudaMemcpyDeviceToHost, g->stream);
		if (are_status st = are_core::cuda_status(cudaStreamSynchronize(g->stream), "guide train")) return st;
		if (herr) {
			// the step's gradients are incomplete: the kernel flagged them, and Adam left the weights as they were
			are_core::set_error("guide train: device error word " + std::to_string(herr) + "; the step was skipped");
			return ARE_ERR_KERNEL_TIMEOUT;
		}
		if (loss) *loss = l / (float)n;
		return ARE_OK;
	});
}

}  // extern "C"
