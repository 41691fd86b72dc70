// guide.cuh — the path-guiding network on the device: layout constants,
// input encoding, the von Mises-Fisher mixture it outputs, and the tensor-core
// building blocks of its fused forward/backward kernels.
//
// The network and its loss are specified in oracle/orc_guide.c (FP64); the
// device computes the same in FP16 on the tensor cores with FP32
// accumulation: the forward and backward passes fused per 128-row tile on the
// 5th-generation tensor cores (tcgen05, guide.cu), in the manner of the fully
// fused MLPs of Mueller et al., "Real-time Neural Radiance Caching", 2021; the
// weight gradients reduce over the batch with mma.sync.m16n8k16; FP32 master
// weights and Adam.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "shade.cuh"
#include "traverse.cuh"

namespace are_core {

constexpr int GN_IN = 9, GN_ENC = 256, GN_H = 64, GN_OUT = 48, GN_LOBES = 8;
// flat FP32 parameters, rows [out][in] (as the oracle)
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + GN_H * GN_ENC;
constexpr int OFF_W2 = OFF_B1 + GN_H, OFF_B2 = OFF_W2 + GN_H * GN_H;
constexpr int OFF_W3 = OFF_B2 + GN_H, OFF_B3 = OFF_W3 + GN_H * GN_H;
constexpr int OFF_W4 = OFF_B3 + GN_H, OFF_B4 = OFF_W4 + GN_H * GN_H;
constexpr int OFF_W5 = OFF_B4 + GN_H, OFF_B5 = OFF_W5 + GN_OUT * GN_H;
constexpr int GN_PARAMS = OFF_B5 + GN_OUT;

// Weight image of the tcgen05 kernels (halves): each layer's
// [out][in] matrix in the canonical no-swizzle K-major layout of the tensor
// core (core matrices of 8 rows x 8 halves, 64 halves each; the core matrices
// of one 8-row group adjacent in K).  The biases ride in the GEMMs: layer 1
// keeps K = 240 (encoding columns 240..255 are always zero) and takes its
// bias in column 225, whose input is the constant 1 (the encoding is zero
// there); the other layers get K = 80, column 64 the bias against a constant
// 1 input, columns 65..79 zero.
constexpr int TC_K1 = 240;
constexpr int TC_KH = 80;
constexpr int TC_ONE1 = 225;                    // constant-1 input column of layer 1
constexpr int TC_W1 = 0;                        // [64][240]
constexpr int TC_W2 = TC_W1 + GN_H * TC_K1;     // [64][80]
constexpr int TC_W3 = TC_W2 + GN_H * TC_KH;
constexpr int TC_W4 = TC_W3 + GN_H * TC_KH;
constexpr int TC_W5 = TC_W4 + GN_H * TC_KH;     // [48][80]
constexpr int TC_HALVES = TC_W5 + GN_OUT * TC_KH;
// index of element (row, k) of a K-column matrix in that layout
__host__ __device__ constexpr int tc_index(int row, int k, int K) {
	return (row >> 3) * (K * 8) + (k >> 3) * 64 + (row & 7) * 8 + (k & 7);
}
// The backward image, right after the forward one in the same buffer: the
// transposed weights W^T ([in][out], K = the layer's outputs) of layers 5..2
// in the same layout, whose product with a row's gradient at a layer's output
// is the gradient at its input.  Layer 5 keeps K = 48 (outputs 40..47 zero).
constexpr int TCB_K5 = GN_OUT;
constexpr int TCB_W5 = 0;                       // [64][48]
constexpr int TCB_W4 = TCB_W5 + GN_H * TCB_K5;  // [64][64]
constexpr int TCB_W3 = TCB_W4 + GN_H * GN_H;
constexpr int TCB_W2 = TCB_W3 + GN_H * GN_H;
constexpr int TCB_HALVES = TCB_W2 + GN_H * GN_H;

// features of a shading point: position scaled to the scene box, normal, outgoing direction
struct GuideBox {
	float lo[3], inv_ext[3];
};

__device__ __forceinline__ void guide_features(const GuideBox &B, f3 p, f3 n, f3 wo, float *x) {
	x[0] = 2.0f * (p.x - B.lo[0]) * B.inv_ext[0] - 1.0f;
	x[1] = 2.0f * (p.y - B.lo[1]) * B.inv_ext[1] - 1.0f;
	x[2] = 2.0f * (p.z - B.lo[2]) * B.inv_ext[2] - 1.0f;
	x[3] = n.x, x[4] = n.y, x[5] = n.z;
	x[6] = wo.x, x[7] = wo.y, x[8] = wo.z;
}

// The input encoding is 128 pairs of FP16 values: pair 12 i + k (i < 9,
// k < 12) is (sin, cos)(pi 2^k x_i), pairs 108..111 the raw features x_0..x_7
// two by two, pair 112 (x_8, 0), the rest zero (guide.cu: enc_chunk).

__device__ __forceinline__ uint32_t h2u(__half2 h) { return *reinterpret_cast<uint32_t *>(&h); }
__device__ __forceinline__ __half2 u2h(uint32_t u) { return *reinterpret_cast<__half2 *>(&u); }

__device__ __forceinline__ void mma16816(float *c, const uint32_t *a, uint32_t b0, uint32_t b1) {
	asm volatile(
		"mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
		"{%0,%1,%2,%3};\n"
		: "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
		: "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// ---- the vMF mixture -------------------------------------------------------

struct Mixture {
	f3 mu[GN_LOBES];
	float kappa[GN_LOBES], pi[GN_LOBES], norm[GN_LOBES];  // norm = kappa / (2 pi (1 - e^-2kappa))
};

__device__ __forceinline__ float softplusf(float x) { return x > 20.f ? x : log1pf(__expf(x)); }

__device__ __forceinline__ void to_mixture(const float *o, Mixture &m) {
	float mx = -1e30f;
#pragma unroll
	for (int l = 0; l < GN_LOBES; ++l) mx = fmaxf(mx, o[5 * l + 4]);
	float z = 0.f;
#pragma unroll
	for (int l = 0; l < GN_LOBES; ++l) {
		float len = sqrtf(o[5 * l] * o[5 * l] + o[5 * l + 1] * o[5 * l + 1] + o[5 * l + 2] * o[5 * l + 2]) + 1e-6f;
		m.mu[l] = f3{ o[5 * l] / len, o[5 * l + 1] / len, o[5 * l + 2] / len };
		float k = softplusf(o[5 * l + 3]) + 0.05f;
		m.kappa[l] = k;
		m.norm[l] = k / (6.28318530717958647692f * -expm1f(-2.f * k));
		m.pi[l] = __expf(o[5 * l + 4] - mx);
		z += m.pi[l];
	}
	float iz = 1.f / z;
#pragma unroll
	for (int l = 0; l < GN_LOBES; ++l) m.pi[l] *= iz;
}

// The packed form the inference kernel writes for rendering, 48 floats per
// row: lobe l's (mu.x, mu.y, mu.z, kappa) at 4 l, then (pi_l, norm_l) at
// 32 + 2 l.  The mean directions are stored at unit length (the network's
// spec divides by |m| + 1e-6): the sampler draws around a unit axis, so the
// density the renderer reports is exactly the density it samples.  Computed
// with the special-function unit's exp/log and reciprocal square roots: the
// renderer needs a density and a sampler that agree with each other (both
// read these stored values), not the oracle's last bit.
__device__ __forceinline__ void pack_mixture_fast(const float *o, float *pk) {
	float mx = -1e30f;
#pragma unroll
	for (int l = 0; l < GN_LOBES; ++l) mx = fmaxf(mx, o[5 * l + 4]);
	float pi[GN_LOBES], z = 0.f;
#pragma unroll
	for (int l = 0; l < GN_LOBES; ++l) {
		const float ax = o[5 * l], ay = o[5 * l + 1], az = o[5 * l + 2];
		const float len2 = ax * ax + ay * ay + az * az;
		float ux = 0.f, uy = 0.f, uz = 1.f;
		if (len2 > 0.f) {
			const float r = rsqrtf(len2);
			ux = ax * r, uy = ay * r, uz = az * r;
			const float r2 = rsqrtf(ux * ux + uy * uy + uz * uz);  // a second pass: unit within an ulp or two
			ux *= r2, uy *= r2, uz *= r2;
		}
		const float x = o[5 * l + 3];
		const float k = (x > 15.f ? x : __logf(1.f + __expf(x))) + 0.05f;
		pk[4 * l] = ux, pk[4 * l + 1] = uy, pk[4 * l + 2] = uz, pk[4 * l + 3] = k;
		pk[33 + 2 * l] = k * __frcp_rn(6.28318530717958647692f * (1.f - __expf(-2.f * k)));
		pi[l] = __expf(o[5 * l + 4] - mx);
		z += pi[l];
	}
	const float iz = __frcp_rn(z);
#pragma unroll
	for (int l = 0; l < GN_LOBES; ++l) pk[32 + 2 * l] = pi[l] * iz;
}

// Density and sampling of the packed mixture (pack_mixture_fast), read lobe by
// lobe from memory so a shading thread does not hold the whole mixture in
// registers.  Sampling picks a lobe by its weight, then draws the vMF sample
// of W. Jakob's stable form, cos(theta) = 1 + log(u1 + (1 - u1) e^-2kappa) /
// kappa, azimuth 2 pi u2; the density is sum_l pi_l norm_l e^(kappa_l (mu_l.w - 1)).
__device__ __forceinline__ float packed_pdf(const float *__restrict__ m, f3 w) {
	float q = 0.f;
#pragma unroll 2
	for (int l = 0; l < GN_LOBES; ++l) {
		const float4 a = reinterpret_cast<const float4 *>(m)[l];
		const float2 b = reinterpret_cast<const float2 *>(m + 32)[l];
		q += b.x * b.y * __expf(a.w * ((a.x * w.x + a.y * w.y + a.z * w.z) - 1.f));
	}
	return q;
}

__device__ __forceinline__ f3 packed_sample(const float *__restrict__ m, float u0, float u1, float u2) {
	// the first lobe whose cumulative weight exceeds u0 (the last if rounding leaves u0 above the total)
	int sel = GN_LOBES - 1;
	float acc = 0.f;
#pragma unroll
	for (int l = 0; l < GN_LOBES - 1; ++l) {
		acc += m[32 + 2 * l];
		if (sel == GN_LOBES - 1 && u0 < acc) sel = l;
	}
	const float4 a = reinterpret_cast<const float4 *>(m)[sel];
	const float k = a.w;
	float w = 1.f + logf(u1 + (1.f - u1) * __expf(-2.f * k)) / k;
	w = fminf(fmaxf(w, -1.f), 1.f);
	float r = sqrtf(fmaxf(0.f, 1.f - w * w));
	float s, c;
	sincospif(2.f * u2, &s, &c);
	const f3 z = f3{ a.x, a.y, a.z };
	const f3 up = fabsf(z.z) < 0.999f ? f3{ 0.f, 0.f, 1.f } : f3{ 1.f, 0.f, 0.f };
	const f3 x = norm(cross(z, up));
	const f3 y = cross(z, x);
	return norm(add(add(scl(x, r * c), scl(y, r * s)), scl(z, w)));
}

}  // namespace are_core
