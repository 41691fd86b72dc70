// traverse.cuh — closest-hit queries on the device.
//
// Primitive tests use __fadd_rn/__fsub_rn/__fmul_rn/__fdiv_rn/__fsqrt_rn so
// no multiply-add is ever contracted: each operation rounds exactly as the
// reference's FP32 code does on the host (rt.cpp:123-138 for the triangle
// test), which makes closest-hit ids, t, u and v bit-identical to the CPU
// restatement.  Box tests are only culling and are free to use FMA: node
// boxes are padded (core.h) so they never reject a primitive hit.
#pragma once

#include <cuda_runtime.h>

#include "core.h"

namespace are_core {

struct f3 {
	float x, y, z;
};

__device__ __forceinline__ f3 mk3(float x, float y, float z) { return f3{ x, y, z }; }
__device__ __forceinline__ f3 ld3(float4 v) { return f3{ v.x, v.y, v.z }; }
__device__ __forceinline__ f3 rsub(f3 a, f3 b) {
	return f3{ __fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z) };
}
__device__ __forceinline__ f3 radd(f3 a, f3 b) {
	return f3{ __fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z) };
}
__device__ __forceinline__ f3 rscl(f3 a, float s) {
	return f3{ __fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s) };
}
// ((ax*bx + ay*by) + az*bz), each step rounded
__device__ __forceinline__ float rdot(f3 a, f3 b) {
	return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ f3 rcross(f3 a, f3 b) {
	return f3{ __fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)), __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
		__fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)) };
}

// Sphere: discriminant a (r^2 - |l|^2) with l = f + (b/a) d (Haines et al.,
// Ray Tracing Gems 2019, ch. 7), roots c/q and q/a.  New primitive.
__device__ __forceinline__ bool hit_sphere(float4 s0, f3 o, f3 d, float tmin, float tmax, float &tout) {
	f3 c = ld3(s0);
	float r = s0.w;
	f3 f = rsub(o, c);
	float a = rdot(d, d);
	float b = -rdot(f, d);
	float s = __fdiv_rn(b, a);
	f3 l = radd(f, rscl(d, s));
	float r2 = __fmul_rn(r, r);
	float disc = __fmul_rn(a, __fsub_rn(r2, rdot(l, l)));
	if (!(disc >= 0.0f)) return false;
	float cc = __fsub_rn(rdot(f, f), r2);
	float sq = __fsqrt_rn(disc);
	float q = __fadd_rn(b, copysignf(sq, b));
	float t0 = __fdiv_rn(cc, q);
	float t1 = __fdiv_rn(q, a);
	float tn = t0 < t1 ? t0 : t1;
	float tf = t0 < t1 ? t1 : t0;
	if (tn > tmin && tn < tmax) {
		tout = tn;
		return true;
	}
	if (tf > tmin && tf < tmax) {
		tout = tf;
		return true;
	}
	return false;
}

// Quad (Q, u, v): plane hit (src/basic/plane.cpp:13-27), then the planar
// coordinates alpha, beta in [0,1]^2.  New primitive.
__device__ __forceinline__ bool quad_t_reject(float num, float denom, float tmin, float tcut);
__device__ __forceinline__ bool coord_reject(float na, float nn);
__device__ __forceinline__ bool coord_inside(float na, float nn);

__device__ __forceinline__ bool hit_quad(f3 Q, f3 u, f3 v, f3 o, f3 d, float tmin, float tmax, float tcut,
	float &tout, float &uo, float &vo) {
	f3 n = rcross(u, v);
	float denom = rdot(n, d);
	if (denom == 0.0f) return false;
	float num = rdot(n, rsub(Q, o));
	if (quad_t_reject(num, denom, tmin, tcut)) return false;
	float t = __fdiv_rn(num, denom);
	if (!(t > tmin && t < tmax)) return false;
	f3 p = rsub(radd(o, rscl(d, t)), Q);
	float nn = rdot(n, n);
	float na = rdot(n, rcross(p, v));
	if (!coord_inside(na, nn)) return false;
	float nb = rdot(n, rcross(u, p));
	if (!coord_inside(nb, nn)) return false;
	float al = __fdiv_rn(na, nn);
	float be = __fdiv_rn(nb, nn);
	tout = t;
	uo = al;
	vo = be;
	return true;
}

// Quad with the normal n = u x v and nn = n.n precomputed by the same rounded
// operations as hit_quad, so the result is bit-identical to hit_quad's.
//
// Two early rejections skip the divisions without changing any answer, both
// for tmin >= 0 only (then every accepted t is positive):
//  * t = num/denom is <= 0 whenever num and denom differ in sign or num is 0,
//    so such planes are behind the ray;
//  * with lim = tcut * |denom| * (1 + 2^-19) a normal float, |num| > lim means
//    the correctly rounded (positive) quotient exceeds tcut (the best hit so
//    far), so the quad cannot win; ties (t == tcut) are never rejected.
// With tmin < 0 a hit may lie behind the origin and every plane is divided.
__device__ __forceinline__ bool quad_t_reject(float num, float denom, float tmin, float tcut) {
	if (!(tmin >= 0.0f)) return false;
	if (!((num > 0.0f) == (denom > 0.0f) && num != 0.0f)) return true;
	float lim = tcut * fabsf(denom) * 1.000002f;
	return lim >= 1.17549435e-38f && fabsf(num) > lim;
}

// With nn >= 2^-60 the rounded quotient q = na / nn lies outside [0, 1]
// whenever na < -nn 2^-60 (then q < -2^-60) or na > fl(nn (1 + 2^-21)) (then
// q > 1 + 2^-22, which rounds above 1); both thresholds are normal floats, the
// first exact.  Those coordinates are rejected without dividing; borderline
// cases and tiny quads divide, so no answer changes.
__device__ __forceinline__ bool coord_reject(float na, float nn) {
	if (!(na == na)) return true;
	if (!(nn >= 8.67361738e-19f)) return false;
	return na < -nn * 8.67361738e-19f || na > nn * 1.00000047683716f;
}

// The same decision as fl(na / nn) in [0, 1] (nn > 0), dividing only in the
// borderline bands: 0 <= na <= fl(nn (1 - 2^-23)) means q <= 1 - 2^-24, which
// rounds to at most 1, so it is inside; coord_reject covers the clear outside.
__device__ __forceinline__ bool coord_inside(float na, float nn) {
	if (coord_reject(na, nn)) return false;
	if (nn >= 8.67361738e-19f && na >= 0.0f && na <= nn * 0.99999988079071f) return true;
	float q = __fdiv_rn(na, nn);
	return q >= 0.0f && q <= 1.0f;
}

__device__ __forceinline__ bool hit_quad_pre(f3 Q, f3 u, f3 v, f3 n, float nn, f3 o, f3 d, float tmin, float tmax,
	float tcut, float &tout, float &uo, float &vo) {
	float denom = rdot(n, d);
	if (denom == 0.0f) return false;
	float num = rdot(n, rsub(Q, o));
	if (quad_t_reject(num, denom, tmin, tcut)) return false;
	float t = __fdiv_rn(num, denom);
	if (!(t > tmin && t < tmax)) return false;
	f3 p = rsub(radd(o, rscl(d, t)), Q);
	float na = rdot(n, rcross(p, v));
	if (!coord_inside(na, nn)) return false;
	float nb = rdot(n, rcross(u, p));
	if (!coord_inside(nb, nn)) return false;
	// uo/vo carry the numerators; the caller divides by nn for the final hit only
	tout = t;
	uo = na;
	vo = nb;
	return true;
}

// Triangle, Möller–Trumbore exactly as rt.cpp Tri::intersect (rt.cpp:123-138),
// with EPS = 1e-5f (rt.cpp:15) as the parallel threshold and the reference's
// NaN-passing comparisons.
__device__ __forceinline__ bool hit_tri_mt(f3 v0, f3 v1, f3 v2, f3 o, f3 d, float tmin, float tmax, float &tout,
	float &uo, float &vo) {
	f3 e1 = rsub(v1, v0), e2 = rsub(v2, v0), h = rcross(d, e2), s = rsub(o, v0);
	float a = rdot(e1, h);
	if (fabsf(a) < 1e-5f) return false;
	float f = __frcp_rn(a);
	float u = __fmul_rn(f, rdot(s, h));
	if (u < 0.0f || u > 1.0f) return false;
	f3 q = rcross(s, e1);
	float v = __fmul_rn(f, rdot(d, q));
	if (v < 0.0f || __fadd_rn(u, v) > 1.0f) return false;
	float t = __fmul_rn(f, rdot(e2, q));
	if (!(t > tmin && t < tmax)) return false;
	tout = t;
	uo = u;
	vo = v;
	return true;
}

// Triangle, watertight (Woop, Benthin, Wald, JCGT 2013).
__device__ __forceinline__ bool hit_tri_wt(f3 v0, f3 v1, f3 v2, f3 o, f3 d, float tmin, float tmax, float &tout,
	float &uo, float &vo) {
	float dd[3] = { d.x, d.y, d.z };
	int kz = 0;
	if (fabsf(dd[1]) > fabsf(dd[kz])) kz = 1;
	if (fabsf(dd[2]) > fabsf(dd[kz])) kz = 2;
	int kx = kz == 2 ? 0 : kz + 1;
	int ky = kx == 2 ? 0 : kx + 1;
	if (dd[kz] < 0.0f) {
		int tmp = kx;
		kx = ky;
		ky = tmp;
	}
	float dkz = dd[kz];
	float Sx = __fdiv_rn(dd[kx], dkz), Sy = __fdiv_rn(dd[ky], dkz), Sz = __frcp_rn(dkz);
	f3 A = rsub(v0, o), B = rsub(v1, o), C = rsub(v2, o);
	float Aa[3] = { A.x, A.y, A.z }, Ba[3] = { B.x, B.y, B.z }, Ca[3] = { C.x, C.y, C.z };
	float Ax = __fsub_rn(Aa[kx], __fmul_rn(Sx, Aa[kz])), Ay = __fsub_rn(Aa[ky], __fmul_rn(Sy, Aa[kz]));
	float Bx = __fsub_rn(Ba[kx], __fmul_rn(Sx, Ba[kz])), By = __fsub_rn(Ba[ky], __fmul_rn(Sy, Ba[kz]));
	float Cx = __fsub_rn(Ca[kx], __fmul_rn(Sx, Ca[kz])), Cy = __fsub_rn(Ca[ky], __fmul_rn(Sy, Ca[kz]));
	float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
	float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
	float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
	if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
	float det = __fadd_rn(__fadd_rn(U, V), W);
	if (det == 0.0f) return false;
	float Az = __fmul_rn(Sz, Aa[kz]), Bz = __fmul_rn(Sz, Ba[kz]), Cz = __fmul_rn(Sz, Ca[kz]);
	float T = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
	float rcp = __frcp_rn(det);
	float t = __fmul_rn(T, rcp);
	if (!(t > tmin && t < tmax)) return false;
	tout = t;
	uo = __fmul_rn(V, rcp);
	vo = __fmul_rn(W, rcp);
	return true;
}

struct Hit {
	float t;
	int32_t leaf;  // leaf-order primitive index, -1 on a miss
	int32_t gid;   // global id
	float u, v;
};

__device__ __forceinline__ float4 ldg4(const float4 *p) { return __ldg(p); }

// Stages the first SMEM_NODES BVH nodes (the breadth-first top levels) into
// shared memory.
__device__ __forceinline__ void stage_nodes(const DevScene &S, float4 *snodes, int &n_snodes) {
	n_snodes = min(S.n_nodes, SMEM_NODES);
	for (int i = threadIdx.x; i < 2 * n_snodes; i += blockDim.x) snodes[i] = __ldg(S.nodes + i);
	__syncthreads();
}

// Stages the primitives of a scene with at most LINEAR_MAX of them into
// shared memory: per primitive [0..2] the leaf-order record (global id in
// [1].w), [3] the quad normal u x v and its squared length; then, from
// sp[4 LINEAR_MAX] on, the BVH's leaf boxes (2 float4 each, node format).
__device__ __forceinline__ void stage_prims(const DevScene &S, float4 *sp) {
	for (int l = threadIdx.x; l < 2 * S.n_leaves; l += blockDim.x) sp[4 * LINEAR_MAX + l] = __ldg(S.leaves + l);
	for (int j = threadIdx.x; j < S.n_prims; j += blockDim.x) {
		const float4 *P = S.prims + 3 * (size_t)j;
		float4 p0 = __ldg(P), p1 = __ldg(P + 1), p2 = __ldg(P + 2);
		p1.w = __int_as_float(__ldg(S.prim_gid + j));
		float4 p3 = make_float4(0.f, 0.f, 0.f, 0.f);
		if (p0.w == PRIM_TAG_QUAD) {
			f3 n = rcross(ld3(p1), ld3(p2));
			p3 = make_float4(n.x, n.y, n.z, rdot(n, n));
		}
		sp[4 * j] = p0, sp[4 * j + 1] = p1, sp[4 * j + 2] = p2, sp[4 * j + 3] = p3;
	}
}

// Closest hit by a linear scan of the staged primitives: rt.cpp's own
// strategy (rt.cpp:209-218).  Every lane of a warp walks the same primitive
// at the same time, so the loads are shared-memory broadcasts and the control
// flow only diverges inside a primitive test.  Same answer as closest_hit.
__device__ __forceinline__ Hit closest_hit_linear(const float4 *__restrict__ sp, int n_leaves, int tri_wt, f3 o, f3 d,
	float tmin, float tmax) {
	Hit best;
	best.t = __int_as_float(0x7f800000);
	best.leaf = -1;
	best.gid = 0x7fffffff;
	best.u = best.v = 0.0f;
	float dx = d.x != 0.0f ? d.x : copysignf(1e-20f, d.x);
	float dy = d.y != 0.0f ? d.y : copysignf(1e-20f, d.y);
	float dz = d.z != 0.0f ? d.z : copysignf(1e-20f, d.z);
	float ix = __frcp_rn(dx), iy = __frcp_rn(dy), iz = __frcp_rn(dz);
	float ox = -o.x * ix, oy = -o.y * iy, oz = -o.z * iz;
	float best_nn = 0.0f;  // quads report numerators; divided once for the final hit
	for (int l = 0; l < n_leaves; ++l) {
		// the leaf's padded box (culling only), then its primitives
		float4 b0 = sp[4 * LINEAR_MAX + 2 * l], b1 = sp[4 * LINEAR_MAX + 2 * l + 1];
		float t0x = fmaf(b0.x, ix, ox), t1x = fmaf(b1.x, ix, ox);
		float t0y = fmaf(b0.y, iy, oy), t1y = fmaf(b1.y, iy, oy);
		float t0z = fmaf(b0.z, iz, oz), t1z = fmaf(b1.z, iz, oz);
		float lo = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
		float hi = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)),
			fminf(fmaxf(t0z, t1z), fminf(best.t, tmax) * 1.0000039f));
		if (!(lo <= hi)) continue;
		const int first = __float_as_int(b0.w), end = first + __float_as_int(b1.w);
	for (int j = first; j < end; ++j) {
		float4 p0 = sp[4 * j];
		float t, u = 0.0f, v = 0.0f;
		bool h;
		float4 p1 = sp[4 * j + 1];
		float qnn = 0.0f;
		if (p0.w > 0.0f) {
			h = hit_sphere(p0, o, d, tmin, tmax, t);
		} else {
			float4 p2 = sp[4 * j + 2];
			if (p0.w == PRIM_TAG_QUAD) {
				float4 p3 = sp[4 * j + 3];
				qnn = p3.w;
				h = hit_quad_pre(ld3(p0), ld3(p1), ld3(p2), ld3(p3), p3.w, o, d, tmin, tmax, best.t, t, u, v);
			} else if (tri_wt) {
				h = hit_tri_wt(ld3(p0), ld3(p1), ld3(p2), o, d, tmin, tmax, t, u, v);
			} else {
				h = hit_tri_mt(ld3(p0), ld3(p1), ld3(p2), o, d, tmin, tmax, t, u, v);
			}
		}
		if (h) {
			int32_t gid = __float_as_int(p1.w);
			if (t < best.t || (t == best.t && gid < best.gid)) {
				best.t = t;
				best.leaf = j;
				best.gid = gid;
				best.u = u;
				best.v = v;
				best_nn = qnn;
			}
		}
	}
	}
	if (best_nn != 0.0f) {
		best.u = __fdiv_rn(best.u, best_nn);
		best.v = __fdiv_rn(best.v, best_nn);
	}
	return best;
}

// ---------------------------------------------------------------------------
// Warp-cooperative linear scan.  In closest_hit_linear every lane tests every
// primitive whose leaf box it enters, so a warp issues the union of its
// lanes' tests with a third of the lanes busy.  Here the warp first finds, for
// all lanes together and one primitive at a time, the (ray, primitive) pairs
// that can hit — the leaf box and, for quads, the side of the plane the ray
// moves toward: exactly closest_hit_linear's own first rejections — and
// queues them in a shared-memory ring; full rounds of 32 pairs then run the
// complete tests with every lane busy, each lane on another lane's ray.  A
// ray's best hit is the minimum of the 64-bit key (t bits << 32 | global id):
// t is finite and > tmin >= 0 for every accepted hit, so the key orders like
// closest_hit_linear's (t, global id) rule and the answer is the same bits.

struct WarpHitScratch {
	unsigned long long key[32];  // per lane: best (t bits << 32 | global id) so far; ~0 = none
	float4 rec[32];              // per lane: u, v (quad: numerators), quad |n|^2 (else 0), leaf index
	unsigned short ring[64];     // queued pairs (lane << 8 | leaf-order primitive)
};

__device__ __forceinline__ float key_t(unsigned long long k) {
	return k == ~0ull ? __int_as_float(0x7f800000) : __uint_as_float((unsigned)(k >> 32));
}

// The test of staged primitive j, as in closest_hit_linear's inner loop; quads
// report u, v as numerators over qnn.
__device__ __forceinline__ bool test_staged(const float4 *__restrict__ sp, int j, int tri_wt, f3 o, f3 d, float tmin,
	float tmax, float tcut, float &t, float &u, float &v, float &qnn, int &gid) {
	const float4 p0 = sp[4 * j], p1 = sp[4 * j + 1];
	gid = __float_as_int(p1.w);
	u = v = qnn = 0.0f;
	if (p0.w > 0.0f) return hit_sphere(p0, o, d, tmin, tmax, t);
	const float4 p2 = sp[4 * j + 2];
	if (p0.w == PRIM_TAG_QUAD) {
		const float4 p3 = sp[4 * j + 3];
		qnn = p3.w;
		return hit_quad_pre(ld3(p0), ld3(p1), ld3(p2), ld3(p3), p3.w, o, d, tmin, tmax, tcut, t, u, v);
	}
	if (tri_wt) return hit_tri_wt(ld3(p0), ld3(p1), ld3(p2), o, d, tmin, tmax, t, u, v);
	return hit_tri_mt(ld3(p0), ld3(p1), ld3(p2), o, d, tmin, tmax, t, u, v);
}

// One round: lane k < n takes queued pair head + k and tests it on its
// owner's ray and interval (shuffled in), then the owner's key keeps the
// minimum and the pair that holds it records u, v.
__device__ __forceinline__ void warp_hit_round(const float4 *__restrict__ sp, int tri_wt, f3 o, f3 d, float tmin,
	float tmax, WarpHitScratch &ws, unsigned head, unsigned n) {
	const unsigned lane = threadIdx.x & 31u;
	const bool has = lane < n;
	const unsigned e = has ? (unsigned)ws.ring[(head + lane) & 63u] : 0u;
	const int owner = (int)(e >> 8), j = (int)(e & 0xffu);
	const f3 oo{ __shfl_sync(0xffffffffu, o.x, owner), __shfl_sync(0xffffffffu, o.y, owner),
		__shfl_sync(0xffffffffu, o.z, owner) };
	const f3 dd{ __shfl_sync(0xffffffffu, d.x, owner), __shfl_sync(0xffffffffu, d.y, owner),
		__shfl_sync(0xffffffffu, d.z, owner) };
	const float t0 = __shfl_sync(0xffffffffu, tmin, owner), t1 = __shfl_sync(0xffffffffu, tmax, owner);
	bool h = false;
	float t = 0.0f, u = 0.0f, v = 0.0f, qnn = 0.0f;
	unsigned long long k = ~0ull;
	if (has) {
		int gid;
		h = test_staged(sp, j, tri_wt, oo, dd, t0, t1, key_t(ws.key[owner]), t, u, v, qnn, gid);
		if (h) {
			k = ((unsigned long long)__float_as_uint(t) << 32) | (unsigned)gid;
			atomicMin(&ws.key[owner], k);
		}
	}
	__syncwarp();
	if (h && ws.key[owner] == k) ws.rec[owner] = make_float4(u, v, qnn, __int_as_float(j));
	__syncwarp();
}

// Same answer as closest_hit_linear (per-lane rays and intervals) for rays
// with tmin >= 0 (every hit then has t > 0, whose bits order like its value).
// Every lane of the warp calls it at the same time (converged, full mask); a
// lane with active == false adds no ray and gets a miss.
__device__ __forceinline__ Hit closest_hit_linear_warp(const float4 *__restrict__ sp, int n_leaves, int tri_wt, f3 o,
	f3 d, float tmin, float tmax, bool active, WarpHitScratch &ws) {
	const unsigned lane = threadIdx.x & 31u;
	const unsigned below = (1u << lane) - 1u;
	ws.key[lane] = ~0ull;
	float dx = d.x != 0.0f ? d.x : copysignf(1e-20f, d.x);
	float dy = d.y != 0.0f ? d.y : copysignf(1e-20f, d.y);
	float dz = d.z != 0.0f ? d.z : copysignf(1e-20f, d.z);
	float ix = __frcp_rn(dx), iy = __frcp_rn(dy), iz = __frcp_rn(dz);
	float ox = -o.x * ix, oy = -o.y * iy, oz = -o.z * iz;
	unsigned queued = 0, head = 0;  // warp-uniform
	__syncwarp();
	for (int l = 0; l < n_leaves; ++l) {
		// the leaf's padded box against this lane's best so far (culling only)
		const float4 b0 = sp[4 * LINEAR_MAX + 2 * l], b1 = sp[4 * LINEAR_MAX + 2 * l + 1];
		float t0x = fmaf(b0.x, ix, ox), t1x = fmaf(b1.x, ix, ox);
		float t0y = fmaf(b0.y, iy, oy), t1y = fmaf(b1.y, iy, oy);
		float t0z = fmaf(b0.z, iz, oz), t1z = fmaf(b1.z, iz, oz);
		float lo = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
		float hi = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)),
			fminf(fmaxf(t0z, t1z), fminf(key_t(ws.key[lane]), tmax) * 1.0000039f));
		const bool pass = active && lo <= hi;
		if (!__any_sync(0xffffffffu, pass)) continue;
		const int first = __float_as_int(b0.w), end = first + __float_as_int(b1.w);
		for (int j = first; j < end; ++j) {
			const float4 p0 = sp[4 * j];
			bool cand = pass;
			if (p0.w == PRIM_TAG_QUAD) {
				// hit_quad_pre's first rejections: plane parallel to the ray or behind it
				const float4 p3 = sp[4 * j + 3];
				const f3 n = ld3(p3);
				const float denom = rdot(n, d);
				const float num = rdot(n, rsub(ld3(p0), o));
				cand = cand && denom != 0.0f && !(tmin >= 0.0f && !((num > 0.0f) == (denom > 0.0f) && num != 0.0f));
			}
			const unsigned m = __ballot_sync(0xffffffffu, cand);
			if (cand) ws.ring[(queued + (unsigned)__popc(m & below)) & 63u] = (unsigned short)((lane << 8) | (unsigned)j);
			queued += (unsigned)__popc(m);
			if (queued - head >= 32u) {
				__syncwarp();
				warp_hit_round(sp, tri_wt, o, d, tmin, tmax, ws, head, 32u);
				head += 32u;
			}
		}
	}
	if (queued > head) {
		__syncwarp();
		warp_hit_round(sp, tri_wt, o, d, tmin, tmax, ws, head, queued - head);
	}
	__syncwarp();
	Hit best;
	best.t = __int_as_float(0x7f800000);
	best.leaf = -1;
	best.gid = 0x7fffffff;
	best.u = best.v = 0.0f;
	const unsigned long long k = ws.key[lane];
	if (k != ~0ull) {
		const float4 r = ws.rec[lane];
		best.t = key_t(k);
		best.gid = (int32_t)(unsigned)(k & 0xffffffffull);
		best.leaf = __float_as_int(r.w);
		best.u = r.z != 0.0f ? __fdiv_rn(r.x, r.z) : r.x;
		best.v = r.z != 0.0f ? __fdiv_rn(r.y, r.z) : r.y;
	}
	__syncwarp();  // the scratch is free for the next call
	return best;
}

// Closest hit with the (t, global id) order.  `snodes` holds the first
// `n_snodes` nodes in shared memory.  err receives ERR_* bits.
// SHORT > 0: the first SHORT stack entries live in shared memory, `sstack`
// holding this thread's column (entry k at sstack[k * blockDim.x]), the rest
// in local memory; SHORT == 0: the whole stack in local memory.
template <int SHORT = 0>
__device__ __forceinline__ Hit closest_hit(const DevScene &S, const float4 *__restrict__ snodes, int n_snodes, f3 o,
	f3 d, float tmin, float tmax, uint32_t &err, int4 *__restrict__ sstack = nullptr) {
	Hit best;
	best.t = __int_as_float(0x7f800000);
	best.leaf = -1;
	best.gid = 0x7fffffff;
	best.u = best.v = 0.0f;
	// slab setup: exact zeros become a tiny value so no 0 * inf appears
	float dx = d.x != 0.0f ? d.x : copysignf(1e-20f, d.x);
	float dy = d.y != 0.0f ? d.y : copysignf(1e-20f, d.y);
	float dz = d.z != 0.0f ? d.z : copysignf(1e-20f, d.z);
	float ix = __frcp_rn(dx), iy = __frcp_rn(dy), iz = __frcp_rn(dz);
	float ox = -o.x * ix, oy = -o.y * iy, oz = -o.z * iz;
	const float4 *__restrict__ G = S.nodes;
	const int32_t tri_wt = S.triangle_test;
	if (S.n_prims == 0) return best;

	int2 stack[MAX_STACK - SHORT];
	float stack_t[MAX_STACK - SHORT];  // entry distance of each pushed node
	int sp = 0;
	// current node (a, b): start with the root's
	float4 r1 = n_snodes > 0 ? snodes[1] : ldg4(G + 1);
	float4 r0 = n_snodes > 0 ? snodes[0] : ldg4(G + 0);
	int a = __float_as_int(r0.w), b = __float_as_int(r1.w);
	{
		// root box test
		float t0x = fmaf(r0.x, ix, ox), t1x = fmaf(r1.x, ix, ox);
		float t0y = fmaf(r0.y, iy, oy), t1y = fmaf(r1.y, iy, oy);
		float t0z = fmaf(r0.z, iz, oz), t1z = fmaf(r1.z, iz, oz);
		float lo = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
		float hi = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), tmax * 1.0000039f));
		if (!(lo <= hi)) return best;
	}
	// a well-formed tree is walked visiting each node pair at most once
	for (int visits = 0;; ++visits) {
		if (visits > S.n_nodes) {
			err |= ERR_BVH_WALK;
			break;
		}
		if (b == 0) {
			// interior: test both children (one 64-byte line)
			int c = a;
			float4 c00, c01, c10, c11;
			if (c + 1 < n_snodes) {
				c00 = snodes[2 * c];
				c01 = snodes[2 * c + 1];
				c10 = snodes[2 * c + 2];
				c11 = snodes[2 * c + 3];
			} else {
				c00 = ldg4(G + 2 * c);
				c01 = ldg4(G + 2 * c + 1);
				c10 = ldg4(G + 2 * c + 2);
				c11 = ldg4(G + 2 * c + 3);
			}
			float bt = fminf(best.t * 1.0000039f, tmax * 1.0000039f);
			float l0, l1;
			bool h0, h1;
			{
				float t0x = fmaf(c00.x, ix, ox), t1x = fmaf(c01.x, ix, ox);
				float t0y = fmaf(c00.y, iy, oy), t1y = fmaf(c01.y, iy, oy);
				float t0z = fmaf(c00.z, iz, oz), t1z = fmaf(c01.z, iz, oz);
				l0 = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
				float hi = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), bt));
				h0 = l0 <= hi;
			}
			{
				float t0x = fmaf(c10.x, ix, ox), t1x = fmaf(c11.x, ix, ox);
				float t0y = fmaf(c10.y, iy, oy), t1y = fmaf(c11.y, iy, oy);
				float t0z = fmaf(c10.z, iz, oz), t1z = fmaf(c11.z, iz, oz);
				l1 = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
				float hi = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), bt));
				h1 = l1 <= hi;
			}
			if (h0 && h1) {
				int2 nearn = make_int2(__float_as_int(c00.w), __float_as_int(c01.w));
				int2 farn = make_int2(__float_as_int(c10.w), __float_as_int(c11.w));
				if (l1 < l0) {
					int2 t = nearn;
					nearn = farn;
					farn = t;
				}
				if (SHORT > 0 && sp < SHORT) {
					sstack[sp++ * (int)blockDim.x] = make_int4(farn.x, farn.y, __float_as_int(fmaxf(l0, l1)), 0);
				} else if (sp < MAX_STACK) {
					stack_t[sp - SHORT] = fmaxf(l0, l1);
					stack[sp++ - SHORT] = farn;
				} else {
					err |= ERR_STACK_OVERFLOW;
				}
				a = nearn.x;
				b = nearn.y;
				continue;
			}
			if (h0) {
				a = __float_as_int(c00.w);
				b = __float_as_int(c01.w);
				continue;
			}
			if (h1) {
				a = __float_as_int(c10.w);
				b = __float_as_int(c11.w);
				continue;
			}
		} else {
			// leaf: primitives [a, a + b)
			for (int i = a; i < a + b; ++i) {
				const float4 *P = S.prims + 3 * (size_t)i;
				float4 p0 = ldg4(P);
				float t, u = 0.0f, v = 0.0f;
				bool h;
				if (p0.w > 0.0f) {
					h = hit_sphere(p0, o, d, tmin, tmax, t);
				} else {
					float4 p1 = ldg4(P + 1), p2 = ldg4(P + 2);
					if (p0.w == PRIM_TAG_QUAD)
						h = hit_quad(ld3(p0), ld3(p1), ld3(p2), o, d, tmin, tmax, best.t, t, u, v);
					else if (tri_wt)
						h = hit_tri_wt(ld3(p0), ld3(p1), ld3(p2), o, d, tmin, tmax, t, u, v);
					else
						h = hit_tri_mt(ld3(p0), ld3(p1), ld3(p2), o, d, tmin, tmax, t, u, v);
				}
				if (h && t <= best.t) {
					int32_t gid = __ldg(S.prim_gid + i);
					if (t < best.t || gid < best.gid) {
						best.t = t;
						best.leaf = i;
						best.gid = gid;
						best.u = u;
						best.v = v;
					}
				}
			}
		}
		// pop, skipping nodes whose entry lies beyond the best hit found since the push
		bool found = false;
		while (sp > 0) {
			--sp;
			int2 e;
			float te;
			if (SHORT > 0 && sp < SHORT) {
				const int4 r = sstack[sp * (int)blockDim.x];
				e = make_int2(r.x, r.y);
				te = __int_as_float(r.z);
			} else {
				e = stack[sp - SHORT];
				te = stack_t[sp - SHORT];
			}
			if (te <= best.t * 1.0000039f) {
				a = e.x;
				b = e.y;
				found = true;
				break;
			}
		}
		if (!found) break;
	}
	return best;
}


// ---------------------------------------------------------------------------
// 4-wide tree (DevScene::nodes4, built on the host by collapse_bvh4): each node
// is four 32-byte child records, so one step tests four boxes from one
// 128-byte line and the tree is half as deep as the binary one.  Same answer
// as closest_hit: boxes only cull (padded as in the binary tree), primitives
// are tested by the same functions and the best hit keeps the (t, global id)
// order, whatever order the nodes are visited in.

// the primitives [a, a + b) of a leaf against the best hit so far
__device__ __forceinline__ void leaf_hits(const DevScene &S, int a, int b, f3 o, f3 d, float tmin, float tmax,
	Hit &best) {
	const int32_t tri_wt = S.triangle_test;
	for (int i = a; i < a + b; ++i) {
		const float4 *P = S.prims + 3 * (size_t)i;
		const float4 p0 = ldg4(P);
		float t, u = 0.0f, v = 0.0f;
		bool h;
		if (p0.w > 0.0f) {
			h = hit_sphere(p0, o, d, tmin, tmax, t);
		} else {
			const float4 p1 = ldg4(P + 1), p2 = ldg4(P + 2);
			if (p0.w == PRIM_TAG_QUAD)
				h = hit_quad(ld3(p0), ld3(p1), ld3(p2), o, d, tmin, tmax, best.t, t, u, v);
			else if (tri_wt)
				h = hit_tri_wt(ld3(p0), ld3(p1), ld3(p2), o, d, tmin, tmax, t, u, v);
			else
				h = hit_tri_mt(ld3(p0), ld3(p1), ld3(p2), o, d, tmin, tmax, t, u, v);
		}
		if (h && t <= best.t) {
			const int32_t gid = __ldg(S.prim_gid + i);
			if (t < best.t || gid < best.gid) {
				best.t = t;
				best.leaf = i;
				best.gid = gid;
				best.u = u;
				best.v = v;
			}
		}
	}
}

// Stages the first SMEM_NODES4 wide nodes (breadth-first top levels) into the
// same 32 KB buffer stage_nodes uses.
__device__ __forceinline__ void stage_nodes4(const DevScene &S, float4 *snodes, int &n_snodes4, int max_nodes = SMEM_NODES4) {
	n_snodes4 = min(S.n_nodes4, max_nodes);
	for (int i = threadIdx.x; i < 8 * n_snodes4; i += blockDim.x) snodes[i] = __ldg(S.nodes4 + i);
	__syncthreads();
}

// SHORT > 0: the first SHORT stack entries in shared memory (this thread's
// column, entry k at sstack[k * blockDim.x]), the rest in local memory.
template <int SHORT = 0>
__device__ __forceinline__ Hit closest_hit4(const DevScene &S, const float4 *__restrict__ snodes, int n_snodes4, f3 o,
	f3 d, float tmin, float tmax, uint32_t &err, int4 *__restrict__ sstack = nullptr) {
	Hit best;
	best.t = __int_as_float(0x7f800000);
	best.leaf = -1;
	best.gid = 0x7fffffff;
	best.u = best.v = 0.0f;
	float dx = d.x != 0.0f ? d.x : copysignf(1e-20f, d.x);
	float dy = d.y != 0.0f ? d.y : copysignf(1e-20f, d.y);
	float dz = d.z != 0.0f ? d.z : copysignf(1e-20f, d.z);
	float ix = __frcp_rn(dx), iy = __frcp_rn(dy), iz = __frcp_rn(dz);
	float ox = -o.x * ix, oy = -o.y * iy, oz = -o.z * iz;
	{
		// the root's box (binary record 0)
		const float4 r0 = ldg4(S.nodes), r1 = ldg4(S.nodes + 1);
		float t0x = fmaf(r0.x, ix, ox), t1x = fmaf(r1.x, ix, ox);
		float t0y = fmaf(r0.y, iy, oy), t1y = fmaf(r1.y, iy, oy);
		float t0z = fmaf(r0.z, iz, oz), t1z = fmaf(r1.z, iz, oz);
		float lo = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
		float hi = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), tmax * 1.0000039f));
		if (!(lo <= hi)) return best;
	}
	// stack entries: (reference, count: 0 = wide node, > 0 = leaf) and the entry distance
	int2 stack[MAX_STACK4 - SHORT];
	float stack_t[MAX_STACK4 - SHORT];
	int sp = 0;
	int a = 0, b = 0;  // current entry: the root's wide node
	const int limit = 4 * S.n_nodes4 + 1;  // a well-formed tree yields each entry once
	for (int steps = 0;; ++steps) {
		if (steps > limit) {
			err |= ERR_BVH_WALK;
			break;
		}
		if (b > 0) {
			leaf_hits(S, a, b, o, d, tmin, tmax, best);
		} else {
			if ((unsigned)a >= (unsigned)S.n_nodes4) {
				err |= ERR_BVH_WALK;
				break;
			}
			// the four children: entry distances of those entered, nearest first
			const bool shared = a < n_snodes4;
			const float4 *__restrict__ src = shared ? snodes + 8 * a : S.nodes4 + 8 * (size_t)a;
			const float bt = fminf(best.t, tmax) * 1.0000039f;
			float l[4];
			int2 e[4];
#pragma unroll
			for (int k = 0; k < 4; ++k) {
				const float4 c0 = shared ? src[2 * k] : ldg4(src + 2 * k);
				const float4 c1 = shared ? src[2 * k + 1] : ldg4(src + 2 * k + 1);
				float t0x = fmaf(c0.x, ix, ox), t1x = fmaf(c1.x, ix, ox);
				float t0y = fmaf(c0.y, iy, oy), t1y = fmaf(c1.y, iy, oy);
				float t0z = fmaf(c0.z, iz, oz), t1z = fmaf(c1.z, iz, oz);
				const float lo = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
				const float hi = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), bt));
				e[k] = make_int2(__float_as_int(c0.w), __float_as_int(c1.w));
				// unused slots (count < 0) and boxes not entered sort last
				l[k] = (lo <= hi && e[k].y >= 0) ? lo : __int_as_float(0x7f800000);
			}
			// sorting network on (l, e), ascending
#define ARE_CSWAP(i, j)                                           \
	if (l[j] < l[i]) {                                            \
		const float tl = l[i];                                    \
		l[i] = l[j], l[j] = tl;                                   \
		const int2 te = e[i];                                     \
		e[i] = e[j], e[j] = te;                                   \
	}
			ARE_CSWAP(0, 1) ARE_CSWAP(2, 3) ARE_CSWAP(0, 2) ARE_CSWAP(1, 3) ARE_CSWAP(1, 2)
#undef ARE_CSWAP
			// push the farther entered children (farthest first), continue with the nearest
			const float inf = __int_as_float(0x7f800000);
#pragma unroll
			for (int k = 3; k >= 1; --k) {
				if (!(l[k] < inf)) continue;
				if (SHORT > 0 && sp < SHORT) {
					sstack[sp++ * (int)blockDim.x] = make_int4(e[k].x, e[k].y, __float_as_int(l[k]), 0);
				} else if (sp < MAX_STACK4) {
					stack[sp - SHORT] = e[k];
					stack_t[sp++ - SHORT] = l[k];
				} else {
					err |= ERR_STACK_OVERFLOW;
				}
			}
			if (l[0] < inf) {
				a = e[0].x;
				b = e[0].y;
				continue;
			}
		}
		// pop, skipping entries that begin beyond the best hit found since the push
		bool found = false;
		while (sp > 0) {
			--sp;
			int2 en;
			float te;
			if (SHORT > 0 && sp < SHORT) {
				const int4 r = sstack[sp * (int)blockDim.x];
				en = make_int2(r.x, r.y);
				te = __int_as_float(r.z);
			} else {
				en = stack[sp - SHORT];
				te = stack_t[sp - SHORT];
			}
			if (te <= best.t * 1.0000039f) {
				a = en.x;
				b = en.y;
				found = true;
				break;
			}
		}
		if (!found) break;
	}
	return best;
}

// ---------------------------------------------------------------------------
// The walks of closest_hit and closest_hit4 as resumable state machines:
// walk2_begin / walk4_begin set a ray up, each walk2_step / walk4_step visits
// one entry (an interior node, a leaf, or for the 4-wide tree one primitive of
// a leaf) and picks the next, in the same order and with the same arithmetic,
// so the hit is the same bit for bit.  A persistent kernel can then hold a lane
// whose walk has ended (its hit waiting to be shaded, or the lane taking its
// next ray) while the other lanes of its warp take further steps, and can let
// only the lanes at an interior node (or only those at a leaf) step at a time,
// instead of every lane waiting for the longest walk of the warp and every
// step running both kinds of visit.

struct Walk {
	float ix, iy, iz, ox, oy, oz;  // reciprocal direction and -origin / direction
	Hit best;
	int a, b;   // current entry: (reference, count: 0 = interior node, > 0 = leaf)
	int sp;     // stack depth
	int steps;  // entries visited
};

// the stack entries past those in shared memory
template <int N>
struct WalkStack {
	int2 e[N];
	float t[N];
};

__device__ __forceinline__ void walk_setup(f3 o, f3 d, Walk &w) {
	w.best.t = __int_as_float(0x7f800000);
	w.best.leaf = -1;
	w.best.gid = 0x7fffffff;
	w.best.u = w.best.v = 0.0f;
	const float dx = d.x != 0.0f ? d.x : copysignf(1e-20f, d.x);
	const float dy = d.y != 0.0f ? d.y : copysignf(1e-20f, d.y);
	const float dz = d.z != 0.0f ? d.z : copysignf(1e-20f, d.z);
	w.ix = __frcp_rn(dx), w.iy = __frcp_rn(dy), w.iz = __frcp_rn(dz);
	w.ox = -o.x * w.ix, w.oy = -o.y * w.iy, w.oz = -o.z * w.iz;
	w.sp = w.steps = 0;
}

// whether the ray of w enters box (r0, r1) between tmin and tmax
__device__ __forceinline__ bool walk_root(const Walk &w, float4 r0, float4 r1, float tmin, float tmax) {
	const float t0x = fmaf(r0.x, w.ix, w.ox), t1x = fmaf(r1.x, w.ix, w.ox);
	const float t0y = fmaf(r0.y, w.iy, w.oy), t1y = fmaf(r1.y, w.iy, w.oy);
	const float t0z = fmaf(r0.z, w.iz, w.oz), t1z = fmaf(r1.z, w.iz, w.oz);
	const float lo = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
	const float hi = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), tmax * 1.0000039f));
	return lo <= hi;
}

// Pops the next entry that begins before the best hit; false when none is left.
template <int SHORT, int N>
__device__ __forceinline__ bool walk_pop(int4 *__restrict__ sstack, WalkStack<N> &st, Walk &w) {
	while (w.sp > 0) {
		--w.sp;
		int2 en;
		float te;
		if (SHORT > 0 && w.sp < SHORT) {
			const int4 r = sstack[w.sp * (int)blockDim.x];
			en = make_int2(r.x, r.y);
			te = __int_as_float(r.z);
		} else {
			en = st.e[w.sp - SHORT];
			te = st.t[w.sp - SHORT];
		}
		if (te <= w.best.t * 1.0000039f) {
			w.a = en.x;
			w.b = en.y;
			return true;
		}
	}
	return false;
}

// Pushes entry e at distance te (SHORT entries in shared memory, then st).
template <int SHORT, int N>
__device__ __forceinline__ void walk_push(int4 *__restrict__ sstack, WalkStack<N> &st, Walk &w, int2 e, float te,
	uint32_t &err) {
	if (SHORT > 0 && w.sp < SHORT) {
		sstack[w.sp++ * (int)blockDim.x] = make_int4(e.x, e.y, __float_as_int(te), 0);
	} else if (w.sp < SHORT + N) {
		st.e[w.sp - SHORT] = e;
		st.t[w.sp++ - SHORT] = te;
	} else {
		err |= ERR_STACK_OVERFLOW;
	}
}

// Binary tree (closest_hit's walk): sets up ray (o, d); false when the walk is
// over before it begins (no primitives, or the root's box missed).
__device__ __forceinline__ bool walk2_begin(const DevScene &S, const float4 *__restrict__ snodes, int n_snodes, f3 o,
	f3 d, float tmin, float tmax, Walk &w) {
	walk_setup(o, d, w);
	if (S.n_prims == 0) return false;
	const float4 r1 = n_snodes > 0 ? snodes[1] : ldg4(S.nodes + 1);
	const float4 r0 = n_snodes > 0 ? snodes[0] : ldg4(S.nodes + 0);
	w.a = __float_as_int(r0.w), w.b = __float_as_int(r1.w);
	return walk_root(w, r0, r1, tmin, tmax);
}

// Binary tree: visits the current entry and moves to the next; false when the walk is over.
template <int SHORT>
__device__ __forceinline__ bool walk2_step(const DevScene &S, const float4 *__restrict__ snodes, int n_snodes, f3 o,
	f3 d, float tmin, float tmax, uint32_t &err, int4 *__restrict__ sstack, WalkStack<MAX_STACK - SHORT> &st, Walk &w) {
	if (w.steps++ > S.n_nodes) {  // a well-formed tree is walked visiting each node pair at most once
		err |= ERR_BVH_WALK;
		return false;
	}
	if (w.b == 0) {
		// interior: both children (one 64-byte line)
		const int c = w.a;
		float4 c00, c01, c10, c11;
		if (c + 1 < n_snodes) {
			c00 = snodes[2 * c], c01 = snodes[2 * c + 1], c10 = snodes[2 * c + 2], c11 = snodes[2 * c + 3];
		} else {
			c00 = ldg4(S.nodes + 2 * c), c01 = ldg4(S.nodes + 2 * c + 1);
			c10 = ldg4(S.nodes + 2 * c + 2), c11 = ldg4(S.nodes + 2 * c + 3);
		}
		const float bt = fminf(w.best.t * 1.0000039f, tmax * 1.0000039f);
		float l0, l1;
		bool h0, h1;
		{
			const float t0x = fmaf(c00.x, w.ix, w.ox), t1x = fmaf(c01.x, w.ix, w.ox);
			const float t0y = fmaf(c00.y, w.iy, w.oy), t1y = fmaf(c01.y, w.iy, w.oy);
			const float t0z = fmaf(c00.z, w.iz, w.oz), t1z = fmaf(c01.z, w.iz, w.oz);
			l0 = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
			const float hi = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), bt));
			h0 = l0 <= hi;
		}
		{
			const float t0x = fmaf(c10.x, w.ix, w.ox), t1x = fmaf(c11.x, w.ix, w.ox);
			const float t0y = fmaf(c10.y, w.iy, w.oy), t1y = fmaf(c11.y, w.iy, w.oy);
			const float t0z = fmaf(c10.z, w.iz, w.oz), t1z = fmaf(c11.z, w.iz, w.oz);
			l1 = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
			const float hi = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), bt));
			h1 = l1 <= hi;
		}
		if (h0 && h1) {
			int2 nearn = make_int2(__float_as_int(c00.w), __float_as_int(c01.w));
			int2 farn = make_int2(__float_as_int(c10.w), __float_as_int(c11.w));
			if (l1 < l0) {
				const int2 t = nearn;
				nearn = farn;
				farn = t;
			}
			walk_push<SHORT>(sstack, st, w, farn, fmaxf(l0, l1), err);
			w.a = nearn.x;
			w.b = nearn.y;
			return true;
		}
		if (h0 || h1) {
			w.a = __float_as_int(h0 ? c00.w : c10.w);
			w.b = __float_as_int(h0 ? c01.w : c11.w);
			return true;
		}
	} else {
		leaf_hits(S, w.a, w.b, o, d, tmin, tmax, w.best);
	}
	return walk_pop<SHORT>(sstack, st, w);
}

// 4-wide tree (closest_hit4's walk): sets up ray (o, d); false when the ray
// misses the root's box (the walk is over: w.best is the miss).
__device__ __forceinline__ bool walk4_begin(const DevScene &S, f3 o, f3 d, float tmin, float tmax, Walk &w) {
	walk_setup(o, d, w);
	w.a = w.b = 0;
	return walk_root(w, ldg4(S.nodes), ldg4(S.nodes + 1), tmin, tmax);
}

// 4-wide tree: visits the current entry and moves to the next; false when the walk is over.
template <int SHORT>
__device__ __forceinline__ bool walk4_step(const DevScene &S, const float4 *__restrict__ snodes, int n_snodes4, f3 o,
	f3 d, float tmin, float tmax, uint32_t &err, int4 *__restrict__ sstack, WalkStack<MAX_STACK4 - SHORT> &st, Walk &w) {
	// a well-formed tree yields each entry once, and a leaf's primitives are visited one per step
	if (w.steps++ > 4 * S.n_nodes4 + 1 + S.n_prims) {
		err |= ERR_BVH_WALK;
		return false;
	}
	const float inf = __int_as_float(0x7f800000);
	if (w.b > 0) {
		// one primitive per step, so a leaf round tests one primitive in every lane taking part
		leaf_hits(S, w.a, 1, o, d, tmin, tmax, w.best);
		if (w.b > 1) {
			++w.a;
			--w.b;
			return true;
		}
	} else {
		if ((unsigned)w.a >= (unsigned)S.n_nodes4) {
			err |= ERR_BVH_WALK;
			return false;
		}
		const bool shared = w.a < n_snodes4;
		const float4 *__restrict__ src = shared ? snodes + 8 * w.a : S.nodes4 + 8 * (size_t)w.a;
		const float bt = fminf(w.best.t, tmax) * 1.0000039f;
		float l[4];
		int2 e[4];
#pragma unroll
		for (int k = 0; k < 4; ++k) {
			const float4 c0 = shared ? src[2 * k] : ldg4(src + 2 * k);
			const float4 c1 = shared ? src[2 * k + 1] : ldg4(src + 2 * k + 1);
			const float t0x = fmaf(c0.x, w.ix, w.ox), t1x = fmaf(c1.x, w.ix, w.ox);
			const float t0y = fmaf(c0.y, w.iy, w.oy), t1y = fmaf(c1.y, w.iy, w.oy);
			const float t0z = fmaf(c0.z, w.iz, w.oz), t1z = fmaf(c1.z, w.iz, w.oz);
			const float lo = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
			const float hi = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), bt));
			e[k] = make_int2(__float_as_int(c0.w), __float_as_int(c1.w));
			l[k] = (lo <= hi && e[k].y >= 0) ? lo : inf;
		}
#define ARE_CSWAP(i, j)                                           \
	if (l[j] < l[i]) {                                            \
		const float tl = l[i];                                    \
		l[i] = l[j], l[j] = tl;                                   \
		const int2 te = e[i];                                     \
		e[i] = e[j], e[j] = te;                                   \
	}
		ARE_CSWAP(0, 1) ARE_CSWAP(2, 3) ARE_CSWAP(0, 2) ARE_CSWAP(1, 3) ARE_CSWAP(1, 2)
#undef ARE_CSWAP
#pragma unroll
		for (int k = 3; k >= 1; --k)
			if (l[k] < inf) walk_push<SHORT>(sstack, st, w, e[k], l[k], err);
		if (l[0] < inf) {
			w.a = e[0].x;
			w.b = e[0].y;
			return true;
		}
	}
	return walk_pop<SHORT>(sstack, st, w);
}

// Stages the top of whichever tree closest_hit_any traverses.
__device__ __forceinline__ void stage_bvh(const DevScene &S, float4 *snodes, int &n_snodes) {
	if (S.n_nodes4 > 0)
		stage_nodes4(S, snodes, n_snodes);
	else
		stage_nodes(S, snodes, n_snodes);
}

// The 4-wide tree when the scene has one, else the binary tree; `snodes` /
// `n_snodes` as staged by stage_bvh.
template <int SHORT = 0>
__device__ __forceinline__ Hit closest_hit_any(const DevScene &S, const float4 *__restrict__ snodes, int n_snodes, f3 o,
	f3 d, float tmin, float tmax, uint32_t &err, int4 *__restrict__ sstack = nullptr) {
	if (S.n_nodes4 > 0) return closest_hit4<SHORT>(S, snodes, n_snodes, o, d, tmin, tmax, err, sstack);
	return closest_hit<SHORT>(S, snodes, n_snodes, o, d, tmin, tmax, err, sstack);
}

}  // namespace are_core
