// legacy.cu — rt.cpp's own estimator on the GPU (ARE_EST_LEGACY_RT).
//
// experiments/rt.cpp trace() / computeAO() (rt.cpp:221-334) per pixel:
// barycentric hit point, 32 ambient-occlusion rays, a mirror bounce at depth
// 0 for MAT_METAL, 32 cosine paths of up to 3 bounces with Russian roulette
// for MAT_DIFFUSE, clamping; camera rays through pixel centres (rt.cpp:337-374).
// Intersections are the bit-exact Möller–Trumbore closest-hit queries of
// traverse.cuh with rt.cpp's EPS = 1e-5 and INF = 1e30.
//
// Random streams:
//  * counter-based (default): draws of pixel p are numbered 0, 1, 2, ... and
//    keyed by (seed, p), so every pixel is an independent thread;
//  * ARE_FLAG_LEGACY_MT19937: rt.cpp's own stream, one std::mt19937 per image
//    row seeded with seed + y (rt.cpp:348-351) and consumed pixel after pixel
//    through uniform_real_distribution<float>(0, 1); one thread per row.  The
//    Mersenne Twister is Matsumoto and Nishimura (1998) with the C++
//    standard's parameters; the float draw is (float)g / 2^32 with a result
//    of 1.0 mapped to the largest float below 1 as GCC 13's libstdc++ does.
#include <cuda_runtime.h>

#include <cmath>
#include <string>

#include "scene.h"
#include "shade.cuh"
#include "traverse.cuh"

namespace are_core {

namespace {

constexpr float LEPS = 1e-5f;
constexpr float LINF = 1e30f;
constexpr int LBLOCK = 128;

struct CounterRng {
	uint64_t key;
	uint32_t ctr;
	__device__ float next() { return uniform(key, ctr++); }
};

// MT19937 state of one row lives in global memory, interleaved across rows
// (word k of row r at k * stride + r) so the threads of a warp touch adjacent words.
struct MtRng {
	uint32_t *x;
	int stride;
	int i;
	__device__ uint32_t &w(int k) { return x[(size_t)k * stride]; }
	__device__ void seed(uint32_t s) {
		w(0) = s;
		uint32_t prev = s;
		for (int k = 1; k < 624; ++k) {
			prev = 1812433253u * (prev ^ (prev >> 30)) + (uint32_t)k;
			w(k) = prev;
		}
		i = 624;
	}
	__device__ uint32_t next_u32() {
		if (i >= 624) {
			for (int k = 0; k < 624; ++k) {
				uint32_t y = (w(k) & 0x80000000u) | (w(k + 1 < 624 ? k + 1 : 0) & 0x7fffffffu);
				int k2 = k + 397 < 624 ? k + 397 : k + 397 - 624;
				w(k) = w(k2) ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
			}
			i = 0;
		}
		uint32_t y = w(i++);
		y ^= y >> 11;
		y ^= (y << 7) & 0x9d2c5680u;
		y ^= (y << 15) & 0xefc60000u;
		y ^= y >> 18;
		return y;
	}
	__device__ float next() {
		float r = __fdiv_rn((float)next_u32(), 4294967296.0f);
		return r >= 1.0f ? 0.99999994f : r;
	}
};

struct LegacyFrame {
	float pos[3], fwd[3], right[3], up[3];
	float aspect, scale;
	int width, height, spp;
	float bg[3];
};

// All vector arithmetic here follows rt.cpp's Vec3/Color operators, each
// operation rounded on its own (no contraction), so the CPU restatement and
// the device agree except where a transcendental differs by an ulp.
__device__ __forceinline__ f3 nrm(f3 a) { return rscl(a, __frcp_rn(__fsqrt_rn(rdot(a, a)))); }
__device__ __forceinline__ f3 vmul(f3 a, f3 b) {
	return f3{ __fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z) };
}
__device__ __forceinline__ f3 clamp01(f3 c) {
	return f3{ fmaxf(0.f, fminf(1.f, c.x)), fmaxf(0.f, fminf(1.f, c.y)), fmaxf(0.f, fminf(1.f, c.z)) };
}

struct LSurf {
	f3 p, n, albedo, tint;
	bool metal;
	float rr;
};

__device__ LSurf lsurface(const DevScene &S, const Hit &h) {
	LSurf o;
	const float4 *P = S.prims + 3 * (size_t)h.leaf;
	f3 v0 = ld3(__ldg(P)), v1 = ld3(__ldg(P + 1)), v2 = ld3(__ldg(P + 2));
	o.n = nrm(rcross(rsub(v1, v0), rsub(v2, v0)));
	float b0 = __fsub_rn(__fsub_rn(1.0f, h.u), h.v);
	o.p = radd(radd(rscl(v0, b0), rscl(v1, h.u)), rscl(v2, h.v));
	float tu = 0.f, tv = 0.f;
	if (S.tri_uv) {
		const float *uv = S.tri_uv + 6 * (size_t)h.leaf;
		tu = __fadd_rn(__fadd_rn(__fmul_rn(uv[0], b0), __fmul_rn(uv[2], h.u)), __fmul_rn(uv[4], h.v));
		tv = __fadd_rn(__fadd_rn(__fmul_rn(uv[1], b0), __fmul_rn(uv[3], h.u)), __fmul_rn(uv[5], h.v));
	}
	const DevMaterial &m = S.mats[__ldg(S.prim_mat + h.leaf)];
	o.albedo = tex_eval(S, m.texture, tu, tv, o.p);
	o.metal = m.type == ARE_MAT_METAL;
	o.rr = m.reflect_ratio;
	o.tint = ldf3(m.tint);
	return o;
}

// rt.cpp:50-55 rotateToHemisphere
__device__ f3 lhemi(f3 n, float u, float v) {
	f3 up = fabsf(n.z) < 0.999f ? f3{ 0.f, 0.f, 1.f } : f3{ 1.f, 0.f, 0.f };
	f3 tg = nrm(rcross(n, up));
	f3 bt = rcross(n, tg);
	float w = __fsub_rn(__fsub_rn(1.0f, __fmul_rn(u, u)), __fmul_rn(v, v));
	return radd(radd(rscl(tg, u), rscl(bt, v)), rscl(n, __fsqrt_rn(w > 0.f ? w : 0.f)));
}

__device__ __forceinline__ float two_pi_times(float u) { return (float)(6.283185307179586 * (double)u); }

template <class Rng>
__device__ float compute_ao(const DevScene &S, const float4 *sn, int nsn, f3 p, f3 n, Rng &rng, uint32_t &err) {
	int unoccluded = 0;
	const f3 zax{ 0.f, 0.f, 1.f };
	f3 o = radd(p, rscl(n, LEPS));
	for (int i = 0; i < 32; ++i) {
		float u = rng.next(), v = rng.next();
		float theta = two_pi_times(u);
		float phi = acosf(__fsub_rn(1.0f, __fmul_rn(2.0f, v)));
		float sp = sinf(phi);
		float x = __fmul_rn(sp, cosf(theta));
		float y = __fmul_rn(sp, sinf(theta));
		float z = cosf(phi);
		if (z < 0.f) z = -z;
		f3 d{ x, y, z };
		f3 axis = rcross(zax, n);
		float sa = __fsqrt_rn(rdot(axis, axis)), ca = rdot(zax, n);
		if (sa > LEPS) {
			axis = nrm(axis);
			float ang = acosf(ca);
			float c = cosf(ang), s = sinf(ang);
			d = radd(radd(rscl(d, c), rscl(rcross(axis, d), s)), rscl(rscl(axis, rdot(axis, d)), __fsub_rn(1.0f, c)));
		}
		d = nrm(d);
		if (closest_hit(S, sn, nsn, o, d, LEPS, LINF, err).leaf < 0) ++unoccluded;
	}
	return __fadd_rn(0.25f, __fmul_rn(0.75f, __fdiv_rn((float)unoccluded, 32.0f)));
}

// rt.cpp:278-329: 32 cosine paths of up to 3 bounces
template <class Rng>
__device__ f3 diffuse_paths(const DevScene &S, const float4 *sn, int nsn, const LSurf &t, Rng &rng, uint32_t &err) {
	f3 accum{ 0.f, 0.f, 0.f };
	for (int s = 0; s < 32; ++s) {
		float r1 = rng.next(), r2 = rng.next();
		float phi = two_pi_times(r1);
		float r2s = __fsqrt_rn(r2);
		f3 dir = lhemi(t.n, __fmul_rn(r2s, cosf(phi)), __fmul_rn(r2s, sinf(phi)));
		f3 org = radd(t.p, rscl(t.n, LEPS));
		f3 thr = t.albedo;
		for (int b = 0; b < 3; ++b) {
			Hit bh = closest_hit(S, sn, nsn, org, dir, LEPS, LINF, err);
			if (bh.leaf < 0) break;
			LSurf bt = lsurface(S, bh);
			thr = vmul(thr, bt.albedo);
			float pr = fmaxf(thr.x, fmaxf(thr.y, thr.z));
			if (rng.next() > pr) break;
			thr = rscl(thr, __frcp_rn(pr));
			f3 nd;
			if (bt.metal) {
				f3 view = nrm(rsub(f3{ 0.f, 0.f, 0.f }, dir));
				nd = rsub(view, rscl(rscl(bt.n, 2.0f), rdot(view, bt.n)));
			} else {
				float nr1 = rng.next(), nr2 = rng.next();
				float nphi = two_pi_times(nr1);
				float nr2s = __fsqrt_rn(nr2);
				nd = lhemi(bt.n, __fmul_rn(nr2s, cosf(nphi)), __fmul_rn(nr2s, sinf(nphi)));
			}
			org = radd(bt.p, rscl(bt.n, LEPS));
			dir = nd;
		}
		accum = radd(accum, thr);
	}
	return rscl(accum, 1.0f / 32.0f);
}

// rt.cpp:251-334 with the depth-0 recursion unrolled (depth 1 never recurses)
template <class Rng>
__device__ f3 ltrace(const DevScene &S, const float4 *sn, int nsn, const LegacyFrame &F, f3 o, f3 d, Rng &rng,
	uint32_t &err) {
	f3 bg = ldf3(F.bg);
	Hit rec = closest_hit(S, sn, nsn, o, d, LEPS, LINF, err);
	if (rec.leaf < 0) return bg;
	LSurf t = lsurface(S, rec);
	f3 albedo = t.albedo;
	float ao = compute_ao(S, sn, nsn, t.p, t.n, rng, err);
	if (t.metal) {
		f3 view = nrm(rsub(o, t.p));
		f3 refl = rsub(view, rscl(rscl(t.n, 2.0f), rdot(view, t.n)));
		// trace(p + n*EPS, refl, depth 1)
		f3 o1 = radd(t.p, rscl(t.n, LEPS));
		f3 reflected;
		Hit r1 = closest_hit(S, sn, nsn, o1, refl, LEPS, LINF, err);
		if (r1.leaf < 0) {
			reflected = bg;
		} else {
			LSurf t1 = lsurface(S, r1);
			f3 a1 = t1.albedo;
			float ao1 = compute_ao(S, sn, nsn, t1.p, t1.n, rng, err);
			if (!t1.metal) a1 = radd(a1, diffuse_paths(S, sn, nsn, t1, rng, err));
			reflected = clamp01(rscl(a1, ao1));
		}
		f3 ret = radd(rscl(albedo, __fsub_rn(1.0f, t.rr)), vmul(rscl(reflected, t.rr), t.tint));
		return clamp01(rscl(ret, ao));
	}
	albedo = radd(albedo, diffuse_paths(S, sn, nsn, t, rng, err));
	return clamp01(rscl(albedo, ao));
}

__device__ f3 primary_dir(const LegacyFrame &F, int x, int y) {
	float fx = __fmul_rn(__fmul_rn(__fsub_rn(__fdiv_rn(__fmul_rn(2.0f, __fadd_rn((float)x, 0.5f)), (float)F.width), 1.0f),
							   F.aspect),
		F.scale);
	float fy = __fmul_rn(
		__fsub_rn(1.0f, __fdiv_rn(__fmul_rn(2.0f, __fadd_rn((float)y, 0.5f)), (float)F.height)), F.scale);
	f3 dir = radd(radd(ldf3(F.fwd), rscl(ldf3(F.right), fx)), rscl(ldf3(F.up), fy));
	return nrm(dir);
}

__device__ void store(float *rgb, int pix, f3 c) {
	rgb[3 * (size_t)pix] = c.x;
	rgb[3 * (size_t)pix + 1] = c.y;
	rgb[3 * (size_t)pix + 2] = c.z;
}

__global__ void __launch_bounds__(LBLOCK) k_legacy_pixels(DevScene S, LegacyFrame F, uint64_t seed, float *rgb,
	unsigned *err_word) {
	__shared__ float4 snodes[2 * SMEM_NODES];
	int nsn = min(S.n_nodes, SMEM_NODES);
	for (int i = threadIdx.x; i < 2 * nsn; i += blockDim.x) snodes[i] = __ldg(S.nodes + i);
	__syncthreads();
	uint32_t err = 0;
	const int npix = F.width * F.height;
	for (int pix = blockIdx.x * blockDim.x + threadIdx.x; pix < npix; pix += gridDim.x * blockDim.x) {
		int x = pix % F.width, y = pix / F.width;
		CounterRng rng{ path_key(seed, (uint32_t)pix, 0u), 0u };
		f3 d = primary_dir(F, x, y);
		f3 acc{ 0.f, 0.f, 0.f };
		for (int s = 0; s < F.spp; ++s) acc = radd(acc, clamp01(ltrace(S, snodes, nsn, F, ldf3(F.pos), d, rng, err)));
		store(rgb, pix, rscl(acc, __frcp_rn((float)F.spp)));
	}
	if (err) atomicOr(err_word, err);
}

__global__ void __launch_bounds__(LBLOCK) k_legacy_rows(DevScene S, LegacyFrame F, uint32_t seed, uint32_t *mt_state,
	float *rgb, unsigned *err_word) {
	__shared__ float4 snodes[2 * SMEM_NODES];
	int nsn = min(S.n_nodes, SMEM_NODES);
	for (int i = threadIdx.x; i < 2 * nsn; i += blockDim.x) snodes[i] = __ldg(S.nodes + i);
	__syncthreads();
	uint32_t err = 0;
	int y = blockIdx.x * blockDim.x + threadIdx.x;
	if (y < F.height) {
		MtRng rng{ mt_state + y, F.height, 624 };
		rng.seed(seed + (uint32_t)y);
		for (int x = 0; x < F.width; ++x) {
			f3 d = primary_dir(F, x, y);
			f3 acc{ 0.f, 0.f, 0.f };
			for (int s = 0; s < F.spp; ++s)
				acc = radd(acc, clamp01(ltrace(S, snodes, nsn, F, ldf3(F.pos), d, rng, err)));
			store(rgb, y * F.width + x, rscl(acc, __frcp_rn((float)F.spp)));
		}
	}
	if (err) atomicOr(err_word, err);
}

}  // namespace

are_status render_legacy(are_scene *sc, const are_camera *cam, const are_render_params &p, float *rgb,
	are_render_stats *stats) {
	if (sc->dev.triangle_test != ARE_TRI_REFERENCE_MT || sc->n_spheres || sc->n_quads) {
		// the reference estimator only knows triangles (rt.cpp:110-143)
		set_error("the reference estimator needs a triangle-only scene with the reference Moller-Trumbore test");
		return ARE_ERR_INVALID_ARGUMENT;
	}
	LegacyFrame F{};
	// rt.cpp:339-343; the scale is evaluated in double as there
	float fw[3] = { cam->lookat[0] - cam->lookfrom[0], cam->lookat[1] - cam->lookfrom[1], cam->lookat[2] - cam->lookfrom[2] };
	auto nrm_h = [](float *v) {
		float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
		float r = 1.0f / l;
		v[0] = v[0] * r, v[1] = v[1] * r, v[2] = v[2] * r;
	};
	nrm_h(fw);
	float rt[3] = { fw[1] * cam->vup[2] - fw[2] * cam->vup[1], fw[2] * cam->vup[0] - fw[0] * cam->vup[2],
		fw[0] * cam->vup[1] - fw[1] * cam->vup[0] };
	nrm_h(rt);
	float up[3] = { rt[1] * fw[2] - rt[2] * fw[1], rt[2] * fw[0] - rt[0] * fw[2], rt[0] * fw[1] - rt[1] * fw[0] };
	for (int k = 0; k < 3; ++k)
		F.pos[k] = cam->lookfrom[k], F.fwd[k] = fw[k], F.right[k] = rt[k], F.up[k] = up[k], F.bg[k] = sc->dev.bg_a[k];
	F.aspect = (float)p.width / (float)p.height;
	F.scale = (float)std::tan((double)(cam->vfov_deg * 0.5f) * 3.14159265358979323846 / 180.f);
	F.width = p.width;
	F.height = p.height;
	F.spp = p.spp;

	cudaStream_t s = sc->stream;
	const bool dev_out = (p.flags & ARE_FLAG_DEVICE_OUTPUT) != 0;
	const bool mt = (p.flags & ARE_FLAG_LEGACY_MT19937) != 0;
	size_t npix = (size_t)p.width * p.height;
	size_t need = 256 + (dev_out ? 0 : npix * 12) + (mt ? (size_t)624 * p.height * 4 : 0);
	void *tmp = nullptr;
	if (are_status st = pool_alloc(sc, need, &tmp)) return st;
	unsigned *err_word = (unsigned *)tmp;
	float *d_rgb = dev_out ? rgb : (float *)((char *)tmp + 256);
	uint32_t *mt_state = (uint32_t *)((char *)tmp + 256 + (dev_out ? 0 : npix * 12));
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	cudaMemsetAsync(err_word, 0, 4, s);
	cudaGetLastError();
	cudaEventRecord(e0, s);
	if (mt) {
		k_legacy_rows<<<(p.height + LBLOCK - 1) / LBLOCK, LBLOCK, 0, s>>>(sc->dev, F, (uint32_t)p.seed, mt_state,
			d_rgb, err_word);
	} else {
		int per_sm = 0;
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)k_legacy_pixels, LBLOCK, 0);
		int grid = std::max(1, per_sm) * sc->n_sms;
		grid = (int)std::min<size_t>(grid, (npix + LBLOCK - 1) / LBLOCK);
		k_legacy_pixels<<<grid, LBLOCK, 0, s>>>(sc->dev, F, p.seed, d_rgb, err_word);
	}
	cudaEventRecord(e1, s);
	are_status st = cuda_status(cudaGetLastError(), "legacy kernel launch");
	unsigned herr = 0;
	if (!st) {
		cudaMemcpyAsync(&herr, err_word, 4, cudaMemcpyDeviceToHost, s);
		if (!dev_out) cudaMemcpyAsync(rgb, d_rgb, npix * 12, cudaMemcpyDeviceToHost, s);
		st = cuda_status(cudaStreamSynchronize(s), "legacy render");
	}
	float ms = 0.f;
	cudaEventElapsedTime(&ms, e0, e1);
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	pool_free(sc, tmp);
	if (!st && herr) {
		set_error("device error word " + std::to_string(herr));
		st = ARE_ERR_INTERNAL;
	}
	if (stats) {
		*stats = are_render_stats{};
		stats->samples = (int64_t)npix * p.spp;
		stats->device_ms = ms;
		stats->kernel_ms[ARE_KERNEL_OTHER] = ms;
		stats->kernel_launches[ARE_KERNEL_OTHER] = 1;
		stats->error_word = (int32_t)herr;
	}
	return st;
}

}  // namespace are_core
