// shade.cuh — per-hit shading math on the device: camera rays, textures,
// material scatter, counter-based random numbers.  Operation order follows
// the CPU restatement so the device and host estimators consume identical
// random numbers; transcendental functions may differ by an ulp, so the
// images agree statistically, not bit for bit.
#pragma once

#include <cuda_runtime.h>

#include "core.h"
#include "traverse.cuh"

namespace are_core {

// ---- random numbers: SplitMix64 finaliser (Steele, Lea, Flood 2014) keyed by
// (seed, pixel, sample) and a per-draw counter.  Replaces rt.cpp's per-row
// std::mt19937 seeded from std::random_device (rt.cpp:348-351).
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
	return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t path_key(uint64_t seed, uint32_t pixel, uint32_t sample) {
	return mix64(((uint64_t)pixel << 32 | (uint64_t)sample) + seed * 0xD1B54A32D192ED03ULL);
}
__device__ __forceinline__ float uniform(uint64_t key, uint32_t ctr) {
	uint32_t u = (uint32_t)(mix64(key + (uint64_t)(ctr + 1u) * 0x9E3779B97F4A7C15ULL) >> 32);
	return (float)(u >> 8) * 5.9604644775390625e-8f;
}
__device__ __forceinline__ uint32_t ctr_bounce(int b) { return 8u + 8u * (uint32_t)b; }

// ---- plain float3 helpers (shading; contraction allowed) ----
__device__ __forceinline__ f3 add(f3 a, f3 b) { return f3{ a.x + b.x, a.y + b.y, a.z + b.z }; }
__device__ __forceinline__ f3 sub(f3 a, f3 b) { return f3{ a.x - b.x, a.y - b.y, a.z - b.z }; }
__device__ __forceinline__ f3 scl(f3 a, float s) { return f3{ a.x * s, a.y * s, a.z * s }; }
__device__ __forceinline__ f3 mulv(f3 a, f3 b) { return f3{ a.x * b.x, a.y * b.y, a.z * b.z }; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
	return f3{ a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x };
}
__device__ __forceinline__ f3 norm(f3 a) { return scl(a, 1.0f / sqrtf(dot(a, a))); }
__device__ __forceinline__ f3 ldf3(const float *p) { return f3{ p[0], p[1], p[2] }; }

struct CameraFrame {
	float pos[3], fwd[3], right[3], up[3];
	float scale, aspect, lens_r, focus;
	int32_t lens, jitter;
	int32_t width, height;
};

// rt.cpp:339-343,364-366 with the pixel-centre 0.5 replaced by a jitter and
// an optional thin lens.
__device__ __forceinline__ void camera_ray(const CameraFrame &c, int px, int py, uint64_t key, f3 &o, f3 &d) {
	float jx = 0.5f, jy = 0.5f;
	if (c.jitter) {
		jx = uniform(key, 0);
		jy = uniform(key, 1);
	}
	float fx = (2.0f * ((float)px + jx) / (float)c.width - 1.0f) * c.aspect * c.scale;
	float fy = (1.0f - 2.0f * ((float)py + jy) / (float)c.height) * c.scale;
	f3 dir = add(add(ldf3(c.fwd), scl(ldf3(c.right), fx)), scl(ldf3(c.up), fy));
	if (!c.lens) {
		o = ldf3(c.pos);
		d = norm(dir);
		return;
	}
	float rr = c.lens_r * sqrtf(uniform(key, 2));
	float s, co;
	sincosf(6.28318530717958647692f * uniform(key, 3), &s, &co);
	f3 focal = add(ldf3(c.pos), scl(dir, c.focus));
	o = add(add(ldf3(c.pos), scl(ldf3(c.right), rr * co)), scl(ldf3(c.up), rr * s));
	d = norm(sub(focal, o));
}

__device__ __forceinline__ void sph_uv(f3 n, float &u, float &v) {
	const float pi = 3.14159265358979323846f;
	u = (atan2f(-n.z, n.x) + pi) / (2.0f * pi);
	v = acosf(-n.y) / pi;
}

// rt.cpp:85-102 (solid, checker) and an [y][x] texel grid (src/texture.cpp:77-83)
__device__ __forceinline__ f3 tex_eval(const DevScene &S, int ti, float u, float v, f3 p) {
	if (ti < 0 || ti >= S.n_textures) return f3{ 0.f, 0.f, 0.f };
	const DevTexture &t = S.texs[ti];
	if (t.mapping == 1) sph_uv(norm(sub(p, ldf3(t.center))), u, v);
	if (t.type == 1) {
		int xx = (int)floorf(u * t.scale), yy = (int)floorf(v * t.scale);
		return ((xx + yy) % 2 == 0) ? ldf3(t.a) : ldf3(t.b);
	}
	if (t.type == 2) {
		float fu = u > 0.f ? (u < 1.f ? u : 1.f) : 0.f;
		float fv = v > 0.f ? (v < 1.f ? v : 1.f) : 0.f;
		const float *tex = S.texels + 3 * (size_t)t.texel_offset;
		if (t.filter == 1) {
			// src/texture.cpp:310-330's bilinear weights, each operation rounded as the oracle's
			float x = __fsub_rn(__fmul_rn(fu, (float)t.width), 0.5f), y = __fsub_rn(__fmul_rn(__fsub_rn(1.0f, fv), (float)t.height), 0.5f);
			x = fminf(fmaxf(x, 0.0f), (float)(t.width - 1));
			y = fminf(fmaxf(y, 0.0f), (float)(t.height - 1));
			const int ix = (int)floorf(x), iy = (int)floorf(y);
			const int ix1 = min(ix + 1, t.width - 1), iy1 = min(iy + 1, t.height - 1);
			const float tx = __fsub_rn(x, (float)ix), ty = __fsub_rn(y, (float)iy);
			const float sx = __fsub_rn(1.0f, tx), sy = __fsub_rn(1.0f, ty);
			const float w00 = __fmul_rn(sx, sy), w10 = __fmul_rn(tx, sy), w01 = __fmul_rn(sx, ty), w11 = __fmul_rn(tx, ty);
			const float *c00 = tex + 3 * ((size_t)iy * t.width + ix), *c10 = tex + 3 * ((size_t)iy * t.width + ix1);
			const float *c01 = tex + 3 * ((size_t)iy1 * t.width + ix), *c11 = tex + 3 * ((size_t)iy1 * t.width + ix1);
			float r[3];
			for (int k = 0; k < 3; ++k)
				r[k] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(c00[k], w00), __fmul_rn(c10[k], w10)), __fmul_rn(c01[k], w01)),
					__fmul_rn(c11[k], w11));
			return f3{ r[0], r[1], r[2] };
		}
		int x = min((int)(fu * (float)t.width), t.width - 1);
		int y = min((int)((1.0f - fv) * (float)t.height), t.height - 1);
		return ldf3(tex + 3 * ((size_t)y * t.width + x));
	}
	return ldf3(t.a);
}

// rt.cpp:50-55 rotateToHemisphere frame
__device__ __forceinline__ f3 hemi(f3 n, float lx, float ly) {
	f3 up = fabsf(n.z) < 0.999f ? f3{ 0.f, 0.f, 1.f } : f3{ 1.f, 0.f, 0.f };
	f3 tg = norm(cross(n, up));
	f3 bt = cross(n, tg);
	float w = 1.0f - lx * lx - ly * ly;
	return add(add(scl(tg, lx), scl(bt, ly)), scl(n, sqrtf(w > 0.f ? w : 0.f)));
}

// are::reflect (src/basic/vec3.cpp:182-184)
__device__ __forceinline__ f3 reflect(f3 v, f3 n) { return sub(v, scl(n, 2.0f * dot(v, n))); }

__device__ __forceinline__ f3 background(const DevScene &S, f3 d) {
	if (S.background == 1) {
		float a = 0.5f * (d.y + 1.0f);
		return add(scl(ldf3(S.bg_a), 1.0f - a), scl(ldf3(S.bg_b), a));
	}
	return ldf3(S.bg_a);
}

// Geometry at a hit: position, geometric normal, material, and what the texture coordinates come
// from: (u, v) as they are (quads, triangles without per-vertex uv), the sphere's normal, or the
// barycentrics (u, v) of a triangle with per-vertex uv.  The coordinates are worked out only when a
// texture looks them up (surface_uv): most materials are solid colours.
enum : int32_t { UV_DIRECT = 0, UV_SPHERE = 1, UV_TRI_VERTEX = 2 };
struct Surface {
	f3 p, ng;
	float u, v;
	int32_t mat;
	int32_t leaf, uv_kind;
};

// the texture coordinates of a surface point (sph_uv; rt.cpp:139-142 bary2uv)
__device__ __forceinline__ void surface_uv(const DevScene &S, const Surface &sf, float &u, float &v) {
	if (sf.uv_kind == UV_SPHERE) {
		sph_uv(sf.ng, u, v);
	} else if (sf.uv_kind == UV_TRI_VERTEX) {
		const float *uv = S.tri_uv + 6 * (size_t)sf.leaf;
		const float b0 = 1.0f - sf.u - sf.v;
		u = uv[0] * b0 + uv[2] * sf.u + uv[4] * sf.v;
		v = uv[1] * b0 + uv[3] * sf.u + uv[5] * sf.v;
	} else {
		u = sf.u, v = sf.v;
	}
}

__device__ __forceinline__ Surface surface_at(const DevScene &S, int leaf, f3 o, f3 d, float t, float hu, float hv) {
	Surface sf;
	sf.p = add(o, scl(d, t));
	const float4 *P = S.prims + 3 * (size_t)leaf;
	float4 p0 = __ldg(P);
	sf.u = hu;
	sf.v = hv;
	sf.leaf = leaf;
	sf.uv_kind = UV_DIRECT;
	if (p0.w > 0.0f) {
		sf.ng = scl(sub(sf.p, ld3(p0)), 1.0f / p0.w);
		sf.uv_kind = UV_SPHERE;
	} else {
		float4 p1 = __ldg(P + 1), p2 = __ldg(P + 2);
		if (p0.w == PRIM_TAG_QUAD) {
			sf.ng = norm(cross(ld3(p1), ld3(p2)));
		} else {
			f3 v0 = ld3(p0);
			sf.ng = norm(cross(sub(ld3(p1), v0), sub(ld3(p2), v0)));
			if (S.tri_uv) sf.uv_kind = UV_TRI_VERTEX;
		}
	}
	sf.mat = __ldg(S.prim_mat + leaf);
	return sf;
}

// tex_eval at a surface point, its texture coordinates worked out only for the textures that use them
// (checker and image textures mapped by surface coordinates)
__device__ __forceinline__ f3 tex_albedo(const DevScene &S, int ti, const Surface &sf) {
	float u = 0.0f, v = 0.0f;
	if (ti >= 0 && ti < S.n_textures) {
		const DevTexture &t = S.texs[ti];
		if (t.type != ARE_TEX_SOLID && t.mapping != ARE_MAP_SPHERICAL) surface_uv(S, sf, u, v);
	}
	return tex_eval(S, ti, u, v, sf.p);
}

// One bounce of the path estimator at depth `depth`.  Returns false if the
// path ends here; on true, `nd` is the next direction and beta was updated.
// L receives emission.  Russian roulette survives with max(beta) * rr_scale
// (capped at 1); rr_scale is 1 except on guided paths, where it removes the
// guided bounces' pdf ratios from the survival probability.
__device__ __forceinline__ bool scatter(const DevScene &S, const Surface &sf, f3 d, uint64_t key, int depth,
	int rr_depth, f3 &beta, f3 &L, f3 &nd, float rr_scale = 1.0f) {
	float cosi = dot(d, sf.ng);
	bool front = cosi < 0.0f;
	f3 n = front ? sf.ng : scl(sf.ng, -1.0f);
	const DevMaterial &m = S.mats[sf.mat];
	uint32_t cb = ctr_bounce(depth);
	if (m.type == ARE_MAT_DIFFUSE_LIGHT) {
		if (front) L = add(L, mulv(beta, ldf3(m.emit)));
		return false;
	}
	if (m.type == ARE_MAT_LAMBERTIAN) {
		// rt.cpp:284-289
		float r1 = uniform(key, cb), r2 = uniform(key, cb + 1);
		float s, c;
		sincosf(6.28318530717958647692f * r1, &s, &c);
		float r2s = sqrtf(r2);
		nd = norm(hemi(n, r2s * c, r2s * s));
		beta = mulv(beta, tex_albedo(S, m.texture, sf));
	} else if (m.type == ARE_MAT_METAL) {
		f3 r = norm(reflect(d, n));
		if (m.fuzz > 0.0f) {
			float z = 1.0f - 2.0f * uniform(key, cb);
			float s, c;
			sincosf(6.28318530717958647692f * uniform(key, cb + 1), &s, &c);
			float rad = cbrtf(uniform(key, cb + 2));
			float w = 1.0f - z * z;
			float sr = sqrtf(w > 0.f ? w : 0.f);
			r = add(r, scl(f3{ sr * c, sr * s, z }, rad * m.fuzz));
		}
		if (!(dot(r, n) > 0.0f)) return false;
		nd = norm(r);
		beta = mulv(beta, tex_albedo(S, m.texture, sf));
	} else {
		float ri = front ? 1.0f / m.ior : m.ior;
		float c = -dot(d, n);
		c = c < 1.0f ? c : 1.0f;
		float sn2 = 1.0f - c * c;
		float sn = sqrtf(sn2 > 0.f ? sn2 : 0.f);
		float r0 = (1.0f - ri) / (1.0f + ri);
		r0 = r0 * r0;
		float om = 1.0f - c;
		float fr = r0 + (1.0f - r0) * (om * om * om * om * om);
		if (ri * sn > 1.0f || fr > uniform(key, cb + 2)) {
			nd = reflect(d, n);
		} else {
			// are::refract (src/basic/vec3.cpp:188-199)
			f3 perp = scl(add(d, scl(n, c)), ri);
			float k = 1.0f - dot(perp, perp);
			nd = add(perp, scl(n, -sqrtf(fabsf(k))));
		}
		nd = norm(nd);
	}
	if (rr_depth >= 0 && depth >= rr_depth) {
		// rt.cpp:304-308, survival probability capped at 1
		float q = fmaxf(fmaxf(beta.x, beta.y), beta.z) * rr_scale;
		if (q < 1.0f) {
			if (uniform(key, cb + 3) >= q) return false;
			beta = scl(beta, 1.0f / q);
		}
	}
	return true;
}

}  // namespace are_core
