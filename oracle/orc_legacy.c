/*
 * orc_legacy.c — the reference's own estimator, restated (TEST
 * INFRASTRUCTURE ONLY).
 *
 * experiments/rt.cpp render() / trace() / computeAO() (rt.cpp:221-374):
 * barycentric hit point, 32-ray ambient occlusion, a mirror bounce at depth 0
 * for MAT_METAL, 32 cosine paths of up to 3 bounces with Russian roulette for
 * MAT_DIFFUSE, clamping.  Two random streams:
 *   mode 1: rt.cpp's own — one std::mt19937 per image row seeded with
 *           seed + y (rt.cpp:348-351 with std::random_device fixed), consumed
 *           pixel after pixel through uniform_real_distribution<float>(0,1);
 *   mode 0: counter-based per pixel (orc_internal.h), draws numbered in order,
 *           so pixels are independent and parallel.
 *
 * std::mt19937 is the Mersenne Twister of Matsumoto and Nishimura (ACM TOMACS
 * 1998) with the C++ standard's parameters and seeding ([rand.predef],
 * [rand.eng.mers]).  uniform_real_distribution<float>(0,1) reduces to
 * generate_canonical<float,24> ([rand.util.canonical]): one 32-bit draw g,
 * (float)g / 2^32, and libstdc++ (GCC 13) maps a result that rounds to 1.0
 * to the largest float below 1.
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>

#include "orc_internal.h"

#define R float
#define SFX(x) x##_lg
#define RSQRT sqrtf
#define RFABS fabsf
#define RCOS cosf
#define RSIN sinf
#define RFLOOR floorf
#define RACOS acosf
#define RATAN2 atan2f
#define RCBRT cbrtf
#define RTAN tanf
#define RCOPYSIGN copysignf
#include "orc_core.inc"

/* ---- std::mt19937 ---------------------------------------------------------- */

typedef struct {
	uint32_t x[624];
	int i;
} mt19937;

static void mt_seed(mt19937 *m, uint32_t s) {
	m->x[0] = s;
	for (int k = 1; k < 624; ++k) m->x[k] = 1812433253u * (m->x[k - 1] ^ (m->x[k - 1] >> 30)) + (uint32_t)k;
	m->i = 624;
}

static uint32_t mt_next(mt19937 *m) {
	if (m->i >= 624) {
		for (int k = 0; k < 624; ++k) {
			uint32_t y = (m->x[k] & 0x80000000u) | (m->x[(k + 1) % 624] & 0x7fffffffu);
			m->x[k] = m->x[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
		}
		m->i = 0;
	}
	uint32_t y = m->x[m->i++];
	y ^= y >> 11;
	y ^= (y << 7) & 0x9d2c5680u;
	y ^= (y << 15) & 0xefc60000u;
	y ^= y >> 18;
	return y;
}

static float mt_canonical(mt19937 *m) {
	float r = (float)mt_next(m) / 4294967296.0f;
	if (r >= 1.0f) r = nextafterf(1.0f, 0.0f);
	return r;
}

void orc_mt19937(uint32_t seed, int64_t n, uint32_t *out, float *canon) {
	mt19937 m;
	mt_seed(&m, seed);
	for (int64_t k = 0; k < n; ++k) out[k] = mt_next(&m);
	mt_seed(&m, seed);
	for (int64_t k = 0; canon && k < n; ++k) canon[k] = mt_canonical(&m);
}

typedef struct {
	int mode;
	mt19937 *mt;
	uint64_t key;
	uint32_t ctr;
} lrng;

static float draw(lrng *r) {
	if (r->mode == 1) return mt_canonical(r->mt);
	return orc_uniform(r->key, r->ctr++);
}

/* ---- rt.cpp's estimator ------------------------------------------------------ */

#define LEPS 1e-5f /* rt.cpp:15 */
#define LINF 1e30f /* rt.cpp:16 */

typedef struct {
	v3_lg c;
} col;

static v3_lg clamp01(v3_lg c) {
	c.x = fmaxf(0.0f, fminf(1.0f, c.x));
	c.y = fmaxf(0.0f, fminf(1.0f, c.y));
	c.z = fmaxf(0.0f, fminf(1.0f, c.z));
	return c;
}

/* Tri of the hit: vertices, normal (rt.cpp:121), bary point (rt.cpp:258),
 * texture colour (rt.cpp:259-261), material tag and metal parameters. */
typedef struct {
	v3_lg p, n, albedo;
	int metal;
	float reflect_ratio;
	v3_lg tint;
} lhit;

static void surface(const orc_ctx *ctx, const hit_lg *h, lhit *o) {
	const orc_scene *s = &ctx->s;
	int32_t li;
	orc_prim_type(s, h->prim, &li);
	const float *tv = s->triangles + 9 * (int64_t)li;
	v3_lg v0 = ld3_lg(tv), v1 = ld3_lg(tv + 3), v2 = ld3_lg(tv + 6);
	o->n = norm_lg(cross_lg(sub_lg(v1, v0), sub_lg(v2, v0)));
	float b0 = 1 - h->u - h->v;
	o->p = add_lg(add_lg(scl_lg(v0, b0), scl_lg(v1, h->u)), scl_lg(v2, h->v));
	float tu = 0, tw = 0;
	if (s->triangle_uv) {
		const float *uv = s->triangle_uv + 6 * (int64_t)li;
		tu = uv[0] * b0 + uv[2] * h->u + uv[4] * h->v;
		tw = uv[1] * b0 + uv[3] * h->u + uv[5] * h->v;
	}
	const orc_material *m = &s->materials[s->triangle_mat[li]];
	o->albedo = tex_eval_lg(s, m->texture, tu, tw, o->p);
	o->metal = m->type == 1;
	o->reflect_ratio = m->reflect_ratio;
	o->tint = ld3_lg(m->tint);
}

/* rt.cpp:221-248 computeAO */
static float compute_ao(const orc_ctx *ctx, v3_lg p, v3_lg n, lrng *rng) {
	const int N = 32;
	int unoccluded = 0;
	for (int i = 0; i < N; ++i) {
		float u = draw(rng), v = draw(rng);
		float theta = (float)(2 * 3.14159265358979323846 * (double)u);
		float phi = acosf(1 - 2 * v);
		float x = sinf(phi) * cosf(theta);
		float y = sinf(phi) * sinf(theta);
		float z = cosf(phi);
		if (z < 0) z = -z;
		v3_lg hemi = mk_lg(x, y, z);
		v3_lg zax = mk_lg(0, 0, 1);
		v3_lg axis = cross_lg(zax, n);
		float sa = sqrtf(dot_lg(axis, axis)), ca = dot_lg(zax, n);
		v3_lg d = hemi;
		if (sa > LEPS) {
			axis = norm_lg(axis);
			float ang = acosf(ca);
			d = add_lg(add_lg(scl_lg(d, cosf(ang)), scl_lg(cross_lg(axis, d), sinf(ang))),
				scl_lg(scl_lg(axis, dot_lg(axis, d)), 1 - cosf(ang)));
		}
		d = norm_lg(d);
		hit_lg h = closest_lg(ctx, add_lg(p, scl_lg(n, LEPS)), d, LEPS, LINF);
		if (h.prim == -1) unoccluded++;
	}
	return 0.25f + 0.75f * (unoccluded / (float)N);
}

/* rt.cpp:251-334 trace */
static v3_lg legacy_trace(const orc_ctx *ctx, v3_lg o, v3_lg d, lrng *rng, int depth) {
	hit_lg rec = closest_lg(ctx, o, d, LEPS, LINF);
	if (rec.prim == -1) return ld3_lg(ctx->s.bg_a);
	lhit t;
	surface(ctx, &rec, &t);
	v3_lg albedo = t.albedo;
	float ao = compute_ao(ctx, t.p, t.n, rng);
	if (t.metal && depth == 0) {
		v3_lg view = norm_lg(sub_lg(o, t.p));
		v3_lg refl = sub_lg(view, scl_lg(scl_lg(t.n, 2), dot_lg(view, t.n)));
		v3_lg reflected = legacy_trace(ctx, add_lg(t.p, scl_lg(t.n, LEPS)), refl, rng, depth + 1);
		v3_lg ret = add_lg(scl_lg(albedo, 1 - t.reflect_ratio), mulv_lg(scl_lg(reflected, t.reflect_ratio), t.tint));
		ret = scl_lg(ret, ao);
		return clamp01(ret);
	}
	if (!t.metal) {
		const int samples = 32, max_bounce = 3;
		v3_lg accum = mk_lg(0, 0, 0);
		for (int s = 0; s < samples; ++s) {
			float r1 = draw(rng), r2 = draw(rng);
			float phi = (float)(2 * 3.14159265358979323846 * (double)r1);
			float r2s = sqrtf(r2);
			v3_lg local = mk_lg(r2s * cosf(phi), r2s * sinf(phi), sqrtf(1 - r2));
			v3_lg world = hemi_lg(t.n, local.x, local.y);
			v3_lg new_origin = add_lg(t.p, scl_lg(t.n, LEPS));
			v3_lg throughput = albedo;
			int b = 0;
			v3_lg dir = world;
			while (b < max_bounce) {
				hit_lg br = closest_lg(ctx, new_origin, dir, LEPS, LINF);
				if (br.prim == -1) break;
				lhit bt;
				surface(ctx, &br, &bt);
				throughput = mulv_lg(throughput, bt.albedo);
				float pr = fmaxf(throughput.x, fmaxf(throughput.y, throughput.z));
				if (draw(rng) > pr) break;
				throughput = scl_lg(throughput, 1 / pr);
				v3_lg nd;
				if (bt.metal) {
					v3_lg view = norm_lg(sub_lg(mk_lg(0, 0, 0), dir));
					nd = sub_lg(view, scl_lg(scl_lg(bt.n, 2), dot_lg(view, bt.n)));
				} else {
					float nr1 = draw(rng), nr2 = draw(rng);
					float nphi = (float)(2 * 3.14159265358979323846 * (double)nr1);
					float nr2s = sqrtf(nr2);
					nd = hemi_lg(bt.n, nr2s * cosf(nphi), nr2s * sinf(nphi));
				}
				new_origin = add_lg(bt.p, scl_lg(bt.n, LEPS));
				dir = nd;
				b++;
			}
			accum = add_lg(accum, throughput);
		}
		albedo = add_lg(albedo, scl_lg(accum, 1.0f / samples));
	}
	albedo = scl_lg(albedo, ao);
	return clamp01(albedo);
}

typedef struct {
	const orc_ctx *ctx;
	const orc_camera *cam;
	const orc_params *p;
	float *rgb;
	int mode, tid, nt;
	uint32_t mt_seed;
	int64_t rays;
} ljob;

static void *legacy_worker(void *arg) {
	ljob *j = (ljob *)arg;
	const orc_params *p = j->p;
	/* rt.cpp:339-343 camera basis; the scale is computed in double as there */
	v3_lg pos = ld3_lg(j->cam->lookfrom);
	v3_lg fwd = norm_lg(sub_lg(ld3_lg(j->cam->lookat), pos));
	v3_lg right = norm_lg(cross_lg(fwd, ld3_lg(j->cam->vup)));
	v3_lg up = cross_lg(right, fwd);
	float aspect = (float)p->width / p->height;
	float scale = (float)tan((double)(j->cam->vfov_deg * 0.5f) * 3.14159265358979323846 / 180.f);
	mt19937 *mt = (mt19937 *)malloc(sizeof(mt19937));
	for (int y = j->tid; y < p->height; y += j->nt) {
		mt_seed(mt, j->mt_seed + (uint32_t)y);
		for (int x = 0; x < p->width; ++x) {
			uint32_t pix = (uint32_t)y * (uint32_t)p->width + (uint32_t)x;
			lrng rng = { j->mode, mt, orc_key(p->seed, pix, 0), 0 };
			float fx = (2 * (x + 0.5f) / p->width - 1) * aspect * scale;
			float fy = (1 - 2 * (y + 0.5f) / p->height) * scale;
			v3_lg dir = norm_lg(add_lg(add_lg(fwd, scl_lg(right, fx)), scl_lg(up, fy)));
			v3_lg acc = mk_lg(0, 0, 0);
			for (int s = 0; s < p->spp; ++s) acc = add_lg(acc, clamp01(legacy_trace(j->ctx, pos, dir, &rng, 0)));
			acc = scl_lg(acc, 1.0f / p->spp);
			j->rgb[3 * (int64_t)pix] = acc.x;
			j->rgb[3 * (int64_t)pix + 1] = acc.y;
			j->rgb[3 * (int64_t)pix + 2] = acc.z;
		}
	}
	free(mt);
	return NULL;
}

/* rng_mode 1: rt.cpp's per-row mt19937 seeded mt_seed + y; 0: counter-based
 * keyed by params->seed.  rgb: width*height*3, row-major from the top. */
int32_t orc_render_legacy(const orc_ctx *ctx, const orc_camera *cam, const orc_params *p, float *rgb, int32_t rng_mode,
	uint32_t mt_seed, int32_t nthreads) {
	if (!ctx || !cam || !p || !rgb || p->width <= 0 || p->height <= 0 || p->spp <= 0) return 1;
	if (nthreads < 1) nthreads = 1;
	ljob *jobs = (ljob *)calloc((size_t)nthreads, sizeof(ljob));
	pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
	if (!jobs || !th) {
		free(jobs);
		free(th);
		return 2;
	}
	for (int t = 0; t < nthreads; ++t) {
		jobs[t] = (ljob){ ctx, cam, p, rgb, rng_mode, t, nthreads, mt_seed, 0 };
		pthread_create(&th[t], NULL, legacy_worker, &jobs[t]);
	}
	for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
	free(jobs);
	free(th);
	return 0;
}
