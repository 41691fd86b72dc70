/*
 * orc_common.c — oracle context, acceleration structure and small helpers.
 * TEST INFRASTRUCTURE ONLY: the checker for the device core, never shipped.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "orc_internal.h"

uint32_t orc_rng_u32(uint64_t key, uint32_t ctr) {
	return orc_u32(key, ctr);
}
uint64_t orc_path_key(uint64_t seed, uint32_t pixel, uint32_t sample) {
	return orc_key(seed, pixel, sample);
}

/* ---- primitive bounds (double, conservative) ------------------------------ */

static void prim_bounds(const orc_scene *s, int32_t id, double lo[3], double hi[3]) {
	int32_t i;
	int t = orc_prim_type(s, id, &i);
	if (t == 0) {
		const float *p = s->spheres + 4 * (int64_t)i;
		double r = fabs((double)p[3]);
		for (int k = 0; k < 3; ++k) {
			lo[k] = (double)p[k] - r;
			hi[k] = (double)p[k] + r;
		}
	} else if (t == 1) {
		const float *q = s->quads + 9 * (int64_t)i;
		for (int k = 0; k < 3; ++k) {
			double c0 = q[k], c1 = (double)q[k] + q[3 + k], c2 = (double)q[k] + q[6 + k],
				   c3 = (double)q[k] + q[3 + k] + q[6 + k];
			lo[k] = fmin(fmin(c0, c1), fmin(c2, c3));
			hi[k] = fmax(fmax(c0, c1), fmax(c2, c3));
		}
	} else {
		const float *v = s->triangles + 9 * (int64_t)i;
		for (int k = 0; k < 3; ++k) {
			lo[k] = fmin(fmin((double)v[k], (double)v[3 + k]), (double)v[6 + k]);
			hi[k] = fmax(fmax((double)v[k], (double)v[3 + k]), (double)v[6 + k]);
		}
	}
}

/* ---- median-split BVH ------------------------------------------------------
 * Independent of the product's SAH builder on purpose: any correct
 * acceleration structure returns the same closest hit (smallest t, lower id on
 * equal t) as the linear scan, so agreement between the two is evidence about
 * the traversal, not a shared bug. */

typedef struct build_ref {
	double c[3];
	double lo[3], hi[3];
	int32_t id;
} build_ref;

static int g_sort_axis;
static int cmp_ref(const void *a, const void *b) {
	const build_ref *x = (const build_ref *)a, *y = (const build_ref *)b;
	double cx = x->c[g_sort_axis], cy = y->c[g_sort_axis];
	if (cx < cy)
		return -1;
	if (cx > cy)
		return 1;
	return (x->id > y->id) - (x->id < y->id);
}

static int32_t build_rec(orc_ctx *ctx, build_ref *refs, int32_t first, int32_t count, int32_t leaf) {
	int32_t me = ctx->n_nodes++;
	orc_node *n = &ctx->nodes[me];
	for (int k = 0; k < 3; ++k) {
		n->bmin[k] = INFINITY;
		n->bmax[k] = -INFINITY;
	}
	double clo[3] = { INFINITY, INFINITY, INFINITY }, chi[3] = { -INFINITY, -INFINITY, -INFINITY };
	for (int32_t i = first; i < first + count; ++i)
		for (int k = 0; k < 3; ++k) {
			n->bmin[k] = fmin(n->bmin[k], refs[i].lo[k]);
			n->bmax[k] = fmax(n->bmax[k], refs[i].hi[k]);
			clo[k] = fmin(clo[k], refs[i].c[k]);
			chi[k] = fmax(chi[k], refs[i].c[k]);
		}
	/* conservative padding: far larger than any FP32 rounding of a hit t */
	for (int k = 0; k < 3; ++k) {
		double mag = fmax(fabs(n->bmin[k]), fabs(n->bmax[k]));
		double pad = 1e-5 * mag + 1e-5 * (n->bmax[k] - n->bmin[k]) + 1e-30;
		n->bmin[k] -= pad;
		n->bmax[k] += pad;
	}
	if (count <= leaf) {
		n->left = n->right = -1;
		n->first = first;
		n->count = count;
		return me;
	}
	int axis = 0;
	for (int k = 1; k < 3; ++k)
		if (chi[k] - clo[k] > chi[axis] - clo[axis])
			axis = k;
	g_sort_axis = axis;
	qsort(refs + first, (size_t)count, sizeof(build_ref), cmp_ref);
	int32_t half = count / 2;
	int32_t l = build_rec(ctx, refs, first, half, leaf);
	int32_t r = build_rec(ctx, refs, first + half, count - half, leaf);
	n = &ctx->nodes[me];
	n->left = l;
	n->right = r;
	n->first = 0;
	n->count = 0;
	return me;
}

orc_ctx *orc_prepare(const orc_scene *scene, int32_t accel) {
	orc_ctx *ctx = (orc_ctx *)calloc(1, sizeof(orc_ctx));
	if (!ctx)
		return NULL;
	ctx->s = *scene;
	ctx->n_prims = scene->n_spheres + scene->n_quads + scene->n_triangles;
	ctx->use_bvh = accel < 0 ? (ctx->n_prims > 64) : accel;
	if (!ctx->use_bvh || ctx->n_prims == 0) {
		ctx->use_bvh = 0;
		return ctx;
	}
	build_ref *refs = (build_ref *)malloc(sizeof(build_ref) * (size_t)ctx->n_prims);
	ctx->nodes = (orc_node *)malloc(sizeof(orc_node) * (size_t)(2 * ctx->n_prims + 1));
	ctx->prim_ids = (int32_t *)malloc(sizeof(int32_t) * (size_t)ctx->n_prims);
	if (!refs || !ctx->nodes || !ctx->prim_ids) {
		free(refs);
		orc_release(ctx);
		return NULL;
	}
	for (int32_t i = 0; i < ctx->n_prims; ++i) {
		refs[i].id = i;
		prim_bounds(scene, i, refs[i].lo, refs[i].hi);
		for (int k = 0; k < 3; ++k)
			refs[i].c[k] = 0.5 * (refs[i].lo[k] + refs[i].hi[k]);
	}
	build_rec(ctx, refs, 0, ctx->n_prims, 4);
	for (int32_t i = 0; i < ctx->n_prims; ++i)
		ctx->prim_ids[i] = refs[i].id;
	free(refs);
	return ctx;
}

void orc_release(orc_ctx *ctx) {
	if (!ctx)
		return;
	free(ctx->nodes);
	free(ctx->prim_ids);
	free(ctx);
}

/* ---- helpers restating reference formulas --------------------------------- */

/* are::reflect, src/basic/vec3.cpp:182-184: v - 2 (v.n) n */
void orc_reflect_f64(const double *v, const double *n, double *out) {
	double k = 2 * (v[0] * n[0] + v[1] * n[1] + v[2] * n[2]);
	for (int i = 0; i < 3; ++i)
		out[i] = v[i] - k * n[i];
}

/* are::refract, src/basic/vec3.cpp:188-199.  The reference takes the
 * absolute value inside the square root, so its NaN-on-total-internal-
 * reflection branch is only reached for non-finite input; restated as is. */
void orc_refract_f64(const double *uv, const double *n, double eta, double *out) {
	double cos_t = fmin(-(uv[0] * n[0] + uv[1] * n[1] + uv[2] * n[2]), 1.0);
	double perp[3], par[3];
	for (int i = 0; i < 3; ++i)
		perp[i] = eta * (uv[i] + cos_t * n[i]);
	double l2 = perp[0] * perp[0] + perp[1] * perp[1] + perp[2] * perp[2];
	double k = -sqrt(fabs(1.0 - l2));
	for (int i = 0; i < 3; ++i)
		par[i] = k * n[i];
	double len = sqrt(par[0] * par[0] + par[1] * par[1] + par[2] * par[2]);
	if (isnan(len) || isinf(len)) {
		out[0] = out[1] = out[2] = NAN;
		return;
	}
	for (int i = 0; i < 3; ++i)
		out[i] = perp[i] + par[i];
}

/* writePPM quantisation, rt.cpp:377-392: clamp to [0,1], pow(c, 1/gamma),
 * times 255, truncate to unsigned char. */
/* are::Texture::save_texture (src/texture.cpp:378-383): the FP64 image value
 * times 255.0, clamped to [0, 255], truncated.  The image is FP32 here, so
 * the product is exact; NaN (undefined in the reference) gives 0. */
void orc_texture_quantize(const float *rgb, int64_t n, uint8_t *out) {
	for (int64_t i = 0; i < n; ++i) {
		double v = (double)rgb[i] * 255.0;
		if (v != v) v = 0.0;
		v = v < 0.0 ? 0.0 : (v > 255.0 ? 255.0 : v);
		out[i] = (uint8_t)v;
	}
}

void orc_ppm_quantize(const float *rgb, int64_t n, float gamma, uint8_t *out) {
	for (int64_t i = 0; i < n; ++i) {
		float c = rgb[i];
		c = fmaxf(0.0f, fminf(1.0f, c));
		out[i] = (uint8_t)(powf(c, 1 / gamma) * 255);
	}
}
