/*
 * orc_f32.c — FP32 instantiation of the oracle (TEST INFRASTRUCTURE ONLY).
 * Compiled with -ffp-contract=off: every operation rounds on its own.
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>

#include "orc_internal.h"

#define R float
#define SFX(x) x##_f32
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

static void *intersect_worker(void *arg) {
	job_f32 *j = (job_f32 *)arg;
	for (int64_t i = j->tid; i < j->n; i += j->nt) {
		const float *r = j->rays + 8 * i;
		v3_f32 o = mk_f32(r[0], r[1], r[2]), d = mk_f32(r[4], r[5], r[6]);
		hit_f32 h = closest_f32(j->ctx, o, d, r[3], r[7]);
		float *out = j->hits + 4 * i;
		union {
			int32_t i;
			float f;
		} id;
		id.i = h.prim;
		out[0] = h.t;
		out[1] = id.f;
		out[2] = h.u;
		out[3] = h.v;
	}
	return NULL;
}

int32_t orc_intersect_f32(const orc_ctx *ctx, const float *rays, int64_t n, float *hits, int32_t nthreads) {
	if (!ctx || (n > 0 && (!rays || !hits)) || n < 0)
		return 1;
	if (nthreads < 1)
		nthreads = 1;
	job_f32 *jobs = (job_f32 *)calloc((size_t)nthreads, sizeof(job_f32));
	pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
	for (int t = 0; t < nthreads; ++t) {
		jobs[t].ctx = ctx;
		jobs[t].rays = rays;
		jobs[t].hits = hits;
		jobs[t].n = n;
		jobs[t].tid = t;
		jobs[t].nt = nthreads;
		pthread_create(&th[t], NULL, intersect_worker, &jobs[t]);
	}
	for (int t = 0; t < nthreads; ++t)
		pthread_join(th[t], NULL);
	free(jobs);
	free(th);
	return 0;
}

int32_t orc_render_f32(const orc_ctx *ctx, const orc_camera *cam, const orc_params *p, float *mean, float *var,
	int32_t row0, int32_t row1, int32_t nthreads, orc_stats *stats) {
	return orc_render_impl_f32(ctx, cam, p, mean, var, row0, row1, nthreads, stats);
}

void orc_texture_eval_f32(const orc_ctx *ctx, int32_t tex, float u, float v, const float *p, float *rgb) {
	v3_f32 c = tex_eval_f32(&ctx->s, tex, u, v, mk_f32(p[0], p[1], p[2]));
	rgb[0] = c.x;
	rgb[1] = c.y;
	rgb[2] = c.z;
}

void orc_hemisphere_f32(const float *n, float u, float v, float *dir) {
	v3_f32 d = hemi_f32(mk_f32(n[0], n[1], n[2]), u, v);
	dir[0] = d.x;
	dir[1] = d.y;
	dir[2] = d.z;
}
