/*
 * orc_f64.c — FP64 instantiation of the oracle (TEST INFRASTRUCTURE ONLY):
 * the same estimator and random numbers in double precision, used as the
 * high-precision reference render.
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>

#include "orc_internal.h"

#define R double
#define SFX(x) x##_f64
#define RSQRT sqrt
#define RFABS fabs
#define RCOS cos
#define RSIN sin
#define RFLOOR floor
#define RACOS acos
#define RATAN2 atan2
#define RCBRT cbrt
#define RTAN tan
#define RCOPYSIGN copysign
#include "orc_core.inc"

int32_t orc_render_f64(const orc_ctx *ctx, const orc_camera *cam, const orc_params *p, double *mean, double *var,
	int32_t row0, int32_t row1, int32_t nthreads, orc_stats *stats) {
	return orc_render_impl_f64(ctx, cam, p, mean, var, row0, row1, nthreads, stats);
}
