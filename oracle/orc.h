/*
 * orc.h — CPU oracle for the per-pixel render loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * render loop (experiments/rt.cpp:209-374 and the scene math of
 * src/basic/vec3.cpp) extended with the primitives and materials the
 * synthetic workloads need.  The tests and the CPU baseline of the benchmark
 * use it as the checker; the product never links or calls it.
 *
 * Parity pins (see tests/test_oracle_pin.py):
 *  - triangle Möller–Trumbore + closest-hit scan: bit-exact against the
 *    reference's own Tri::intersect / intersect() (rt.cpp:123-138, 209-218)
 *    compiled from its sources into oracle/_ref;
 *  - checker/solid textures (rt.cpp:85-102), the hemisphere frame
 *    (rt.cpp:50-55), reflect/refract (src/basic/vec3.cpp:182-199) and the PPM
 *    quantisation (rt.cpp:377-392): against oracle/_ref and committed fixtures.
 *  - sphere, quad, watertight triangle, dielectric, emission and the thin lens
 *    have no reference code: parity for those is unpinned by the reference and
 *    is anchored on analytic known-answer tests instead.
 *
 * The scene / camera / params structs have the same memory layout as the
 * product's are_scene_desc / are_camera / are_render_params so one set of
 * arrays feeds both sides.
 */
#ifndef ORC_H
#define ORC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_material {
	int32_t type; /* 0 lambertian, 1 metal, 2 dielectric, 3 diffuse light */
	int32_t texture;
	float fuzz;
	float ior;
	float emit[3];
	float reflect_ratio;
	float tint[3];
	float pad_;
} orc_material;

typedef struct orc_texture {
	int32_t type; /* 0 solid, 1 checker, 2 image */
	int32_t mapping; /* 0 surface uv, 1 spherical about center */
	float scale;
	int32_t width, height;
	int32_t texel_offset;
	float a[3];
	float b[3];
	float center[3];
	int32_t filter; /* image: 0 nearest, 1 bilinear */
} orc_texture;

typedef struct orc_scene {
	int32_t n_spheres;
	const float *spheres;
	const int32_t *sphere_mat;
	int32_t n_quads;
	const float *quads;
	const int32_t *quad_mat;
	int32_t n_triangles;
	const float *triangles;
	const float *triangle_uv;
	const int32_t *triangle_mat;
	int32_t n_materials;
	const orc_material *materials;
	int32_t n_textures;
	const orc_texture *textures;
	int64_t n_texels;
	const float *texels;
	int32_t background;
	float bg_a[3];
	float bg_b[3];
	int32_t triangle_test; /* 0 reference Möller–Trumbore, 1 watertight */
	int32_t bvh_leaf_size;
} orc_scene;

typedef struct orc_camera {
	float lookfrom[3];
	float lookat[3];
	float vup[3];
	float vfov_deg;
	float aperture;
	float focus_dist;
} orc_camera;

typedef struct orc_params {
	int32_t width, height;
	int32_t spp;
	int32_t max_depth;
	uint64_t seed;
	int32_t rr_depth;
	float t_min;
	int32_t estimator;
	int32_t flags; /* 2 = no jitter, 4 = clamp output */
	int32_t pool_size;
	int32_t chunk;
	int32_t block_size;
	int32_t reserved_;
} orc_params;

typedef struct orc_stats {
	int64_t samples;
	int64_t segments;
} orc_stats;

typedef struct orc_ctx orc_ctx; /* scene + optional acceleration structure */

/* Prepares a scene for queries.  accel: 0 = linear scan over all primitives
 * in id order (the reference's own strategy, rt.cpp:211), 1 = the oracle's
 * median-split BVH (same results: closest t, lower id on ties), -1 = auto
 * (BVH above 64 primitives).  The scene arrays must outlive the context. */
orc_ctx *orc_prepare(const orc_scene *scene, int32_t accel);
void orc_release(orc_ctx *ctx);

/* Closest hit per ray.  rays: n x 8 (o, t_min, d, t_max); hits: n x 4
 * (t, prim id bits, u, v), id -1 / t=+inf on a miss.  FP32 arithmetic. */
int32_t orc_intersect_f32(const orc_ctx *ctx, const float *rays, int64_t n, float *hits, int32_t nthreads);

/* Path-traced render of width x height pixels with spp samples.  mean and
 * var (variance of the mean) are width*height*3 floats.  Rows are split
 * across nthreads host threads.  rows [row0, row1) only; row1 <= 0 means all. */
int32_t orc_render_f32(const orc_ctx *ctx, const orc_camera *cam, const orc_params *p, float *mean, float *var,
	int32_t row0, int32_t row1, int32_t nthreads, orc_stats *stats);
int32_t orc_render_f64(const orc_ctx *ctx, const orc_camera *cam, const orc_params *p, double *mean, double *var,
	int32_t row0, int32_t row1, int32_t nthreads, orc_stats *stats);

/* Single-path helpers exposed for known-answer tests. */
uint32_t orc_rng_u32(uint64_t key, uint32_t ctr);
uint64_t orc_path_key(uint64_t seed, uint32_t pixel, uint32_t sample);
void orc_texture_eval_f32(const orc_ctx *ctx, int32_t tex, float u, float v, const float *p, float *rgb);
void orc_hemisphere_f32(const float *n, float u, float v, float *dir); /* rt.cpp:50-55 frame */
void orc_reflect_f64(const double *v, const double *n, double *out);
void orc_refract_f64(const double *uv, const double *n, double eta, double *out);
void orc_ppm_quantize(const float *rgb, int64_t n, float gamma, uint8_t *out); /* rt.cpp:384-386 */
void orc_texture_quantize(const float *rgb, int64_t n, uint8_t *out);          /* texture.cpp:378-383 */

/* The reference's own estimator, rt.cpp trace()/computeAO() (rt.cpp:221-374).
 * rng_mode 1: rt.cpp's per-row std::mt19937 seeded mt_seed + y; rng_mode 0:
 * counter-based per pixel keyed by p->seed.  rgb: width*height*3. */
int32_t orc_render_legacy(const orc_ctx *ctx, const orc_camera *cam, const orc_params *p, float *rgb, int32_t rng_mode,
	uint32_t mt_seed, int32_t nthreads);
/* Path-guiding network in FP64 (orc_guide.c): parameters are one flat float array. */
int32_t orc_guide_num_params(void);
void orc_guide_encode(const double *x, double *e);
void orc_guide_forward(const float *params, const float *feat, int64_t n, double *out);
double orc_guide_pdf(const double *o48, const double *w);
double orc_guide_loss_grad(const float *params, const float *samples, int64_t n, double *grad);
void orc_guide_adam(float *params, float *m, float *v, const double *grad, int64_t step, double lr, double b1, double b2,
	double eps);
/* std::mt19937(seed): n raw outputs and n uniform_real_distribution<float>(0,1) draws */
void orc_mt19937(uint32_t seed, int64_t n, uint32_t *out, float *canon);

#ifdef __cplusplus
}
#endif

#endif
