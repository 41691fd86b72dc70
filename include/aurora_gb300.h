/*
 * aurora_gb300.h — C ABI of the GB300 path-tracing core.
 *
 * This is the drop-in boundary for the reference's per-pixel render loop.
 * The reference has no FFI of its own; the call it replaces is
 *
 *     void render(const Scene&, const Vec3& camPos, const Vec3& camTarget,
 *                 const Vec3& camUp, float fov, Viewport& vp)
 *
 * in experiments/rt.cpp:337-374, which walks every pixel, builds the camera
 * ray (rt.cpp:339-343,364-366), calls trace() (rt.cpp:251-334) and stores the
 * clamped colour (rt.cpp:368-369).  The scene the reference renders is a
 * caller-owned list of triangles with a material tag and a texture pointer
 * each (rt.cpp:110-186); the library's scene types are are::ObjectSet /
 * are::Triangle / are::Material / are::Texture (include/object/object_set.h:10-12,
 * include/object/triangle.h:15-46, include/material/material.h:10-29,
 * include/texture.h:9-31).
 *
 * Conventions
 *  - Plain C types only; every pointer is caller-owned unless stated.
 *  - Errors are returned as are_status codes, never thrown.  are_last_error()
 *    gives a human-readable message for the calling thread's last failure.
 *  - A scene handle is immutable after creation and may be rendered from one
 *    host thread at a time (renders on one handle are serialised by the caller).
 *  - Primitive ids are global: spheres first, then quads, then triangles, in
 *    the order of the descriptor's arrays.  Closest-hit ties (equal t) go to
 *    the lower id, as rt.cpp:209-218 keeps the first triangle on equal t.
 */
#ifndef AURORA_GB300_H
#define AURORA_GB300_H

#include <stdint.h>

#if defined(_WIN32)
#define ARE_API __declspec(dllexport)
#else
#define ARE_API __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum are_status {
	ARE_OK = 0,
	ARE_ERR_INVALID_ARGUMENT = 1, /* malformed descriptor, bad sizes, null pointers */
	ARE_ERR_CUDA = 2,             /* a CUDA runtime call failed */
	ARE_ERR_OUT_OF_MEMORY = 3,    /* device or host allocation failed */
	ARE_ERR_NO_DEVICE = 4,        /* no usable sm_103 device */
	ARE_ERR_KERNEL_TIMEOUT = 5,   /* a bounded device-side wait gave up */
	ARE_ERR_INTERNAL = 6,         /* device error word set (queue overflow, bad index) */
	ARE_ERR_IO = 7                /* an image file could not be opened, read or written */
} are_status;

/* ---- scene description (flat arrays, copied by are_scene_create) -------- */

enum { ARE_MAT_LAMBERTIAN = 0, ARE_MAT_METAL = 1, ARE_MAT_DIELECTRIC = 2, ARE_MAT_DIFFUSE_LIGHT = 3 };
enum { ARE_TEX_SOLID = 0, ARE_TEX_CHECKER = 1, ARE_TEX_IMAGE = 2 };
enum { ARE_MAP_SURFACE_UV = 0, ARE_MAP_SPHERICAL = 1 };
enum { ARE_BG_CONSTANT = 0, ARE_BG_SKY_GRADIENT = 1 };
enum { ARE_TRI_REFERENCE_MT = 0, ARE_TRI_WATERTIGHT = 1 };

/* 48 bytes.  Material kinds follow rt.cpp's MaterialType (rt.cpp:104-107:
 * MAT_DIFFUSE -> LAMBERTIAN, MAT_METAL -> METAL) and the library's
 * Diffuse / Reflective (src/material/diffuse.cpp, src/material/reflective.cpp);
 * DIELECTRIC and DIFFUSE_LIGHT have no counterpart in the reference. */
typedef struct are_material {
	int32_t type;            /* ARE_MAT_* */
	int32_t texture;         /* index into textures (albedo); -1 = none (black) */
	float fuzz;              /* METAL: radius of the random perturbation, [0,1] */
	float ior;               /* DIELECTRIC: index of refraction */
	float emit[3];           /* DIFFUSE_LIGHT: radiance emitted from the front face */
	float reflect_ratio;     /* legacy estimator: rt.cpp Tri::reflect_ratio */
	float tint[3];           /* legacy estimator: rt.cpp Tri::metal_tint */
	float pad_;
} are_material;

/* 64 bytes.  SOLID and CHECKER follow rt.cpp:85-102; IMAGE samples an
 * RGB texel grid addressed [y][x] like are::Texture::pixel (src/texture.cpp:77-83). */
typedef struct are_texture {
	int32_t type;            /* ARE_TEX_* */
	int32_t mapping;         /* ARE_MAP_* : where (u,v) comes from */
	float scale;             /* CHECKER: cells per unit of u and v */
	int32_t width, height;   /* IMAGE: texel grid size */
	int32_t texel_offset;    /* IMAGE: first texel (RGB float triple) in texels[] */
	float a[3];              /* SOLID colour / CHECKER even cells */
	float b[3];              /* CHECKER odd cells */
	float center[3];         /* SPHERICAL mapping: centre of the sphere */
	int32_t filter;          /* IMAGE: ARE_FILTER_NEAREST (Texture::pixel, src/texture.cpp:77-83) or
	                            ARE_FILTER_BILINEAR (the weights of src/texture.cpp:310-330; texel centres
	                            at i + 1/2, coordinates clamped to the grid) */
} are_texture;

enum { ARE_FILTER_NEAREST = 0, ARE_FILTER_BILINEAR = 1 };

typedef struct are_scene_desc {
	int32_t n_spheres;
	const float *spheres;       /* n_spheres x 4: centre xyz, radius */
	const int32_t *sphere_mat;  /* n_spheres material indices */
	int32_t n_quads;
	const float *quads;         /* n_quads x 9: corner Q, edge u, edge v */
	const int32_t *quad_mat;
	int32_t n_triangles;
	const float *triangles;     /* n_triangles x 9: v0, v1, v2 */
	const float *triangle_uv;   /* n_triangles x 6 per-vertex (u,v), or NULL */
	const int32_t *triangle_mat;
	int32_t n_materials;
	const are_material *materials;
	int32_t n_textures;
	const are_texture *textures;
	int64_t n_texels;
	const float *texels;        /* n_texels x 3 RGB, linear [0,1] */
	int32_t background;         /* ARE_BG_* */
	float bg_a[3];              /* constant colour, or gradient bottom (d.y=-1) */
	float bg_b[3];              /* gradient top (d.y=+1) */
	int32_t triangle_test;      /* ARE_TRI_* */
	int32_t bvh_leaf_size;      /* max primitives per BVH leaf; 0 = default (4) */
	int32_t bvh_build;          /* ARE_BVH_*: where the tree is built (same answers either way) */
	int32_t bvh_width;          /* children per BVH node traversed: 0 = automatic (4 above 2^19 primitives,
	                               else 2), 2, or 4 (host build only); same answers either way */
	int32_t accel;              /* ARE_ACCEL_*: how closest hits are found (same answers either way) */
} are_scene_desc;

enum {
	ARE_ACCEL_AUTO = 0,  /* scenes of at most 48 primitives: a warp-cooperative linear scan of the
	                        primitives staged in shared memory; larger scenes: the BVH */
	ARE_ACCEL_BVH = 1    /* always traverse the BVH, whatever the scene's size */
};

enum {
	ARE_BVH_HOST_SAH = 0,  /* binned SAH on the host (best trees; seconds for millions of primitives) */
	ARE_BVH_DEVICE = 1     /* linear BVH over Morton codes on the GPU (milliseconds); scenes of at most
	                          48 primitives, which are scanned linearly, always use the host build */
};

typedef struct are_scene are_scene; /* opaque: device-resident SoA + BVH */

/* ---- camera and render parameters -------------------------------------- */

/* The reference camera is (camPos, camTarget, camUp, fov) with fov the
 * vertical field of view in degrees (rt.cpp:337-343).  aperture/focus_dist add
 * a thin lens; aperture 0 is the reference's pinhole exactly. */
typedef struct are_camera {
	float lookfrom[3];
	float lookat[3];
	float vup[3];
	float vfov_deg;
	float aperture;
	float focus_dist;
} are_camera;

enum { ARE_EST_PATH = 0, ARE_EST_LEGACY_RT = 1, ARE_EST_GUIDED = 2 };
enum {
	ARE_FLAG_DEVICE_OUTPUT = 1,   /* rgb_out / var_out are device pointers */
	ARE_FLAG_NO_JITTER = 2,       /* sample pixel centres (rt.cpp:364-365) */
	ARE_FLAG_CLAMP_OUTPUT = 4,    /* clamp each pixel to [0,1] (rt.cpp:368) */
	ARE_FLAG_LEGACY_MT19937 = 8   /* ARE_EST_LEGACY_RT with rt.cpp's per-row std::mt19937 stream
	                                 seeded (uint32)seed + y (rt.cpp:348-351): one thread per row */
};

typedef struct are_render_params {
	int32_t width, height;
	int32_t spp;                /* samples (camera paths) per pixel */
	int32_t max_depth;          /* segments per path, >= 1 */
	uint64_t seed;
	int32_t rr_depth;           /* Russian roulette from this depth on; <0 = off */
	float t_min;                /* hits must have t > t_min */
	int32_t estimator;          /* ARE_EST_* */
	int32_t flags;              /* ARE_FLAG_* */
	int32_t pool_size;          /* paths in flight; 0 = auto */
	int32_t chunk;              /* samples per work item; 0 = auto */
	int32_t block_size;         /* threads per block; 0 = auto */
	int32_t schedule;           /* ARE_SCHEDULE_*; the image does not depend on it */
} are_render_params;

/* How are_render (ARE_EST_PATH) runs its paths.  Both produce the same image
 * bit for bit for the same chunk (every work item's samples run in one slot,
 * in order).
 *   WAVEFRONT:  a pool of paths in device memory, one closest-hit and one
 *               shading kernel per bounce over compacted queues, in CUDA graphs;
 *   MEGAKERNEL: one persistent launch, one path per resident thread, each
 *               thread tracing its paths to the end and taking the next work
 *               item itself; the path state stays in registers;
 *   AUTO:       MEGAKERNEL (the faster of the two on every scene measured).
 * The automatic chunk differs between the two, so set chunk to compare. */
enum { ARE_SCHEDULE_AUTO = 0, ARE_SCHEDULE_WAVEFRONT = 1, ARE_SCHEDULE_MEGAKERNEL = 2 };

enum { ARE_KERNEL_INTERSECT = 0, ARE_KERNEL_SHADE = 1, ARE_KERNEL_GENERATE = 2, ARE_KERNEL_OTHER = 3 };

typedef struct are_render_stats {
	int64_t samples;            /* camera paths completed */
	int64_t segments;           /* extension rays traced (closest-hit queries) */
	int64_t iterations;         /* wavefront iterations executed */
	double device_ms;           /* CUDA-event time of the whole render on its stream */
	double kernel_ms[4];        /* CUDA-event time per kernel kind (ARE_KERNEL_*) */
	int64_t kernel_launches[4]; /* launches per kernel kind */
	int32_t error_word;         /* device error bits, 0 = clean: 1 traversal stack overflow, 2 path queue
	                               overflow, 4 bad index, 8 non-finite radiance (dropped), 16 tensor-core
	                               wait timed out, 32 BVH walk visited more nodes than the tree has */
	int32_t reserved_;
	double aux[4];              /* are_render: [0] segments traced by the end-of-render tail kernel;
	                               are_render_guided: training samples, Adam steps, guided vertices, last loss */
} are_render_stats;

/* ---- entry points ------------------------------------------------------- */

ARE_API const char *are_status_string(are_status s);
/* Message of the calling thread's most recent failure ("" if none). */
ARE_API const char *are_last_error(void);
/* Library version as MAJOR*10000 + MINOR*100 + PATCH. */
ARE_API int32_t are_version(void);
/* Number of CUDA devices visible (0 when no GPU; never fails). */
ARE_API int32_t are_device_count(void);
/* Scenes and render workspaces take device memory from a per-device pool
 * that keeps up to an eighth of the device's memory (at least 1 GiB) cached
 * after frees, so per-frame scene rebuilds do not allocate anew.  This returns the cached memory of `device` (-1: every
 * device the library has used) to the driver; memory in use stays. */
ARE_API are_status are_trim_memory(int32_t device);

/* Replaces building rt.cpp's Scene (rt.cpp:146-186) / filling an
 * are::ObjectSet: validates the descriptor, builds the SAH BVH on the host,
 * and uploads SoA primitive records, BVH nodes, materials and textures to
 * the current CUDA device.  The descriptor's arrays are copied. */
ARE_API are_status are_scene_create(const are_scene_desc *desc, are_scene **out);
ARE_API are_status are_scene_destroy(are_scene *scene);
/* Host-side BVH statistics of a created scene (no device work). */
ARE_API are_status are_scene_info(const are_scene *scene, int64_t *n_prims, int64_t *n_nodes,
	int32_t *max_leaf, int32_t *depth);

/* Replaces rt.cpp:337-374 render(): renders width x height pixels, spp
 * samples each, writing the mean linear radiance to rgb_out (row-major from
 * the top row, 3 floats per pixel).  var_out, if not NULL, receives the
 * per-pixel sample variance of the mean (3 floats per pixel).  Both are host
 * pointers unless params->flags has ARE_FLAG_DEVICE_OUTPUT.  stats may be NULL. */
ARE_API are_status are_render(are_scene *scene, const are_camera *camera, const are_render_params *params,
	float *rgb_out, float *var_out, are_render_stats *stats);

/* Replaces rt.cpp:209-218 intersect() for a batch: closest hit of each ray.
 * rays: n x 8 floats (origin xyz, t_min, direction xyz, t_max).
 * hits: n x 4 (t, prim id as int32 bits, u, v); prim id -1 and t = +inf on a miss.
 * For triangles (u,v) are the barycentrics of v1 and v2 (rt.cpp:123-138);
 * for quads the planar coordinates along edges u and v; for spheres 0.
 * device_ptrs != 0 means rays/hits are device pointers.  ms_out may be NULL;
 * it receives the kernel's CUDA-event time. */
ARE_API are_status are_intersect(are_scene *scene, const float *rays, int64_t n, float *hits,
	int32_t device_ptrs, float *ms_out);

/* ---- rendering without allocating -------------------------------------- */

/* No counterpart in the reference: an extra entry point for callers that may
 * not allocate device memory while they render — for example a plugin host
 * that hands each plugin a fixed device-memory budget and forbids allocations
 * of its own, or an application whose memory is owned by its own allocator and
 * that must not see the device-wide synchronisation a cudaMalloc/cudaFree can
 * cause in the middle of a frame.  Such a caller creates the scene first
 * (are_scene_create allocates) and then calls are_render_noalloc, which
 * renders the path estimator (ARE_EST_PATH, either schedule) like are_render
 * but calls no cudaMalloc, cudaFree or other allocating routine and creates
 * no streams, events or graphs.  The render runs on the scene's own stream and
 * the call returns when it is done.
 *
 * Its scratch — at most ARE_NOALLOC_MAX_PATHS paths in flight and at most
 * ARE_NOALLOC_MAX_PIXELS work items (a work item is one pixel's chunk of
 * samples) — is one static device array of ARE_NOALLOC_SCRATCH_BYTES in the
 * library, which every GPU that loads the library holds until the process
 * exits.  Larger images, or a params->chunk that gives more work items, are
 * rejected with ARE_ERR_INVALID_ARGUMENT.  params->chunk = 0 picks the
 * smallest chunk whose work items fit; the result equals are_render's with
 * the same chunk.
 *
 * rgb_out (required) and var_out (optional) are DEVICE pointers of
 * width*height*3 floats, and params->flags must include
 * ARE_FLAG_DEVICE_OUTPUT (host pointers are rejected).  The first call on a
 * device looks up the array's device address (with that device current) and
 * keeps it for the life of the process; make that first call before any stream
 * capture, and do not call this entry point after a cudaDeviceReset of that
 * device.  All calls share the array and it keeps the last call's contents
 * (each call clears what must start at zero); calls that overlap on the GPU
 * race on it, so serialise them.  Statistics report counts; device_ms and
 * kernel_ms stay 0 because no events are created. */
#define ARE_NOALLOC_MAX_PATHS 65536
#define ARE_NOALLOC_MAX_PIXELS 524288
#define ARE_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
ARE_API are_status are_render_noalloc(are_scene *scene, const are_camera *camera, const are_render_params *params,
	float *rgb_out, float *var_out, are_render_stats *stats);

/* ---- path guiding ------------------------------------------------------- */

/* No counterpart in the reference (it has no guiding).  A small network
 * (12-frequency encoding of position, normal and outgoing direction; four
 * 64-wide ReLU layers; 8 von Mises-Fisher lobes) that learns where incident
 * radiance comes from, trained online from the renderer's own samples with
 * Adam.  FP16 tensor-core arithmetic, FP32 accumulation and master weights.
 * Parameter layout and loss: oracle/orc_guide.c. */
typedef struct are_guide are_guide;
ARE_API int32_t are_guide_param_count(void);
ARE_API are_status are_guide_create(uint64_t seed, are_guide **out);
ARE_API are_status are_guide_destroy(are_guide *guide);
ARE_API are_status are_guide_get_params(are_guide *guide, float *params_out);
ARE_API are_status are_guide_set_params(are_guide *guide, const float *params);  /* also resets Adam */
/* raw network outputs (n x 48, host) for features (n x 9, host) */
ARE_API are_status are_guide_forward(are_guide *guide, const float *features, int64_t n, float *out);
/* samples: n x 13 host floats (features 9, direction 3, weight 1).  Mean loss
 * and its gradient (are_guide_param_count() floats), parameters unchanged. */
ARE_API are_status are_guide_gradient(are_guide *guide, const float *samples, int64_t n, float *loss, float *grad);
/* The mixture the renderer samples, n x 48 floats per row: lobe l's
 * (mu.x, mu.y, mu.z, kappa) at 4 l and (weight pi_l, normaliser
 * kappa / (2 pi (1 - e^-2 kappa))) at 32 + 2 l; the density of a unit
 * direction w is sum_l pi_l norm_l exp(kappa_l (mu_l . w - 1)). */
ARE_API are_status are_guide_mixture(are_guide *guide, const float *features, int64_t n, float *out);
/* losses of the most recent Adam steps taken inside renders (oldest first);
 * returns how many were written (at most max) */
ARE_API int32_t are_guide_loss_history(are_guide *guide, float *out, int32_t max);
/* one Adam step (beta1 0.9, beta2 0.99) on a batch; loss before the step */
ARE_API are_status are_guide_train(are_guide *guide, const float *samples, int64_t n, float lr, float *loss);

/* Test hook for the bounded device-side waits of the tensor-core inference
 * and training kernels: each warpgroup's first wait for its tensor-core MMAs
 * gives up after `polls` polls (-1 restores the default bound of 2^22).  A
 * wait that gives up sets the device error bit 16, lets the work already in
 * flight land, frees the block's tensor memory and returns, and the call
 * reports ARE_ERR_KERNEL_TIMEOUT (inside a render, ARE_ERR_INTERNAL); a
 * training step that gave up is not applied (the weights stay as they
 * were).  With polls = 0 every inference and training call of this guide
 * takes that path.  No counterpart in the reference. */
ARE_API are_status are_guide_set_wait_limit(are_guide *guide, int32_t polls);

typedef struct are_guide_params {
	float mix;            /* probability of drawing a guided vertex's direction from the network (one-sample MIS) */
	int32_t guide_depth;  /* diffuse bounces guided per path: 0 .. 4 on the wavefront schedule, any number on the
	                         megakernel (training samples come from the first four either way) */
	int32_t train;        /* Adam steps on each collected batch during the render (0 = network frozen, at most 16) */
	int32_t batch;        /* training samples per Adam step (e.g. 2^18); a step is taken between
	                         graph launches once a quarter batch has been collected */
	float lr;             /* Adam learning rate */
	float weight_clip;    /* cap on a sample's weight relative to the batch mean (0 = none) */
	int32_t cache_res;    /* megakernel schedule: cells per axis of the mixture cache (0 = 32, at most 128) */
	int32_t max_steps;    /* megakernel schedule: Adam steps per render at most (0 = no limit); once they are
	                         taken the render goes on with the network frozen, without training records */
} are_guide_params;

/* The path estimator (ARE_EST_PATH) with guided diffuse bounces: at each of
 * the first guide_depth diffuse vertices the direction is drawn from the
 * network's mixture with probability mix, else by cosine sampling, and
 * weighted by the combined density, so the image stays unbiased whatever the
 * network has learned.  With train != 0 the network trains on the render's
 * own paths; stats->aux holds the training samples emitted, the Adam steps
 * taken, the guided vertices and the last loss.  params->schedule picks how:
 *   MEGAKERNEL (and AUTO): the persistent path loop of are_render; the
 *     network is evaluated on a mixture cache (cache_res^3 cells of the
 *     scene's box x six normal directions, at the cell's centre) after every
 *     training step, and a guided vertex samples its cell's cached mixture.
 *     The frame runs as passes of growing size with the Adam steps and the
 *     cache refresh between them.  stats->kernel_ms: [ARE_KERNEL_SHADE] the
 *     path megakernel, [ARE_KERNEL_GENERATE] cache inference,
 *     [ARE_KERNEL_OTHER] training; stats->iterations the passes.
 *   WAVEFRONT: the network runs on every guided vertex itself (one batch per
 *     bounce); stats->kernel_ms holds [ARE_KERNEL_INTERSECT] closest hits and
 *     input selection, [ARE_KERNEL_GENERATE] network inference,
 *     [ARE_KERNEL_SHADE] guided shading, [ARE_KERNEL_OTHER] the training steps. */
ARE_API are_status are_render_guided(are_scene *scene, are_guide *guide, const are_camera *camera,
	const are_render_params *params, const are_guide_params *guide_params, float *rgb_out, float *var_out,
	are_render_stats *stats);

/* ---- many scenes in one launch ------------------------------------------ */

/* Launch shape of are_render_batch; 0 fields take defaults (256 threads, 4). */
typedef struct are_batch_options {
	int32_t block_size;   /* threads per block of the persistent kernel */
	int32_t fetch;        /* work items per lane taken with each atomic on the shared queue */
	int32_t leaf_size;    /* BVH leaf size the scenes were built with (reported by the autotuner) */
	int32_t bvh_width;    /* BVH node layout the scenes were built with, 2 or 4 (reported by the autotuner) */
} are_batch_options;

/* No counterpart in the reference (it renders one scene).  Renders n scenes of
 * any size, resolution and spp in one persistent kernel launch over a shared
 * work queue (pixel x sample-chunk items of all scenes), captured with its
 * clears and resolves in one CUDA graph.  Same path estimator and random
 * numbers as are_render with ARE_EST_PATH; per-pixel sums use FP32 atomics.
 * rgb_out[i] (host, may be NULL to skip) receives scene i's mean radiance;
 * scene_ms[i] (may be NULL) its completion time from the start of the launch.
 * All scenes must live on one device. */
ARE_API are_status are_render_batch(are_scene *const *scenes, const are_camera *cameras,
	const are_render_params *params, int32_t n, const are_batch_options *options, float *const *rgb_out,
	double *scene_ms, are_render_stats *stats);

/* Times the batch on a calibration run (spp capped at calib_spp), building
 * the scenes from their descriptors: first every BVH leaf size {2,4,8} x
 * block size {128,256,512} x fetch {1,4,16} on the binary tree, then the node
 * layout (binary or 4-wide tree, bvh_width 2 or 4) x leaf size at the best
 * block size and fetch; returns the fastest combination. */
ARE_API are_status are_batch_autotune(const are_scene_desc *const *descs, const are_camera *cameras,
	const are_render_params *params, int32_t n, int32_t calib_spp, are_batch_options *best, double *best_ms);

/* ---- output formats ----------------------------------------------------- */

typedef enum are_tonemap_mode {
	/* Replaces writePPM's quantisation (experiments/rt.cpp:380-386): clamp to
	 * [0,1] (NaN -> 1), powf(c, 1 / gamma) * 255 in FP32, truncated; gamma 2.2
	 * there. */
	ARE_TONEMAP_GAMMA = 0,
	/* Replaces are::Texture::save_texture's quantisation (src/texture.cpp:378-383):
	 * clamp(c * 255.0, 0, 255) in FP64, truncated (NaN -> 0, undefined there). */
	ARE_TONEMAP_LINEAR = 1
} are_tonemap_mode;

typedef struct are_tonemap_params {
	int32_t mode;       /* are_tonemap_mode */
	float gamma;        /* ARE_TONEMAP_GAMMA: 0.1 .. 10 */
	uint32_t flags;     /* ARE_FLAG_DEVICE_OUTPUT: rgb and out are device pointers of the current device */
	int32_t reserved_;
} are_tonemap_params;

/* n_values FP32 linear values (pixels x 3) -> bytes on the GPU, byte-identical
 * to the reference formula of the mode for every input.  Host pointers are
 * staged through a device buffer; device pointers are used in place.  Runs on
 * the calling thread's default stream and returns when the bytes are written. */
ARE_API are_status are_tonemap(const float *rgb, int64_t n_values, const are_tonemap_params *params, uint8_t *out);
/* Replaces writePPM's file output (rt.cpp:377-392) and save_texture's
 * (texture.cpp:362-395): "P6\n<w> <h>\n255\n" then the RGB bytes, top row first. */
ARE_API are_status are_write_ppm(const char *path, const uint8_t *rgb8, int32_t width, int32_t height);
/* FP32 RGB Portable Float Map (no reference counterpart: the linear image
 * before quantisation), little-endian, bottom row first as the format wants. */
ARE_API are_status are_write_pfm(const char *path, const float *rgb, int32_t width, int32_t height);
/* Replaces are::Texture's PPM constructor (src/texture.cpp:9-50): a P6 file
 * with maximum 255 -> width, height and, if texels is not null, width x height
 * RGB floats byte / 255.0 in file order, ready for are_scene_desc.texels. */
ARE_API are_status are_read_ppm(const char *path, int32_t *width, int32_t *height, float *texels);

/* ---- synthetic workloads ------------------------------------------------ */

enum {
	ARE_CONFIG_RANDOM_SPHERES = 0,  /* 488 spheres, 400x225, 32 spp, depth 50 */
	ARE_CONFIG_CORNELL = 1,         /* 19 quads, 600x600, 1024 spp, depth 50 */
	ARE_CONFIG_MESH = 2,            /* displaced icosphere, 1920x1080, 256 spp, depth 16 */
	ARE_CONFIG_CORNELL_OCCLUDED = 4,/* Cornell + occluder under the light, depth 16 */
	ARE_CONFIG_LEGACY_RT = 5,       /* rt.cpp's own 34-triangle scene (rt.cpp:153-167) */
	ARE_CONFIG_SPHERE_FIELD = 6     /* one scene of the uneven batch: mesh_frequency = sphere count
	                                   (>= 1) on a jittered grid, materials as RANDOM_SPHERES; the
	                                   resolution (256x256, 640x360, 1280x720) and spp (16, 64, 256)
	                                   are drawn from the seed */
};

typedef struct are_config are_config; /* owns the arrays its descriptor points at */

/* Builds one of the seeded synthetic scenes.  mesh_frequency only affects
 * ARE_CONFIG_MESH (geodesic frequency n gives 20 n^2 triangles; 0 = 316). */
ARE_API are_status are_config_build(int32_t config, uint64_t seed, int32_t mesh_frequency, are_config **out);
ARE_API const are_scene_desc *are_config_desc(const are_config *cfg);
ARE_API are_status are_config_defaults(const are_config *cfg, are_camera *camera, are_render_params *params);
ARE_API void are_config_free(are_config *cfg);

#ifdef __cplusplus
}
#endif

#endif /* AURORA_GB300_H */
