// scene.cpp — are_scene_create: validate a flat scene descriptor, build the
// BVH on the host and upload the SoA primitive records to the device.
//
// Replaces the construction of rt.cpp's Scene (experiments/rt.cpp:146-186)
// and of an are::ObjectSet of are::Triangle objects.  Validation mirrors the
// reference's error behaviour where it has one: are::Triangle's constructor
// rejects null materials/textures, zero edge vectors and collinear edges
// (src/object/triangle.cpp:9-46); here those become ARE_ERR_INVALID_ARGUMENT.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "bvh.h"
#include "lbvh.h"
#include "scene.h"

namespace are_core {

// ---- memory ----------------------------------------------------------------

namespace {

// cached in the pool between frees: an eighth of the device's memory (at least 1 GiB), so the
// one-sample item sums of a large frame (several GB) are reused by the next scene, not mapped anew
uint64_t pool_keep_bytes(int device) {
	size_t total = 0;
	cudaDeviceProp prop{};
	if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) total = prop.totalGlobalMem;
	cudaGetLastError();
	return std::max<uint64_t>(1ull << 30, (uint64_t)total / 8);
}

std::mutex g_pool_mu;
cudaMemPool_t g_pools[256];
bool g_pool_failed[256];

std::mutex g_pinned_mu;
std::vector<unsigned *> g_pinned_free;

// small scenes are uploaded through one pinned staging buffer: one copy instead of one per array.  The
// copy is not waited for: g_stage_done marks it, and the next scene waits for that event before it
// overwrites the buffer, so a create-render-destroy frame synchronises once, in the render.
constexpr size_t STAGE_BYTES = 8u << 20;
std::mutex g_stage_mu;
unsigned char *g_stage = nullptr;
cudaEvent_t g_stage_done = nullptr;
bool g_stage_failed = false;

// Streams and timing events of destroyed scenes, per device, idle and ready for the next scene: a
// caller that creates and destroys a scene every frame does not create a stream and events each time.
struct SceneRuntime {
	cudaStream_t stream;
	std::vector<cudaEvent_t> events;
};
constexpr size_t RUNTIME_CACHE = 32;
std::mutex g_runtime_mu;
std::vector<SceneRuntime> g_runtime_free[256];

}  // namespace

// a stream (and the timing events that came with it) for a new scene on the current device
static are_status acquire_runtime(are_scene *sc) {
	if (sc->device >= 0 && sc->device < 256) {
		std::lock_guard<std::mutex> lk(g_runtime_mu);
		std::vector<SceneRuntime> &f = g_runtime_free[sc->device];
		if (!f.empty()) {
			sc->stream = f.back().stream;
			sc->render_events = std::move(f.back().events);
			f.pop_back();
			return ARE_OK;
		}
	}
	return cuda_status(cudaStreamCreateWithFlags(&sc->stream, cudaStreamNonBlocking), "cudaStreamCreate");
}

// the idle stream and events of a scene being destroyed: kept for the next scene, or released
static void release_runtime(are_scene *sc) {
	if (!sc->stream) return;
	if (sc->device >= 0 && sc->device < 256) {
		std::lock_guard<std::mutex> lk(g_runtime_mu);
		std::vector<SceneRuntime> &f = g_runtime_free[sc->device];
		if (f.size() < RUNTIME_CACHE) {
			f.push_back(SceneRuntime{ sc->stream, std::move(sc->render_events) });
			sc->stream = nullptr;
			sc->render_events.clear();
			return;
		}
	}
	for (cudaEvent_t e : sc->render_events) cudaEventDestroy(e);
	sc->render_events.clear();
	cudaStreamDestroy(sc->stream);
	sc->stream = nullptr;
}

// Falls back to cudaMalloc (recorded in sc->allocations) if the device has no
// pool support.
are_status pool_alloc(are_scene *sc, size_t bytes, void **p) {
	*p = nullptr;
	if (bytes == 0) return ARE_OK;
	cudaMemPool_t pool = nullptr;
	if (sc->device >= 0 && sc->device < 256) {
		std::lock_guard<std::mutex> lk(g_pool_mu);
		if (!g_pools[sc->device] && !g_pool_failed[sc->device]) {
			cudaMemPoolProps props{};
			props.allocType = cudaMemAllocationTypePinned;
			props.location.type = cudaMemLocationTypeDevice;
			props.location.id = sc->device;
			if (cudaMemPoolCreate(&g_pools[sc->device], &props) == cudaSuccess) {
				uint64_t keep = pool_keep_bytes(sc->device);
				cudaMemPoolSetAttribute(g_pools[sc->device], cudaMemPoolAttrReleaseThreshold, &keep);
			} else {
				cudaGetLastError();
				g_pools[sc->device] = nullptr;
				g_pool_failed[sc->device] = true;
			}
		}
		pool = g_pools[sc->device];
	}
	if (pool) {
		if (are_status st = cuda_status(cudaMallocFromPoolAsync(p, bytes, pool, sc->stream), "cudaMallocFromPoolAsync"))
			return st;
		sc->pool_allocations.push_back(*p);
		return ARE_OK;
	}
	if (are_status st = cuda_status(cudaMalloc(p, bytes), "cudaMalloc")) return st;
	sc->allocations.push_back(*p);
	return ARE_OK;
}

void pool_free(are_scene *sc, void *p) {
	if (!p) return;
	for (size_t i = 0; i < sc->pool_allocations.size(); ++i)
		if (sc->pool_allocations[i] == p) {
			cudaFreeAsync(p, sc->stream);
			sc->pool_allocations.erase(sc->pool_allocations.begin() + (long)i);
			return;
		}
	for (size_t i = 0; i < sc->allocations.size(); ++i)
		if (sc->allocations[i] == p) {
			cudaFree(p);
			sc->allocations.erase(sc->allocations.begin() + (long)i);
			return;
		}
}

are_status pool_trim(int device) {
	if (device < -1 || device >= 256) {
		set_error("device ordinal out of range");
		return ARE_ERR_INVALID_ARGUMENT;
	}
	std::lock_guard<std::mutex> lk(g_pool_mu);
	for (int d = device < 0 ? 0 : device; d < (device < 0 ? 256 : device + 1); ++d) {
		if (!g_pools[d]) continue;
		// frees are stream-ordered: let them land before trimming
		int cur = 0;
		cudaGetDevice(&cur);
		cudaSetDevice(d);
		cudaDeviceSynchronize();
		cudaSetDevice(cur);
		if (are_status st = cuda_status(cudaMemPoolTrimTo(g_pools[d], 0), "cudaMemPoolTrimTo")) return st;
	}
	return ARE_OK;
}

unsigned *pinned_block_acquire() {
	std::lock_guard<std::mutex> lk(g_pinned_mu);
	if (g_pinned_free.empty()) {
		// a new chunk of 64 blocks; chunks live as long as the process
		constexpr size_t BLOCK_BYTES = 256, BLOCKS = 64;
		unsigned char *chunk = nullptr;
		if (cudaMallocHost((void **)&chunk, BLOCK_BYTES * BLOCKS) != cudaSuccess) {
			cudaGetLastError();
			return nullptr;
		}
		for (size_t k = 0; k < BLOCKS; ++k) g_pinned_free.push_back((unsigned *)(chunk + BLOCK_BYTES * k));
	}
	unsigned *p = g_pinned_free.back();
	g_pinned_free.pop_back();
	return p;
}

void pinned_block_release(unsigned *p) {
	if (!p) return;
	std::lock_guard<std::mutex> lk(g_pinned_mu);
	g_pinned_free.push_back(p);
}


static thread_local std::string g_err;
void set_error(const std::string &msg) { g_err = msg; }
const char *last_error() { return g_err.c_str(); }

are_status cuda_status(cudaError_t e, const char *what) {
	if (e == cudaSuccess) return ARE_OK;
	set_error(std::string(what) + ": " + cudaGetErrorString(e));
	if (e == cudaErrorMemoryAllocation) return ARE_ERR_OUT_OF_MEMORY;
	if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return ARE_ERR_NO_DEVICE;
	return ARE_ERR_CUDA;
}

namespace {

are_status invalid(const std::string &msg) {
	set_error(msg);
	return ARE_ERR_INVALID_ARGUMENT;
}

bool finite3(const float *p) { return std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]); }

// are::Vec3::near_zero (src/basic/vec3.cpp:143-146): every |component| < 1e-8
bool near_zero(const double *v) { return std::fabs(v[0]) < 1e-8 && std::fabs(v[1]) < 1e-8 && std::fabs(v[2]) < 1e-8; }

void cross_d(const double *a, const double *b, double *c) {
	c[0] = a[1] * b[2] - a[2] * b[1];
	c[1] = a[2] * b[0] - a[0] * b[2];
	c[2] = a[0] * b[1] - a[1] * b[0];
}

are_status validate(const are_scene_desc *d) {
	if (!d) return invalid("scene descriptor is null");
	if (d->n_spheres < 0 || d->n_quads < 0 || d->n_triangles < 0 || d->n_materials < 0 || d->n_textures < 0 ||
		d->n_texels < 0)
		return invalid("negative count in scene descriptor");
	if ((d->n_spheres && (!d->spheres || !d->sphere_mat)) || (d->n_quads && (!d->quads || !d->quad_mat)) ||
		(d->n_triangles && (!d->triangles || !d->triangle_mat)) || (d->n_materials && !d->materials) ||
		(d->n_textures && !d->textures) || (d->n_texels && !d->texels))
		return invalid("null array with a non-zero count in scene descriptor");
	int64_t total = (int64_t)d->n_spheres + d->n_quads + d->n_triangles;
	if (total > (int64_t)INT32_MAX / 4) return invalid("too many primitives");
	if (d->background != ARE_BG_CONSTANT && d->background != ARE_BG_SKY_GRADIENT) return invalid("unknown background");
	if (d->bvh_build != ARE_BVH_HOST_SAH && d->bvh_build != ARE_BVH_DEVICE) return invalid("unknown bvh_build");
	if (d->bvh_width != 0 && d->bvh_width != 2 && d->bvh_width != 4) return invalid("bvh_width must be 0, 2 or 4");
	if (d->accel != ARE_ACCEL_AUTO && d->accel != ARE_ACCEL_BVH) return invalid("unknown accel");
	if (d->bvh_width == 4 && d->bvh_build == ARE_BVH_DEVICE)
		return invalid("bvh_width 4 needs the host build (the device build's tree is traversed two-wide)");
	if (d->triangle_test != ARE_TRI_REFERENCE_MT && d->triangle_test != ARE_TRI_WATERTIGHT)
		return invalid("unknown triangle test");
	for (int32_t i = 0; i < d->n_textures; ++i) {
		const are_texture &t = d->textures[i];
		if (t.type < ARE_TEX_SOLID || t.type > ARE_TEX_IMAGE) return invalid("texture " + std::to_string(i) + ": unknown type");
		if (t.mapping != ARE_MAP_SURFACE_UV && t.mapping != ARE_MAP_SPHERICAL)
			return invalid("texture " + std::to_string(i) + ": unknown mapping");
		if (t.type == ARE_TEX_IMAGE) {
			// are::Texture rejects non-positive sizes (src/texture.cpp:52-55)
			if (t.width <= 0 || t.height <= 0) return invalid("texture " + std::to_string(i) + ": width and height must be positive");
			if (t.texel_offset < 0 || (int64_t)t.texel_offset + (int64_t)t.width * t.height > d->n_texels)
				return invalid("texture " + std::to_string(i) + ": texel range outside texels[]");
			if (t.filter != ARE_FILTER_NEAREST && t.filter != ARE_FILTER_BILINEAR)
				return invalid("texture " + std::to_string(i) + ": unknown filter");
		}
	}
	for (int32_t i = 0; i < d->n_materials; ++i) {
		const are_material &m = d->materials[i];
		if (m.type < ARE_MAT_LAMBERTIAN || m.type > ARE_MAT_DIFFUSE_LIGHT)
			return invalid("material " + std::to_string(i) + ": unknown type");
		if (m.texture < -1 || m.texture >= d->n_textures)
			return invalid("material " + std::to_string(i) + ": texture index out of range");
		if (m.type == ARE_MAT_DIELECTRIC && !(m.ior > 0.0f)) return invalid("material " + std::to_string(i) + ": ior must be > 0");
		if (m.type == ARE_MAT_METAL && !(m.fuzz >= 0.0f)) return invalid("material " + std::to_string(i) + ": fuzz must be >= 0");
	}
	auto check_mat = [&](int32_t m, const char *what, int32_t i) -> are_status {
		if (m < 0 || m >= d->n_materials)
			return invalid(std::string(what) + " " + std::to_string(i) + ": material index out of range");
		return ARE_OK;
	};
	for (int32_t i = 0; i < d->n_spheres; ++i) {
		const float *s = d->spheres + 4 * (size_t)i;
		if (!finite3(s) || !(s[3] > 0.0f) || !std::isfinite(s[3]))
			return invalid("sphere " + std::to_string(i) + ": centre must be finite and radius > 0");
		if (are_status st = check_mat(d->sphere_mat[i], "sphere", i)) return st;
	}
	for (int32_t i = 0; i < d->n_quads; ++i) {
		const float *q = d->quads + 9 * (size_t)i;
		if (!finite3(q) || !finite3(q + 3) || !finite3(q + 6)) return invalid("quad " + std::to_string(i) + ": non-finite");
		double u[3] = { q[3], q[4], q[5] }, v[3] = { q[6], q[7], q[8] }, c[3];
		cross_d(u, v, c);
		if (near_zero(u) || near_zero(v) || near_zero(c)) return invalid("quad " + std::to_string(i) + ": degenerate edges");
		if (are_status st = check_mat(d->quad_mat[i], "quad", i)) return st;
	}
	auto check_tri = [&](int32_t i) -> are_status {
		const float *t = d->triangles + 9 * (size_t)i;
		if (!finite3(t) || !finite3(t + 3) || !finite3(t + 6))
			return invalid("triangle " + std::to_string(i) + ": non-finite vertex");
		double u[3], v[3], c[3];
		for (int k = 0; k < 3; ++k) u[k] = (double)t[3 + k] - t[k], v[k] = (double)t[6 + k] - t[k];
		cross_d(u, v, c);
		// src/object/triangle.cpp:21-36: zero or collinear edge vectors throw
		if (near_zero(u) || near_zero(v)) return invalid("triangle " + std::to_string(i) + ": edge vector is zero");
		if (near_zero(c)) return invalid("triangle " + std::to_string(i) + ": edge vectors are collinear");
		return check_mat(d->triangle_mat[i], "triangle", i);
	};
	// the lowest-numbered bad triangle, searched in parallel, is the one reported (on this thread)
	std::atomic<int32_t> first_bad{ d->n_triangles };
	parallel_ranges((size_t)d->n_triangles, [&](size_t i0, size_t i1) {
		for (size_t i = i0; i < i1 && (int32_t)i < first_bad.load(std::memory_order_relaxed); ++i)
			if (check_tri((int32_t)i) != ARE_OK) {
				int32_t cur = first_bad.load();
				while ((int32_t)i < cur && !first_bad.compare_exchange_weak(cur, (int32_t)i)) {}
				break;
			}
	});
	return first_bad < d->n_triangles ? check_tri(first_bad) : ARE_OK;
}

template <class T>
are_status upload(are_scene *sc, const T *src, size_t count, const T **dst) {
	if (count == 0) {
		*dst = nullptr;
		return ARE_OK;
	}
	void *p = nullptr;
	if (are_status st = cuda_status(cudaMalloc(&p, count * sizeof(T)), "cudaMalloc(scene)")) return st;
	sc->allocations.push_back(p);
	if (are_status st = cuda_status(cudaMemcpy(p, src, count * sizeof(T), cudaMemcpyHostToDevice), "cudaMemcpy(scene)"))
		return st;
	*dst = (const T *)p;
	return ARE_OK;
}

}  // namespace

namespace {

// record j of the descriptor in the DevScene layout (3 float4), input order
void pack_record(const are_scene_desc *d, int32_t g, float *o, int32_t &mat) {
	const int32_t ns = d->n_spheres, nq = d->n_quads;
	std::memset(o, 0, 48);
	if (g < ns) {
		std::memcpy(o, d->spheres + 4 * (size_t)g, 16);
		mat = d->sphere_mat[g];
	} else if (g < ns + nq) {
		const float *q = d->quads + 9 * (size_t)(g - ns);
		for (int r = 0; r < 3; ++r) std::memcpy(o + 4 * r, q + 3 * r, 12);
		o[3] = PRIM_TAG_QUAD;
		mat = d->quad_mat[g - ns];
	} else {
		const float *t = d->triangles + 9 * (size_t)(g - ns - nq);
		for (int r = 0; r < 3; ++r) std::memcpy(o + 4 * r, t + 3 * r, 12);
		o[3] = PRIM_TAG_TRI;
		mat = d->triangle_mat[g - ns - nq];
	}
}

// The scene with its BVH built on the device: records are packed on the host
// in input order (one pass), uploaded, and sorted into leaf order there.
are_status scene_create_device(const are_scene_desc *d, are_scene **out) {
	const int32_t ns = d->n_spheres, nq = d->n_quads, nt = d->n_triangles;
	const int32_t n = ns + nq + nt;
	std::vector<float> rec(12 * (size_t)n);
	std::vector<int32_t> mat((size_t)n);
	for (int32_t g = 0; g < n; ++g) pack_record(d, g, &rec[12 * (size_t)g], mat[g]);
	std::vector<float> uv;
	if (d->triangle_uv && nt) {
		uv.assign(6 * (size_t)n, 0.0f);
		std::memcpy(&uv[6 * (size_t)(ns + nq)], d->triangle_uv, 24 * (size_t)nt);
	}
	are_scene *sc = new are_scene();
	cudaGetDevice(&sc->device);
	cudaDeviceGetAttribute(&sc->n_sms, cudaDevAttrMultiProcessorCount, sc->device);
	are_status st = acquire_runtime(sc);
	void *tmp = nullptr;
	const size_t rec_b = ((48 * (size_t)n + 255) & ~(size_t)255), mat_b = ((4 * (size_t)n + 255) & ~(size_t)255);
	if (!st) st = cuda_status(cudaMalloc(&tmp, rec_b + mat_b + 24 * uv.size() / 6), "cudaMalloc(scene upload)");
	LbvhResult r;
	if (!st) {
		char *z = (char *)tmp;
		const float4 *d_rec = (const float4 *)z;
		const int32_t *d_mat = (const int32_t *)(z + rec_b);
		const float *d_uv = uv.empty() ? nullptr : (const float *)(z + rec_b + mat_b);
		cudaMemcpyAsync(z, rec.data(), 48 * (size_t)n, cudaMemcpyHostToDevice, sc->stream);
		cudaMemcpyAsync(z + rec_b, mat.data(), 4 * (size_t)n, cudaMemcpyHostToDevice, sc->stream);
		if (d_uv) cudaMemcpyAsync(z + rec_b + mat_b, uv.data(), 4 * uv.size(), cudaMemcpyHostToDevice, sc->stream);
		st = build_bvh_device(sc, d_rec, d_mat, d_uv, n, d->bvh_leaf_size, r, sc->stream);
	}
	if (tmp) {
		cudaStreamSynchronize(sc->stream);
		cudaFree(tmp);
	}
	DevScene &S = sc->dev;
	if (!st) st = upload(sc, (const DevMaterial *)d->materials, (size_t)d->n_materials, &S.mats);
	if (!st) st = upload(sc, (const DevTexture *)d->textures, (size_t)d->n_textures, &S.texs);
	if (!st) st = upload(sc, d->texels, 3 * (size_t)d->n_texels, &S.texels);
	if (!st && !(sc->host_counters = pinned_block_acquire())) {
		set_error("pinned host memory for the render counters");
		st = ARE_ERR_OUT_OF_MEMORY;
	}
	if (st) {
		delete sc;
		return st;
	}
	S.prims = r.prims;
	S.prim_gid = r.gid;
	S.prim_mat = r.mat;
	S.tri_uv = r.uv;
	S.nodes = r.nodes;
	S.nodes4 = nullptr;  // the device-built tree is traversed two-wide
	S.n_nodes4 = 0;
	S.leaves = nullptr;
	S.n_leaves = 0;
	S.n_prims = n;
	S.n_nodes = (int32_t)r.n_nodes;
	S.n_materials = d->n_materials;
	S.n_textures = d->n_textures;
	S.background = d->background;
	S.triangle_test = d->triangle_test;
	S.interleave = (d->n_quads + d->n_triangles) > 0 ? 1 : 0;
	for (int k = 0; k < 3; ++k) S.bg_a[k] = d->bg_a[k], S.bg_b[k] = d->bg_b[k];
	S.box_pad = r.box_pad;
	sc->n_prims = n;
	sc->n_spheres = ns, sc->n_quads = nq, sc->n_triangles = nt;
	for (int k = 0; k < 3; ++k) sc->box_lo[k] = r.lo[k], sc->box_hi[k] = r.hi[k];
	sc->n_nodes = r.n_nodes;
	sc->max_leaf = r.max_leaf;
	sc->depth = r.depth;
	*out = sc;
	return ARE_OK;
}

}  // namespace

are_status scene_create(const are_scene_desc *d, are_scene **out) {
	if (!out) return invalid("output handle pointer is null");
	*out = nullptr;
	if (are_status st = validate(d)) return st;
	int ndev = 0;
	if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
		cudaGetLastError();
		set_error("no CUDA device");
		return ARE_ERR_NO_DEVICE;
	}
	const int32_t ns = d->n_spheres, nq = d->n_quads, nt = d->n_triangles;
	const int32_t n = ns + nq + nt;
	if (d->bvh_build == ARE_BVH_DEVICE && n > LINEAR_MAX) return scene_create_device(d, out);

	// primitive bounds in double
	std::vector<PrimBox> boxes((size_t)n);
	parallel_ranges((size_t)n, [&](size_t i0, size_t i1) {
		for (size_t i = i0; i < i1; ++i) {
			PrimBox &b = boxes[i];
			if (i < (size_t)ns) {
				const float *s = d->spheres + 4 * i;
				for (int k = 0; k < 3; ++k) b.lo[k] = (double)s[k] - s[3], b.hi[k] = (double)s[k] + s[3];
			} else if (i < (size_t)(ns + nq)) {
				const float *q = d->quads + 9 * (i - ns);
				for (int k = 0; k < 3; ++k) {
					double c0 = q[k], c1 = (double)q[k] + q[3 + k], c2 = (double)q[k] + q[6 + k], c3 = c1 + q[6 + k];
					b.lo[k] = std::fmin(std::fmin(c0, c1), std::fmin(c2, c3));
					b.hi[k] = std::fmax(std::fmax(c0, c1), std::fmax(c2, c3));
				}
			} else {
				const float *t = d->triangles + 9 * (i - ns - nq);
				for (int k = 0; k < 3; ++k) {
					b.lo[k] = std::fmin(std::fmin((double)t[k], (double)t[3 + k]), (double)t[6 + k]);
					b.hi[k] = std::fmax(std::fmax((double)t[k], (double)t[3 + k]), (double)t[6 + k]);
				}
			}
		}
	});
	BvhResult bvh = build_bvh(boxes, d->bvh_leaf_size);

	// SoA records in leaf order
	std::vector<float> prims(12 * (size_t)std::max(n, 1), 0.0f);
	std::vector<int32_t> gid((size_t)std::max(n, 1), 0), mat((size_t)std::max(n, 1), 0);
	std::vector<float> tri_uv;
	if (d->triangle_uv && nt) tri_uv.assign(6 * (size_t)n, 0.0f);
	parallel_ranges((size_t)n, [&](size_t j0, size_t j1) {
		for (size_t j = j0; j < j1; ++j) {
			const int32_t g = bvh.order[j];
			float *o = &prims[12 * j];
			gid[j] = g;
			if (g < ns) {
				std::memcpy(o, d->spheres + 4 * (size_t)g, 16);
				mat[j] = d->sphere_mat[g];
			} else if (g < ns + nq) {
				const float *q = d->quads + 9 * (size_t)(g - ns);
				for (int r = 0; r < 3; ++r) std::memcpy(o + 4 * r, q + 3 * r, 12);
				o[3] = PRIM_TAG_QUAD;
				mat[j] = d->quad_mat[g - ns];
			} else {
				const float *t = d->triangles + 9 * (size_t)(g - ns - nq);
				for (int r = 0; r < 3; ++r) std::memcpy(o + 4 * r, t + 3 * r, 12);
				o[3] = PRIM_TAG_TRI;
				mat[j] = d->triangle_mat[g - ns - nq];
				if (!tri_uv.empty()) std::memcpy(&tri_uv[6 * j], d->triangle_uv + 6 * (size_t)(g - ns - nq), 24);
			}
		}
	});

	// the 4-wide tree: measured faster for the 2M-triangle mesh (trees deep in HBM: half the dependent
	// node fetches), slower for sphere fields of up to 152k spheres and for trees held in shared memory
	std::vector<float> wide;
	const bool four = d->bvh_width == 4 || (d->bvh_width == 0 && n > WIDE_BVH_MIN_PRIMS);
	if (n > LINEAR_MAX && four) wide = collapse_bvh4(bvh, SMEM_NODES4);
	std::vector<float> leaves;
	const bool linear = n <= LINEAR_MAX && d->accel != ARE_ACCEL_BVH;
	if (n > 0 && linear)
		for (int32_t i = 0; i < bvh.n_nodes; ++i) {
			int32_t cnt;
			std::memcpy(&cnt, &bvh.nodes[8 * (size_t)i + 7], 4);
			if (cnt > 0) leaves.insert(leaves.end(), &bvh.nodes[8 * (size_t)i], &bvh.nodes[8 * (size_t)i] + 8);
		}

	are_scene *sc = new are_scene();
	sc->linear = linear;
	cudaGetDevice(&sc->device);
	cudaDeviceGetAttribute(&sc->n_sms, cudaDevAttrMultiProcessorCount, sc->device);
	DevScene &S = sc->dev;
	are_status st = acquire_runtime(sc);
	if (!st && !(sc->host_counters = pinned_block_acquire())) {
		set_error("pinned host memory for the render counters");
		st = ARE_ERR_OUT_OF_MEMORY;
	}
	// every array of the scene in one block from the device's pool, at 256-byte offsets, copied on the
	// scene's stream (one allocation and one synchronisation per scene)
	struct Part {
		const void *src;
		size_t bytes;
		size_t off;
	};
	Part parts[] = { { prims.data(), prims.size() * 4, 0 }, { gid.data(), gid.size() * 4, 0 },
		{ mat.data(), mat.size() * 4, 0 }, { tri_uv.data(), tri_uv.size() * 4, 0 },
		{ bvh.nodes.data(), bvh.nodes.size() * 4, 0 }, { wide.data(), wide.size() * 4, 0 },
		{ leaves.data(), leaves.size() * 4, 0 }, { d->materials, sizeof(DevMaterial) * (size_t)d->n_materials, 0 },
		{ d->textures, sizeof(DevTexture) * (size_t)d->n_textures, 0 }, { d->texels, 12 * (size_t)d->n_texels, 0 } };
	static_assert(sizeof(DevMaterial) == sizeof(are_material) && sizeof(DevTexture) == sizeof(are_texture),
		"device records mirror the descriptor's");
	size_t total = 0;
	for (Part &q : parts) {
		q.off = total;
		total += (q.bytes + 255) & ~(size_t)255;
	}
	char *block = nullptr;
	if (!st) st = pool_alloc(sc, total, (void **)&block);
	bool staged = false;
	if (!st && total <= STAGE_BYTES) {
		std::lock_guard<std::mutex> lk(g_stage_mu);
		if (!g_stage && !g_stage_failed) {
			if (cudaMallocHost((void **)&g_stage, STAGE_BYTES) != cudaSuccess ||
				cudaEventCreateWithFlags(&g_stage_done, cudaEventDisableTiming) != cudaSuccess) {
				cudaGetLastError();
				if (g_stage) cudaFreeHost(g_stage);
				g_stage = nullptr;
				g_stage_failed = true;
			}
		}
		if (g_stage) {
			// the previous scene's copy out of the buffer must have finished
			st = cuda_status(cudaEventSynchronize(g_stage_done), "scene upload");
			for (const Part &q : parts)
				if (!st && q.bytes) std::memcpy(g_stage + q.off, q.src, q.bytes);
			if (!st) st = cuda_status(cudaMemcpyAsync(block, g_stage, total, cudaMemcpyHostToDevice, sc->stream), "scene upload");
			if (!st) st = cuda_status(cudaEventRecord(g_stage_done, sc->stream), "scene upload");
			staged = true;
		}
	}
	for (Part &q : parts) {
		if (st || staged) break;
		if (q.bytes) st = cuda_status(cudaMemcpyAsync(block + q.off, q.src, q.bytes, cudaMemcpyHostToDevice, sc->stream),
						  "scene upload");
	}
	if (!st && !staged) st = cuda_status(cudaStreamSynchronize(sc->stream), "scene upload");
	if (st) {
		delete sc;
		return st;
	}
	auto at = [&](int k) -> const void * { return parts[k].bytes ? block + parts[k].off : nullptr; };
	const float4 *pp = (const float4 *)at(0), *np = (const float4 *)at(4), *np4 = (const float4 *)at(5);
	const float4 *lp = (const float4 *)at(6);
	S.prim_gid = (const int32_t *)at(1);
	S.prim_mat = (const int32_t *)at(2);
	S.tri_uv = (const float *)at(3);
	S.mats = (const DevMaterial *)at(7);
	S.texs = (const DevTexture *)at(8);
	S.texels = (const float *)at(9);
	S.prims = pp;
	S.nodes = np;
	S.nodes4 = np4;
	S.n_nodes4 = (int32_t)(wide.size() / 32);
	S.leaves = lp;
	S.n_leaves = (int32_t)(leaves.size() / 8);
	S.n_prims = n;
	S.n_nodes = bvh.n_nodes;
	S.n_materials = d->n_materials;
	S.n_textures = d->n_textures;
	S.background = d->background;
	S.triangle_test = d->triangle_test;
	S.interleave = (d->n_quads + d->n_triangles) > 0 ? 1 : 0;
	for (int k = 0; k < 3; ++k) S.bg_a[k] = d->bg_a[k], S.bg_b[k] = d->bg_b[k];
	S.box_pad = bvh.box_pad;
	sc->n_prims = n;
	sc->n_spheres = ns, sc->n_quads = nq, sc->n_triangles = nt;
	for (int k = 0; k < 3; ++k) {
		double lo = n ? boxes[0].lo[k] : 0.0, hi = n ? boxes[0].hi[k] : 0.0;
		for (const PrimBox &b : boxes) lo = std::fmin(lo, b.lo[k]), hi = std::fmax(hi, b.hi[k]);
		sc->box_lo[k] = (float)lo, sc->box_hi[k] = (float)hi;
	}
	sc->n_nodes = bvh.n_nodes;
	sc->max_leaf = bvh.max_leaf;
	sc->depth = bvh.depth;
	*out = sc;
	return ARE_OK;
}

}  // namespace are_core

are_scene::~are_scene() {
	if (stream) cudaStreamSynchronize(stream);
	if (render_exec) cudaGraphExecDestroy(render_exec);
	for (void *p : allocations) cudaFree(p);
	// pool blocks (the scene arrays, the render workspace) go back to the pool in stream order
	for (void *p : pool_allocations) cudaFreeAsync(p, stream);
	// the host counters are read only after a synchronisation, and nothing of this scene is left in
	// flight that writes them
	are_core::pinned_block_release(host_counters);
	are_core::release_runtime(this);
}
