// guided_mega.cu — are_render_guided on the megakernel schedule: online
// neural path guiding inside the persistent path loop.
//
// The network cannot run once per guided vertex at megakernel rates (63.5
// kFLOP per row: billions of vertices per second would need hundreds of
// PFLOP/s), so its outputs are cached.  The scene's bounding box is split
// into cache_res^3 cells, each with six entries, one per dominant normal
// direction (+x, -x, +y, -y, +z, -z).  After every training step the
// network (tcgen05 inference, guide.cu) is evaluated once per entry at the
// cell's centre, with the entry's axis as the normal and as the outgoing
// direction, and writes the entry's packed 8-lobe vMF mixture (192 bytes).
// A guided vertex reads the entry of its cell and normal: one-sample MIS of
// that mixture and cosine sampling, weighted by the combined density, so the
// image is unbiased whatever the cache holds (the density used is exactly
// the one sampled).
//
// A frame runs as passes: pass k renders samples [s_k, s_k+1) of every pixel
// (work items are chunk-major, so a pass is a contiguous range of one-sample
// items) in one persistent launch; between passes the host runs the Adam
// steps on the training samples the pass collected and refreshes the cache.
// Passes grow from about 2^18 samples to about 2^24, so a fresh network gets
// its first steps early.  Training samples come from a random subset of
// paths (probability chosen per pass for about one batch): such a path
// records its guided vertices (features, direction, density, cosine,
// throughput after the vertex, radiance gathered before it) in its slot's
// records in device memory, and when it ends each recorded vertex becomes a
// sample (features, direction, weight = lum(incident radiance) cos / pdf).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "guide.cuh"
#include "guide_host.h"
#include "mega.cuh"
#include "path.cuh"
#include "scene.h"
#include "wave.cuh"

namespace are_core {

namespace {

constexpr int MG_GV = 4;  // recorded guided vertices per path (the first diffuse bounces)

struct MixtureCache {
	const float *mix;  // packed mixtures, GN_OUT floats per entry
	int32_t gx, gy, gz;
	float lo[3], inv_cell[3];
};

struct GuidedMega {
	MixtureCache C;
	float4 *vrec;      // per slot, MG_GV records of 6 float4
	float *tbuf;       // training samples, 16 floats each
	unsigned *tcount;  // samples written (may pass the capacity)
	unsigned tcap;
	GuideBox box;
	float mix;
	float rec_prob;    // probability that a path records training samples
	int32_t guide_depth;
};

// entry of the cell holding p, for the normal bin of n (the axis of |n|'s largest component and its sign)
__device__ __forceinline__ int cache_entry(const MixtureCache &C, f3 p, f3 n) {
	const int ix = min(max((int)((p.x - C.lo[0]) * C.inv_cell[0]), 0), C.gx - 1);
	const int iy = min(max((int)((p.y - C.lo[1]) * C.inv_cell[1]), 0), C.gy - 1);
	const int iz = min(max((int)((p.z - C.lo[2]) * C.inv_cell[2]), 0), C.gz - 1);
	const float ax = fabsf(n.x), ay = fabsf(n.y), az = fabsf(n.z);
	const int axis = ax >= ay && ax >= az ? 0 : (ay >= az ? 1 : 2);
	const float c = axis == 0 ? n.x : axis == 1 ? n.y : n.z;
	return ((iz * C.gy + iy) * C.gx + ix) * 6 + 2 * axis + (c < 0.f ? 1 : 0);
}

// network inputs of every cache entry: the cell's centre, the entry's axis as normal and outgoing direction
__global__ void k_cache_features(MixtureCache C, GuideBox B, float *__restrict__ feat, int n_entries) {
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n_entries; e += gridDim.x * blockDim.x) {
		const int bin = e % 6, cell = e / 6;
		const int ix = cell % C.gx, iy = (cell / C.gx) % C.gy, iz = cell / (C.gx * C.gy);
		const f3 p{ C.inv_cell[0] > 0.f ? C.lo[0] + (ix + 0.5f) / C.inv_cell[0] : C.lo[0],
			C.inv_cell[1] > 0.f ? C.lo[1] + (iy + 0.5f) / C.inv_cell[1] : C.lo[1],
			C.inv_cell[2] > 0.f ? C.lo[2] + (iz + 0.5f) / C.inv_cell[2] : C.lo[2] };
		const float sgn = (bin & 1) ? -1.f : 1.f;
		const f3 n{ bin / 2 == 0 ? sgn : 0.f, bin / 2 == 1 ? sgn : 0.f, bin / 2 == 2 ? sgn : 0.f };
		float x[GN_IN];
		guide_features(B, p, n, n, x);
		for (int k = 0; k < GN_IN; ++k) feat[(size_t)e * GN_IN + k] = x[k];
	}
}

// queue 0 takes the first camera rays of work items [item_begin, item_begin + n_first); slot sums cleared
__global__ void __launch_bounds__(BLOCK) k_init_range(Wave W, int n_first, int64_t item_begin) {
	for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < W.P; s += gridDim.x * blockDim.x) {
		W.acc_s[s] = make_float4(0.f, 0.f, 0.f, 0.f);
		W.acc_c[s] = make_float4(0.f, 0.f, 0.f, 0.f);
		W.acc_q[s] = make_float4(0.f, 0.f, 0.f, 0.f);
		if (s < n_first) put_camera_ray(W, 0, (unsigned)s, s, item_begin + s, 0);
	}
}

// whether the path with random-number key `key` records training samples (counter 5 of its key: unused
// by the camera ray, 0..3, and by the bounces, 8 on)
__device__ __forceinline__ bool records(const GuidedMega &G, uint64_t key) {
	return G.rec_prob > 0.f && uniform(key, 5) < G.rec_prob;
}

// A finished path's recorded vertices become training samples: incident radiance along the sampled
// direction L_in = (L_final - L_before) / beta_after, weight lum(L_in) cos / pdf.
__device__ __forceinline__ void emit_samples(const GuidedMega &G, int slot, f3 L, unsigned vmask,
	unsigned long long &emitted) {
	for (int v = 0; v < MG_GV; ++v) {
		if (!((vmask >> v) & 1u)) continue;
		const float4 *r = G.vrec + ((size_t)slot * MG_GV + v) * 6;
		const float4 r3 = r[3], r4 = r[4], r5 = r[5];
		const float li[3] = { r4.x > 0.f ? (L.x - r5.x) / r4.x : 0.f, r4.y > 0.f ? (L.y - r5.y) / r4.y : 0.f,
			r4.z > 0.f ? (L.z - r5.z) / r4.z : 0.f };
		const float lum = 0.2126f * li[0] + 0.7152f * li[1] + 0.0722f * li[2];
		const float wt = lum * r3.y / r3.x;
		if (!(wt > 0.f && isfinite(wt))) continue;
		const unsigned pos = atomicAdd(G.tcount, 1u);
		++emitted;
		if (pos >= G.tcap) continue;
		float4 *o = reinterpret_cast<float4 *>(G.tbuf + (size_t)pos * 16);
		o[0] = r[0], o[1] = r[1], o[2] = r[2], o[3] = make_float4(wt, 0.f, 0.f, 0.f);
	}
}

// A guided diffuse vertex: direction from the cached mixture with probability mix, else cosine
// sampling; throughput times albedo cos / (pi pdf) with pdf = mix q + (1 - mix) cos / pi.  Russian
// roulette survives with max(beta) rrs, rrs dividing out the guided bounces' pdf ratios.  Returns
// false if the path ends here.
template <bool TRAIN>
__device__ __forceinline__ bool guided_bounce(const DevScene &S, const GuidedMega &G, const Surface &sf, f3 d,
	uint64_t key, int depth, int rr_depth, f3 &beta, f3 L, f3 &nd, float &rrs, bool rec, int slot, unsigned &vmask,
	unsigned long long &gverts, unsigned long long &recorded) {
	const f3 nrm = dot(d, sf.ng) < 0.f ? sf.ng : scl(sf.ng, -1.f);
	const float *M = G.C.mix + (size_t)cache_entry(G.C, sf.p, nrm) * GN_OUT;
	const uint32_t cb = ctr_bounce(depth);
	++gverts;
	// Both techniques draw a direction around an axis: the cosine lobe around the normal (rt.cpp:284-289,
	// the plain lambertian bounce's random numbers and arithmetic), or a vMF lobe around its mean; only the
	// choice of axis and of the polar cosine differs, so the warp shares the rest (one sincos, one frame).
	const bool guide = uniform(key, cb + 4) < G.mix;
	f3 axis = nrm;
	float phi_u, rs, wz = 0.f;
	if (guide) {
		// the first lobe whose cumulative weight exceeds u0 (the last if rounding leaves u0 above the total)
		const float u0 = uniform(key, cb + 7), u1 = uniform(key, cb + 5);
		int sel = GN_LOBES - 1;
		float acc = 0.f;
#pragma unroll
		for (int l = 0; l < GN_LOBES - 1; ++l) {
			acc += M[32 + 2 * l];
			if (sel == GN_LOBES - 1 && u0 < acc) sel = l;
		}
		const float4 a = reinterpret_cast<const float4 *>(M)[sel];
		// W. Jakob's stable vMF sampling: cos(theta) = 1 + log(u1 + (1 - u1) e^-2kappa) / kappa
		wz = fminf(fmaxf(1.f + logf(u1 + (1.f - u1) * __expf(-2.f * a.w)) / a.w, -1.f), 1.f);
		rs = sqrtf(fmaxf(0.f, 1.f - wz * wz));
		axis = f3{ a.x, a.y, a.z };
		phi_u = uniform(key, cb + 6);
	} else {
		phi_u = uniform(key, cb);
		rs = sqrtf(uniform(key, cb + 1));
	}
	float s, c;
	sincosf(6.28318530717958647692f * phi_u, &s, &c);
	const float lx = rs * c, ly = rs * s;
	if (!guide) {
		const float t = 1.0f - lx * lx - ly * ly;  // rt.cpp:50-55 rotateToHemisphere, as hemi()
		wz = sqrtf(t > 0.f ? t : 0.f);
	}
	const f3 up = fabsf(axis.z) < 0.999f ? f3{ 0.f, 0.f, 1.f } : f3{ 1.f, 0.f, 0.f };
	const f3 tg = norm(cross(axis, up));
	const f3 bt = cross(axis, tg);
	const f3 w = norm(add(add(scl(tg, lx), scl(bt, ly)), scl(axis, wz)));
	const float cosw = dot(w, nrm);
	if (!(cosw > 0.f)) return false;
	const float inv_pi = 0.31830988618379067154f;
	const float pdf = G.mix * packed_pdf(M, w) + (1.f - G.mix) * cosw * inv_pi;
	const DevMaterial &m = S.mats[sf.mat];
	const f3 alb = tex_albedo(S, m.texture, sf);
	const float ratio = cosw * inv_pi / pdf;  // cosine-sampling pdf over the MIS pdf
	beta = mulv(beta, scl(alb, ratio));
	rrs = fminf(fmaxf(rrs / ratio, 1e-30f), 1e30f);
	if (rr_depth >= 0 && depth >= rr_depth) {
		const float q = fmaxf(fmaxf(beta.x, beta.y), beta.z) * rrs;
		if (q < 1.0f) {
			if (uniform(key, cb + 3) >= q) return false;
			beta = scl(beta, 1.0f / q);
		}
	}
	if (TRAIN && rec && depth < MG_GV) {
		float x[GN_IN];
		guide_features(G.box, sf.p, nrm, scl(d, -1.f), x);
		float4 *v = G.vrec + ((size_t)slot * MG_GV + depth) * 6;
		v[0] = make_float4(x[0], x[1], x[2], x[3]);
		v[1] = make_float4(x[4], x[5], x[6], x[7]);
		v[2] = make_float4(x[8], w.x, w.y, w.z);
		v[3] = make_float4(pdf, cosw, 0.f, 0.f);
		v[4] = make_float4(beta.x, beta.y, beta.z, 0.f);
		v[5] = make_float4(L.x, L.y, L.z, 0.f);
		vmask |= 1u << depth;
		++recorded;
	}
	nd = w;
	return true;
}

// Per-path guiding state carried beside PathState.
struct GuideTrack {
	float rrs;       // roulette scale (1 on unguided paths)
	unsigned vmask;  // recorded vertices
	bool rec;        // this path records training samples
};

// One bounce of path P at hit h, as render.cu's shade_step with the slot's sums in registers, plus the
// guided vertices and the training samples.  Returns true if P holds a ray to trace.
template <bool TRAIN>
__device__ __forceinline__ bool guided_step(const DevScene &S, const Wave &W, const GuidedMega &G, PathState &P,
	GuideTrack &T, float4 h, uint32_t &err, unsigned long long &done, unsigned long long &gverts,
	unsigned long long &emitted, unsigned long long &recorded, float4 &sm, float4 &cm, float4 &q) {
	const int leaf = __float_as_int(h.y);
	if (leaf < 0) {
		P.L = add(P.L, mulv(P.beta, background(S, P.d)));
	} else {
		const uint64_t key = P.key;
		const Surface sf = surface_at(S, leaf, P.o, P.d, h.x, h.z, h.w);
		f3 nd;
		bool cont;
		if (P.depth < G.guide_depth && S.mats[sf.mat].type == ARE_MAT_LAMBERTIAN)
			cont = guided_bounce<TRAIN>(S, G, sf, P.d, key, P.depth, W.rr_depth, P.beta, P.L, nd, T.rrs, T.rec, P.slot,
				T.vmask, gverts, recorded);
		else
			cont = scatter(S, sf, P.d, key, P.depth, W.rr_depth, P.beta, P.L, nd, T.rrs);
		if (cont && P.depth + 1 >= W.max_depth) cont = false;
		if (cont) {
			P.o = sf.p;
			P.d = nd;
			++P.depth;
			return true;
		}
	}
	if (TRAIN && T.vmask) emit_samples(G, P.slot, P.L, T.vmask, emitted);
	++done;
	int64_t item = P.item;
	int j = P.j;
	if (!accumulate(W, P.L, item, j, err, &W.cnt[3], sm, cm, q)) return false;
	camera_path(W, P.slot, item, j, P);
	T = GuideTrack{ 1.0f, 0u, TRAIN && records(G, P.key) };
	return true;
}

// The guided megakernel: k_tail (render.cu) with guided_step for the bounce.  One path per resident
// thread, the slot's sums in registers; queue 0 holds the pass's first camera paths.  TRAIN: the
// instantiation that records training samples (a render with a frozen network runs the one without,
// a smaller loop).
template <bool LINEAR, bool WIDE, bool TRAIN>
__global__ void __launch_bounds__(BLOCK, tail_min_blocks(LINEAR, WIDE, WIDE))
	k_guided_tail(DevScene S, Wave W, GuidedMega G) {
	__shared__ float4 snodes[LINEAR ? 6 * LINEAR_MAX : WIDE ? 8 * TAIL_SMEM_NODES4 : 2 * SMEM_NODES];
	__shared__ WarpHitScratch scratch[LINEAR ? BLOCK / 32 : 1];
	constexpr int SHORT = WIDE ? TAIL_SHORT_STACK_WIDE : TAIL_SHORT_STACK;
	__shared__ int4 sstack[LINEAR ? 1 : SHORT * BLOCK];
	int n_snodes = 0;
	const unsigned n = W.cnt[0];
	if ((unsigned)(blockIdx.x * blockDim.x) >= n) return;
	if (LINEAR) {
		stage_prims(S, snodes);
		__syncthreads();
	} else if (WIDE) {
		stage_nodes4(S, snodes, n_snodes, TAIL_SMEM_NODES4);
	} else {
		stage_nodes(S, snodes, n_snodes);
	}
	uint32_t err = 0;
	unsigned long long done = 0, segments = 0, gverts = 0, emitted = 0, recorded = 0;
	const float inf = __int_as_float(0x7f800000);
	if constexpr (WIDE) {
		PathState P{};
		GuideTrack T{ 1.0f, 0u, false };
		float4 sm{}, cm{}, q{};
		interleaved_walks<SHORT, true>(S, snodes, n_snodes, sstack + threadIdx.x, W.t_min, blockIdx.x * blockDim.x + threadIdx.x,
			n, gridDim.x * blockDim.x, P, err, segments,
			[&](unsigned i) {
				P = load_path(W, 0, i);
				sm = W.acc_s[P.slot], cm = W.acc_c[P.slot], q = W.acc_q[P.slot];
				sm.w = cm.w = q.w = 0.f;
				T = GuideTrack{ 1.0f, 0u, TRAIN && records(G, P.key) };
			},
			[&](float4 h) {
				return guided_step<TRAIN>(S, W, G, P, T, h, err, done, gverts, emitted, recorded, sm, cm, q);
			},
			[&]() { W.acc_s[P.slot] = sm, W.acc_c[P.slot] = cm, W.acc_q[P.slot] = q; });
	} else {
		for (unsigned base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
			const unsigned i = base + threadIdx.x;
			bool live = i < n;
			PathState P{};
			GuideTrack T{ 1.0f, 0u, false };
			float4 sm{}, cm{}, q{};
			if (live) {
				P = load_path(W, 0, i);
				sm = W.acc_s[P.slot], cm = W.acc_c[P.slot], q = W.acc_q[P.slot];
				sm.w = cm.w = q.w = 0.f;
				T.rec = TRAIN && records(G, P.key);
			}
			const int slot = P.slot;
			if (LINEAR) {
				// every lane stays in the loop while any lane of its warp has a path (cooperative closest hit)
				WarpHitScratch &ws = scratch[threadIdx.x >> 5];
				while (__any_sync(0xffffffffu, live)) {
					Hit hh = closest_hit_linear_warp(snodes, S.n_leaves, S.triangle_test, P.o, P.d, W.t_min, inf, live, ws);
					if (live) {
						++segments;
						live = guided_step<TRAIN>(S, W, G, P, T, make_float4(hh.t, __int_as_float(hh.leaf), hh.u, hh.v),
							err, done, gverts, emitted, recorded, sm, cm, q);
					}
				}
			} else {
				while (live) {
					Hit hh = closest_hit<SHORT>(S, snodes, n_snodes, P.o, P.d, W.t_min, inf, err, sstack + threadIdx.x);
					++segments;
					live = guided_step<TRAIN>(S, W, G, P, T, make_float4(hh.t, __int_as_float(hh.leaf), hh.u, hh.v), err,
						done, gverts, emitted, recorded, sm, cm, q);
				}
			}
			if (i < n) W.acc_s[slot] = sm, W.acc_c[slot] = cm, W.acc_q[slot] = q;
		}
	}
	for (int o = 16; o > 0; o >>= 1) {
		done += __shfl_down_sync(0xffffffffu, done, o);
		segments += __shfl_down_sync(0xffffffffu, segments, o);
		gverts += __shfl_down_sync(0xffffffffu, gverts, o);
		emitted += __shfl_down_sync(0xffffffffu, emitted, o);
		recorded += __shfl_down_sync(0xffffffffu, recorded, o);
	}
	if (lane_id() == 0) {
		if (done) atomicAdd(&W.stat[1], done);
		if (segments) atomicAdd(&W.stat[0], segments);
		if (emitted) atomicAdd(&W.stat[2], emitted);
		if (gverts) atomicAdd(&W.stat[3], gverts);
		if (recorded) atomicAdd(&W.stat[4], recorded);
	}
	if (err) atomicOr(&W.cnt[4], err);
}

const void *guided_tail_fn(bool linear, const DevScene &S) {
	// both instantiations of a scene kind have the same launch bounds; the training one sizes the grid
	if (linear) return (const void *)k_guided_tail<true, false, true>;
	return S.n_nodes4 > 0 ? (const void *)k_guided_tail<false, true, true> : (const void *)k_guided_tail<false, false, true>;
}

void launch_guided_tail(bool linear, bool train, int grid, cudaStream_t s, const DevScene &S, const Wave &W,
	const GuidedMega &G) {
	const bool wide = S.n_nodes4 > 0;
	if (train) {
		if (linear)
			k_guided_tail<true, false, true><<<grid, BLOCK, 0, s>>>(S, W, G);
		else if (wide)
			k_guided_tail<false, true, true><<<grid, BLOCK, 0, s>>>(S, W, G);
		else
			k_guided_tail<false, false, true><<<grid, BLOCK, 0, s>>>(S, W, G);
	} else {
		if (linear)
			k_guided_tail<true, false, false><<<grid, BLOCK, 0, s>>>(S, W, G);
		else if (wide)
			k_guided_tail<false, true, false><<<grid, BLOCK, 0, s>>>(S, W, G);
		else
			k_guided_tail<false, false, false><<<grid, BLOCK, 0, s>>>(S, W, G);
	}
}

are_status bad(const std::string &m) {
	set_error(m);
	return ARE_ERR_INVALID_ARGUMENT;
}

template <class T>
T *carve(char *&p, size_t count) {
	T *r = (T *)p;
	p += (count * sizeof(T) + 255) & ~(size_t)255;
	return r;
}

int grid_of(const void *k, int n_sms) {
	int per = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, BLOCK, 0);
	return std::max(1, per) * n_sms;
}

}  // namespace

// pass sizes in samples: the first about 2^18, doubling to about 2^24
constexpr int64_t MG_FIRST_PASS = 1 << 18, MG_MAX_PASS = 1 << 24;
// Adam steps a network must have taken in its lifetime before a training render samples from it: a
// fresh network's mixture sends paths in arbitrary directions, which costs more samples than it saves,
// so until then such a pass guides with mix 0 (cosine sampling only) and only collects training samples
constexpr int64_t MG_MIN_STEPS = 16;

are_status render_guided_mega(are_scene *sc, GuideNet *net, const are_camera *cam, const are_render_params &p,
	const are_guide_params *gp, float *rgb, float *var, are_render_stats *stats) {
	const int res = gp->cache_res > 0 ? gp->cache_res : 32;
	if (res > 128) return bad("cache_res must be at most 128");
	Wave W{};
	W.npix = p.width * p.height;
	W.spp = p.spp;
	W.chunk = 1;  // one-sample work items: a pass is a contiguous range of items
	W.nchunk = p.spp;
	const int64_t total_items = (int64_t)W.npix * p.spp;
	if (total_items >= (int64_t)UINT32_MAX - (1 << 24)) return bad("too many samples in one frame");
	const bool linear = sc->linear;
	const int g_tail = grid_of(guided_tail_fn(linear, sc->dev), sc->n_sms);
	int P = p.pool_size > 0 ? std::min(p.pool_size, g_tail * BLOCK) : g_tail * BLOCK;
	P = (P + 31) & ~31;
	W.P = P;
	W.max_depth = p.max_depth;
	W.rr_depth = p.rr_depth;
	W.t_min = p.t_min;
	W.seed = p.seed;
	camera_frame(*cam, p.width, p.height, p.flags, W.cam);

	GuidedMega G{};
	G.mix = gp->mix;
	G.guide_depth = gp->guide_depth;
	// training samples collect across passes, up to four batches, until a step takes them
	const unsigned batch = (unsigned)std::max(gp->batch, 256);
	const unsigned tcap = 4 * batch;
	G.tcap = tcap;
	for (int k = 0; k < 3; ++k) {
		const float lo = sc->box_lo[k], ext = sc->box_hi[k] - sc->box_lo[k];
		G.box.lo[k] = lo;
		G.box.inv_ext[k] = ext > 0.f ? 1.f / ext : 0.f;
		G.C.lo[k] = lo;
		G.C.inv_cell[k] = ext > 0.f ? (float)res / ext : 0.f;
	}
	G.C.gx = G.C.gy = G.C.gz = res;
	const int n_entries = res * res * res * 6;

	size_t need = 0;
	char *z = nullptr;
	carve<float4>(z, P), carve<float4>(z, P), carve<float4>(z, P), carve<float4>(z, P);  // queue 0
	carve<float4>(z, P), carve<float4>(z, P), carve<float4>(z, P);                        // slot sums
	carve<unsigned>(z, 64), carve<unsigned long long>(z, 8);
	carve<float>(z, (size_t)n_entries * GN_OUT), carve<float>(z, (size_t)n_entries * GN_IN);
	carve<float4>(z, (size_t)P * MG_GV * 6), carve<float>(z, (size_t)tcap * 16);
	carve<float4>(z, total_items), carve<float>(z, 3 * (size_t)W.npix), carve<float>(z, 3 * (size_t)W.npix);
	need = (size_t)z;
	void *mem = nullptr;
	if (are_status st = pool_alloc(sc, need, &mem)) return st;
	z = (char *)mem;
	W.qa[0] = W.qa[1] = carve<float4>(z, P);
	W.qb[0] = W.qb[1] = carve<float4>(z, P);
	W.qc[0] = W.qc[1] = carve<float4>(z, P);
	W.qd[0] = W.qd[1] = carve<float4>(z, P);
	W.hit = nullptr;
	W.acc_s = carve<float4>(z, P), W.acc_c = carve<float4>(z, P), W.acc_q = carve<float4>(z, P);
	W.cnt = carve<unsigned>(z, 64);
	W.stat = carve<unsigned long long>(z, 8);
	float *cache_mix = carve<float>(z, (size_t)n_entries * GN_OUT);
	float *cache_feat = carve<float>(z, (size_t)n_entries * GN_IN);
	G.C.mix = cache_mix;
	G.vrec = carve<float4>(z, (size_t)P * MG_GV * 6);
	G.tbuf = carve<float>(z, (size_t)tcap * 16);
	W.item_s = carve<float4>(z, total_items);
	W.item_q = nullptr;  // one-sample items: resolve squares the sums
	float *d_rgb = carve<float>(z, 3 * (size_t)W.npix);
	float *d_var = carve<float>(z, 3 * (size_t)W.npix);
	G.tcount = W.cnt + 7;

	cudaStream_t s = sc->stream;
	const bool dev_out = (p.flags & ARE_FLAG_DEVICE_OUTPUT) != 0;
	// events: [0] [1] around the render; per pass two around the megakernel, two around training and
	// the cache refresh (reused pass after pass: each pass synchronises before the next)
	while (sc->render_events.size() < 8) {
		cudaEvent_t e = nullptr;
		cudaEventCreate(&e);
		sc->render_events.push_back(e);
	}
	cudaEvent_t *ev = sc->render_events.data();
	double kms[4] = { 0.0, 0.0, 0.0, 0.0 };
	int64_t launches[4] = { 0, 0, 0, 0 }, train_steps = 0, passes = 0;
	unsigned *hc = sc->host_counters;
	cudaGetLastError();
	cudaEventRecord(ev[0], s);
	are_status st = cuda_status(cudaMemsetAsync(W.stat, 0, 8 * sizeof(unsigned long long), s), "stats");
	if (!st) st = cuda_status(cudaMemsetAsync(W.cnt, 0, 64 * sizeof(unsigned), s), "counters");
	if (!st) {
		k_cache_features<<<std::max(1, std::min(4096, (n_entries + 255) / 256)), 256, 0, s>>>(G.C, G.box, cache_feat,
			n_entries);
		++launches[ARE_KERNEL_OTHER];
		st = cuda_status(cudaGetLastError(), "k_cache_features");
	}
	auto refresh = [&]() -> are_status {
		++launches[ARE_KERNEL_GENERATE];
		return net->infer(cache_feat, n_entries, cache_mix, s, nullptr, W.cnt + 4, true);
	};
	if (!st) {
		cudaEventRecord(ev[4], s);
		st = refresh();
		cudaEventRecord(ev[5], s);
	}
	bool refresh_timed = !st;
	const unsigned tmin = std::max(256u, batch / 4);  // a step needs a quarter batch: fewer make a noisy gradient
	// measured after each pass: guided vertices per sample, and the fraction of recorded vertices whose
	// path brought back radiance (a training sample needs a positive weight; in a scene lit mostly
	// indirectly that is a small fraction, and the paths record with probability up to 1)
	double gv_per_sample = 1.5, useful = 0.01;
	unsigned held = 0;  // samples in the training buffer
	unsigned long long prev_samples = 0, prev_gverts = 0, prev_emitted = 0, prev_recorded = 0;
	int64_t spp_done = 0;
	int64_t pass_spp = std::max<int64_t>(1, MG_FIRST_PASS / W.npix);
	const int64_t max_pass_spp = std::max<int64_t>(1, MG_MAX_PASS / W.npix);
	while (!st && spp_done < p.spp) {
		const int64_t sp = std::min<int64_t>(pass_spp, p.spp - spp_done);
		const int64_t begin = spp_done * W.npix, end = (spp_done + sp) * W.npix;
		W.n_items = end;
		const int n_first = (int)std::min<int64_t>(P, end - begin);
		G.mix = (gp->train && net->steps < MG_MIN_STEPS) ? 0.0f : gp->mix;
		// training samples: a random subset of the pass's paths, sized to fill about 0.8 of the room left
		// in the buffer with positive weights
		const double expect = (double)(end - begin) * std::max(0.05, gv_per_sample) * std::max(1e-5, useful);
		const bool training = gp->train && (gp->max_steps <= 0 || train_steps < gp->max_steps);
		G.rec_prob = training ? (float)std::min(1.0, 0.8 * (double)(tcap - held) / expect) : 0.f;
		for (int k = 0; k < 8; ++k) hc[k] = 0u;
		hc[0] = (unsigned)n_first;
		hc[3] = (unsigned)(begin + n_first);
		st = cuda_status(cudaMemcpyAsync(W.cnt, hc, 4 * sizeof(unsigned), cudaMemcpyHostToDevice, s), "counters");
		if (!st) {
			k_init_range<<<grid_of((const void *)k_init_range, sc->n_sms), BLOCK, 0, s>>>(W, n_first, begin);
			++launches[ARE_KERNEL_OTHER];
			cudaEventRecord(ev[2], s);
			launch_guided_tail(linear, G.rec_prob > 0.f, g_tail, s, sc->dev, W, G);
			cudaEventRecord(ev[3], s);
			++launches[ARE_KERNEL_SHADE];
			st = cuda_status(cudaGetLastError(), "k_guided_tail launch");
		}
		if (!st) {
			cudaMemcpyAsync(hc + 16, W.stat, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
			cudaMemcpyAsync(hc + 8, G.tcount, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
			st = cuda_status(cudaStreamSynchronize(s), "guided pass");
		}
		if (st) break;
		++passes;
		float ms = 0.f;
		if (cudaEventElapsedTime(&ms, ev[2], ev[3]) == cudaSuccess) kms[ARE_KERNEL_SHADE] += ms;
		if (refresh_timed && cudaEventElapsedTime(&ms, ev[4], ev[5]) == cudaSuccess) kms[ARE_KERNEL_GENERATE] += ms;
		refresh_timed = false;
		const unsigned long long *hs = reinterpret_cast<const unsigned long long *>(hc + 16);
		if (hs[1] > prev_samples) gv_per_sample = (double)(hs[3] - prev_gverts) / (double)(hs[1] - prev_samples);
		if (hs[4] > prev_recorded + 64) useful = (double)(hs[2] - prev_emitted) / (double)(hs[4] - prev_recorded);
		prev_samples = hs[1], prev_gverts = hs[3], prev_emitted = hs[2], prev_recorded = hs[4];
		spp_done += sp;
		pass_spp = std::min(max_pass_spp, 2 * pass_spp);
		const unsigned have = std::min(hc[8], tcap);
		held = have;
		if (training && have >= tmin && spp_done < p.spp) {
			// `train` Adam steps on each full batch collected (or on the partial batch when there is no
			// full one), then the cache for the next pass; the buffer starts over
			net->weight_clip = gp->weight_clip > 0.f ? gp->weight_clip : 1e30f;
			const unsigned nb = std::max(1u, have / batch), rows = have >= batch ? batch : have;
			cudaEventRecord(ev[6], s);
			for (unsigned b = 0; b < nb && !st; ++b)
				for (int k = 0; k < gp->train && !st && (gp->max_steps <= 0 || train_steps < gp->max_steps); ++k) {
					st = net->train_step(G.tbuf + (size_t)b * batch * 16, (int)rows, -1.0f, gp->lr, s, W.cnt + 4);
					++train_steps;
					launches[ARE_KERNEL_OTHER] += 7;
				}
			cudaEventRecord(ev[7], s);
			cudaMemsetAsync(G.tcount, 0, sizeof(unsigned), s);
			held = 0;
			cudaMemcpyAsync(hc + 28, net->grad + GN_PARAMS, 4, cudaMemcpyDeviceToHost, s);
			cudaEventRecord(ev[4], s);
			if (!st) st = refresh();
			cudaEventRecord(ev[5], s);
			refresh_timed = true;
			if (!st) st = cuda_status(cudaStreamSynchronize(s), "guided training");
			if (!st) {
				net->loss_log.push_back(*reinterpret_cast<float *>(&hc[28]) / (float)rows);
				if (cudaEventElapsedTime(&ms, ev[6], ev[7]) == cudaSuccess) kms[ARE_KERNEL_OTHER] += ms;
			}
		}
	}
	if (!st) {
		k_resolve<<<std::max(1, std::min(4096, (W.npix + BLOCK - 1) / BLOCK)), BLOCK, 0, s>>>(
			W, dev_out ? rgb : d_rgb, var ? (dev_out ? var : d_var) : nullptr, (p.flags & ARE_FLAG_CLAMP_OUTPUT) != 0);
		++launches[ARE_KERNEL_OTHER];
		st = cuda_status(cudaGetLastError(), "k_resolve");
	}
	cudaEventRecord(ev[1], s);
	unsigned long long hstat[4] = { 0, 0, 0, 0 };
	unsigned herr = 0;
	if (!st) {
		unsigned long long *ps = reinterpret_cast<unsigned long long *>(hc + 32);
		cudaMemcpyAsync(ps, W.stat, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
		cudaMemcpyAsync(hc + 40, W.cnt + 4, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
		if (!dev_out) {
			cudaMemcpyAsync(rgb, d_rgb, 3 * sizeof(float) * W.npix, cudaMemcpyDeviceToHost, s);
			if (var) cudaMemcpyAsync(var, d_var, 3 * sizeof(float) * W.npix, cudaMemcpyDeviceToHost, s);
		}
		st = cuda_status(cudaStreamSynchronize(s), "guided render");
		if (!st) {
			for (int k = 0; k < 4; ++k) hstat[k] = ps[k];
			herr = hc[40];
		}
	}
	cudaStreamSynchronize(s);
	float total_ms = 0.f;
	cudaEventElapsedTime(&total_ms, ev[0], ev[1]);
	pool_free(sc, mem);
	if (!st && herr) {
		set_error("device error word " + std::to_string(herr));
		st = ARE_ERR_INTERNAL;
	}
	if (stats) {
		*stats = are_render_stats{};
		stats->samples = (int64_t)hstat[1];
		stats->segments = (int64_t)hstat[0];
		stats->iterations = passes;
		stats->device_ms = total_ms;
		for (int k = 0; k < 4; ++k) stats->kernel_launches[k] = launches[k], stats->kernel_ms[k] = kms[k];
		stats->error_word = (int32_t)herr;
		stats->aux[0] = (double)hstat[2];
		stats->aux[1] = (double)train_steps;
		stats->aux[2] = (double)hstat[3];
		stats->aux[3] = net->loss_log.empty() ? 0.0 : (double)net->loss_log.back();
	}
	return st;
}

}  // namespace are_core
