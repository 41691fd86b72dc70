// guided.cu — are_render_guided: the wavefront path tracer with online
// neural path guiding.
//
// Per iteration: intersect (shared with the plain render) -> select (diffuse
// hits of the first guided bounces: features into a compact list) -> infer
// (the network on the tensor cores, one row per selected hit) -> shade (at a
// guided vertex, one-sample MIS: with probability `mix` the direction comes
// from the network's vMF mixture, otherwise from cosine sampling; the weight
// is f cos / (mix q + (1 - mix) cos / pi), unbiased for any network) ->
// generate (finished paths: accumulate, then turn each recorded guided vertex
// into a training sample (features, direction, weight = luminance of the
// incident radiance the path carried back times cos / pdf) and start the next
// camera path).  Between graph launches the host runs an Adam step whenever a
// full training batch has been collected.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "guide.cuh"
#include "guide_host.h"
#include "path.cuh"
#include "scene.h"
#include "wave.cuh"

namespace are_core {

constexpr int GV = 4;  // guided vertices recorded per path (the first diffuse bounces)
// iterations per graph launch; training steps are taken between launches
constexpr int GUIDED_ITERS = 8;

struct GuidedState {
	int32_t *gidx;        // per queue position: row in the compact list or -1
	float *gfeat;         // compact list: 9 features per selected hit
	float *gout;          // compact list: 48 network outputs
	float4 *vrec;         // per slot, GV records of 6 float4
	float *tbuf;          // training samples, 16 floats each
	unsigned *tcount;     // number of samples written (may exceed capacity)
	unsigned tcap;
	GuideBox box;
	float mix;
	int guide_depth;
};

// Closest hits of the queued rays (as k_intersect), then the network's input
// list: every diffuse hit at depth < guide_depth gets its features written to
// the compact list (its row in gidx), so inference runs on that list only.
// The compact list's counter W.cnt[6] is zeroed before this kernel.
template <bool LINEAR>
__global__ void __launch_bounds__(BLOCK) k_intersect_select(DevScene S, Wave W, GuidedState G, int par) {
	__shared__ float4 snodes[LINEAR ? 6 * LINEAR_MAX : 2 * SMEM_NODES];
	__shared__ WarpHitScratch scratch[LINEAR ? BLOCK / 32 : 1];
	int n_snodes = 0;
	const unsigned n = W.cnt[par];
	if (blockIdx.x == 0 && threadIdx.x == 0) {
		W.cnt[par ^ 1] = 0;  // output queue of this iteration
		atomicAdd(&W.stat[0], (unsigned long long)n);
	}
	if ((unsigned)(blockIdx.x * blockDim.x) >= n) return;
	if (LINEAR) {
		stage_prims(S, snodes);
		__syncthreads();
	} else {
		stage_bvh(S, snodes, n_snodes);
	}
	uint32_t err = 0;
	const float inf = __int_as_float(0x7f800000);
	for (unsigned base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
		const unsigned i = base + threadIdx.x;
		bool sel = false;
		float x[GN_IN];
		float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
		if (i < n) a = W.qa[par][i], b = W.qb[par][i];
		Hit h;
		if (LINEAR)  // warp-cooperative: every lane of the warp takes part
			h = closest_hit_linear_warp(snodes, S.n_leaves, S.triangle_test, ld3(a), ld3(b), W.t_min, inf, i < n,
				scratch[threadIdx.x >> 5]);
		else if (i < n)
			h = closest_hit_any(S, snodes, n_snodes, ld3(a), ld3(b), W.t_min, inf, err);
		if (i < n) {
			const f3 o = ld3(a), d = ld3(b);
			W.hit[i] = make_float4(h.t, __int_as_float(h.leaf), h.u, h.v);
			const int depth = __float_as_int(b.w) & 0xff;
			if (h.leaf >= 0 && depth < G.guide_depth) {
				const int mat = __ldg(S.prim_mat + h.leaf);
				if (S.mats[mat].type == ARE_MAT_LAMBERTIAN) {
					const Surface sf = surface_at(S, h.leaf, o, d, h.t, h.u, h.v);
					const f3 nrm = dot(d, sf.ng) < 0.f ? sf.ng : scl(sf.ng, -1.f);
					guide_features(G.box, sf.p, nrm, scl(d, -1.f), x);
					sel = true;
				}
			}
		}
		const unsigned pos = warp_append(&W.cnt[6], sel);
		const unsigned m = __ballot_sync(0xffffffffu, sel);
		if (lane_id() == 0 && m) atomicAdd(&W.stat[3], (unsigned long long)__popc(m));
		if (i < n) G.gidx[i] = sel ? (int)pos : -1;
		if (sel)
			for (int k = 0; k < GN_IN; ++k) G.gfeat[(size_t)pos * GN_IN + k] = x[k];
	}
	if (err) atomicOr(&W.cnt[4], err);
}

__global__ void __launch_bounds__(BLOCK) k_shade_guided(DevScene S, Wave W, GuidedState G, int par) {
	const unsigned n = W.cnt[par];
	const int out = par ^ 1;
	uint32_t err = 0;
	unsigned long long done = 0;
	for (unsigned base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
		unsigned i = base + threadIdx.x;
		bool valid = i < n;
		bool cont = false, term = false;
		f3 p, nd, beta, L;
		float4 ra, rb, rc;
		// qd.w packs the path's roulette scale (a positive float, low 4 mantissa
		// bits dropped; 0 at the camera means 1) with the recorded-vertex mask:
		// bit v set = guided vertex v of this path is recorded in vrec
		unsigned vmask = 0;
		float rrs = 1.0f;
		if (valid) {
			ra = W.qa[par][i];
			rb = W.qb[par][i];
			rc = W.qc[par][i];
			float4 rd = W.qd[par][i];
			const unsigned packed = __float_as_uint(rd.w);
			vmask = packed & 0xfu;
			if (packed & ~0xfu) rrs = __uint_as_float(packed & ~0xfu);
			float4 h = W.hit[i];
			beta = ld3(rc);
			L = ld3(rd);
			int meta = __float_as_int(rb.w);
			int depth = meta & 0xff, j = meta >> 8;
			int slot = __float_as_int(ra.w);
			f3 o = ld3(ra), d = ld3(rb);
			int leaf = __float_as_int(h.y);
			if (leaf < 0) {
				L = add(L, mulv(beta, background(S, d)));
			} else {
				int pixel, sample;
				{
					const uint32_t it = (uint32_t)__float_as_int(rc.w), np = (uint32_t)W.npix;
					const uint32_t ch = it / np;
					pixel = (int)(it - ch * np);
					sample = (int)ch * W.chunk + j;
				}
				uint64_t key = path_key(W.seed, (uint32_t)pixel, (uint32_t)sample);
				Surface sf = surface_at(S, leaf, o, d, h.x, h.z, h.w);
				int gi = G.gidx[i];
				if (gi >= 0) {
					// guided diffuse vertex: one-sample MIS of the vMF mixture and cosine sampling
					const float *M = G.gout + (size_t)gi * GN_OUT;
					f3 nrm = dot(d, sf.ng) < 0.f ? sf.ng : scl(sf.ng, -1.f);
					uint32_t cb = ctr_bounce(depth);
					f3 w;
					if (uniform(key, cb + 4) < G.mix) {
						w = packed_sample(M, uniform(key, cb + 7), uniform(key, cb + 5), uniform(key, cb + 6));
					} else {
						float r1 = uniform(key, cb), r2 = uniform(key, cb + 1);
						float s, c;
						sincosf(6.28318530717958647692f * r1, &s, &c);
						float r2s = sqrtf(r2);
						w = norm(hemi(nrm, r2s * c, r2s * s));
					}
					float cosw = dot(w, nrm);
					if (cosw > 0.f) {
						const float inv_pi = 0.31830988618379067154f;
						float pdf = G.mix * packed_pdf(M, w) + (1.f - G.mix) * cosw * inv_pi;
						const DevMaterial &m = S.mats[sf.mat];
						f3 alb = tex_albedo(S, m.texture, sf);
						f3 L_before = L;
						const float ratio = cosw * inv_pi / pdf;  // cosine-sampling pdf over the MIS pdf
						beta = mulv(beta, scl(alb, ratio));
						rrs = fminf(fmaxf(rrs / ratio, 1e-30f), 1e30f);
						nd = w;
						cont = true;
						if (W.rr_depth >= 0 && depth >= W.rr_depth) {
							float q = fmaxf(fmaxf(beta.x, beta.y), beta.z) * rrs;
							if (q < 1.0f) {
								if (uniform(key, cb + 3) >= q)
									cont = false;
								else
									beta = scl(beta, 1.0f / q);
							}
						}
						if (cont && depth < GV) {
							// record the vertex for training: features, direction, pdf, cos, the throughput
							// after this vertex (roulette included) and the radiance gathered before it
							float x[GN_IN];
							guide_features(G.box, sf.p, nrm, scl(d, -1.f), x);
							float4 *v = G.vrec + ((size_t)slot * GV + depth) * 6;
							v[0] = make_float4(x[0], x[1], x[2], x[3]);
							v[1] = make_float4(x[4], x[5], x[6], x[7]);
							v[2] = make_float4(x[8], w.x, w.y, w.z);
							v[3] = make_float4(pdf, cosw, 0.f, 0.f);
							v[4] = make_float4(beta.x, beta.y, beta.z, 0.f);
							v[5] = make_float4(L_before.x, L_before.y, L_before.z, 0.f);
							vmask |= 1u << depth;
						}
					}
				} else {
					cont = scatter(S, sf, d, key, depth, W.rr_depth, beta, L, nd, rrs);
				}
				if (cont && depth + 1 >= W.max_depth) cont = false;
				p = sf.p;
			}
			term = !cont;
		}
		// a finished path: its recorded guided vertices become training samples
		// (incident radiance L_in = (L_final - L_before) / beta_after along the
		// sampled direction, weight lum(L_in) cos / pdf) ...
		const int slot = __float_as_int(ra.w);
		// vertices recorded by any finished path of the warp (warp-uniform)
		const unsigned wmask = __reduce_or_sync(0xffffffffu, term ? vmask : 0u);
		for (int v = 0; v < GV; ++v) {
			if (!((wmask >> v) & 1u)) continue;
			bool emit = false;
			float4 o0, o1, o2, o3;
			if (term && ((vmask >> v) & 1u)) {
				const float4 *r = G.vrec + ((size_t)slot * GV + v) * 6;
				const float4 r0 = r[0], r1 = r[1], r2 = r[2], r3 = r[3], r4 = r[4], r5 = r[5];
				const float li[3] = { r4.x > 0.f ? (L.x - r5.x) / r4.x : 0.f, r4.y > 0.f ? (L.y - r5.y) / r4.y : 0.f,
					r4.z > 0.f ? (L.z - r5.z) / r4.z : 0.f };
				const float lum = 0.2126f * li[0] + 0.7152f * li[1] + 0.0722f * li[2];
				const float wt = lum * r3.y / r3.x;
				if (wt > 0.f && isfinite(wt)) {
					o0 = r0, o1 = r1, o2 = r2, o3 = make_float4(wt, 0.f, 0.f, 0.f);
					emit = true;
				}
			}
			const unsigned tpos = warp_append(G.tcount, emit);
			const unsigned m = __ballot_sync(0xffffffffu, emit);
			if (lane_id() == 0 && m) atomicAdd(&W.stat[2], (unsigned long long)__popc(m));
			if (emit && tpos < G.tcap) {
				float4 *o = reinterpret_cast<float4 *>(G.tbuf + (size_t)tpos * 16);
				o[0] = o0, o[1] = o1, o[2] = o2, o[3] = o3;
			}
		}
		// ... then the accumulate step and the slot's next camera path (as the plain shading kernel)
		bool spawn = false;
		PathState C;
		if (term) {
			++done;
			int64_t item = (int64_t)(unsigned)__float_as_int(rc.w);
			int j = __float_as_int(rb.w) >> 8;
			spawn = finish_path(W, slot, L, item, j, err, &W.cnt[3]);
			if (spawn) camera_path(W, slot, item, j, C);
		}
		const unsigned pos = warp_append(&W.cnt[out], cont || spawn);
		if (cont || spawn) {
			if (pos >= (unsigned)W.P) {
				err |= ERR_QUEUE_OVERFLOW;
			} else if (cont) {
				W.qa[out][pos] = make_float4(p.x, p.y, p.z, ra.w);
				W.qb[out][pos] = make_float4(nd.x, nd.y, nd.z, __int_as_float(__float_as_int(rb.w) + 1));
				W.qc[out][pos] = make_float4(beta.x, beta.y, beta.z, rc.w);
				W.qd[out][pos] = make_float4(L.x, L.y, L.z, __uint_as_float((__float_as_uint(rrs) & ~0xfu) | vmask));
			} else {
				store_path(W, out, pos, C);  // qd.w = 0: no recorded vertex, roulette scale 1
			}
		}
	}
	for (int o = 16; o > 0; o >>= 1) done += __shfl_down_sync(0xffffffffu, done, o);
	if (lane_id() == 0 && done) atomicAdd(&W.stat[1], done);
	if (err) atomicOr(&W.cnt[4], err);
}

namespace {
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
int grid_of(const void *k, int n_sms, size_t smem = 0) {
	int per = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, BLOCK, smem);
	return std::max(1, per) * n_sms;
}
}  // namespace

are_status render_guided(are_scene *sc, GuideNet *net, const are_camera *cam, const are_render_params *prm,
	const are_guide_params *gp, float *rgb, float *var, are_render_stats *stats) {
	if (!sc || !net || !cam || !prm || !gp || !rgb) return bad("null scene, guide, camera, params or output");
	const are_render_params &p = *prm;
	if (p.width <= 0 || p.height <= 0 || p.spp <= 0 || p.max_depth <= 0 || p.max_depth > 255)
		return bad("width, height, spp must be > 0 and max_depth in [1, 255]");
	if (!(gp->mix >= 0.f && gp->mix <= 1.f)) return bad("mix must be in [0, 1]");
	if (gp->guide_depth < 0 || gp->guide_depth > 255) return bad("guide_depth must be in [0, 255]");
	if (p.schedule == ARE_SCHEDULE_WAVEFRONT && gp->guide_depth > GV)
		return bad("guide_depth must be in [0, 4] on the wavefront schedule");
	if (gp->train < 0 || gp->train > 16) return bad("train must be in [0, 16]");
	if (gp->train && (gp->batch < 256 || gp->batch > (1 << 20) || !(gp->lr > 0.f))) return bad("bad training batch or lr");
	if (!(cam->vfov_deg > 0.0f && cam->vfov_deg < 180.0f)) return bad("vfov must be in (0, 180)");
	if (net->device != sc->device) return bad("guide and scene live on different devices");
	if (!(p.t_min >= 0.0f) || !std::isfinite(p.t_min)) return bad("t_min must be finite and >= 0");
	if (p.schedule < ARE_SCHEDULE_AUTO || p.schedule > ARE_SCHEDULE_MEGAKERNEL) return bad("unknown schedule");
	if (gp->cache_res < 0 || gp->cache_res > 128) return bad("cache_res must be in [0, 128]");
	if (gp->max_steps < 0) return bad("max_steps must be >= 0");
	cudaSetDevice(sc->device);
	if (p.schedule != ARE_SCHEDULE_WAVEFRONT) return render_guided_mega(sc, net, cam, p, gp, rgb, var, stats);

	Wave W{};
	W.npix = p.width * p.height;
	W.spp = p.spp;
	int64_t total = (int64_t)W.npix * p.spp;
	int P = p.pool_size > 0 ? p.pool_size : (1 << 20);
	int chunk = p.chunk > 0 ? p.chunk : (int)std::min<int64_t>(16, std::max<int64_t>(1, total / (16 * (int64_t)P)));
	chunk = std::min(chunk, p.spp);
	W.chunk = chunk;
	W.nchunk = (p.spp + chunk - 1) / chunk;
	W.n_items = (int64_t)W.npix * W.nchunk;
	if (W.n_items >= (int64_t)UINT32_MAX - (int64_t)P) return bad("too many work items; raise chunk");
	P = (int)std::min<int64_t>(P, W.n_items);
	P = (P + 31) & ~31;
	W.P = P;
	W.max_depth = p.max_depth;
	W.rr_depth = p.rr_depth;
	W.t_min = p.t_min;
	W.seed = p.seed;
	camera_frame(*cam, p.width, p.height, p.flags, W.cam);

	GuidedState G{};
	G.mix = gp->mix;
	G.guide_depth = gp->guide_depth;
	const unsigned tcap = (unsigned)std::max(gp->batch, 256);
	G.tcap = tcap;
	for (int k = 0; k < 3; ++k) {
		float lo = sc->box_lo[k], ext = sc->box_hi[k] - sc->box_lo[k];
		G.box.lo[k] = lo;
		G.box.inv_ext[k] = ext > 0.f ? 1.f / ext : 0.f;
	}
	// one allocation for the wavefront, guiding state and item sums (freed at the end)
	size_t need = 0;
	char *z = nullptr;
	for (int q = 0; q < 2; ++q) carve<float4>(z, P), carve<float4>(z, P), carve<float4>(z, P), carve<float4>(z, P);
	carve<float4>(z, P), carve<float4>(z, P), carve<float4>(z, P), carve<float4>(z, P);  // hit, accumulators
	carve<unsigned>(z, 64), carve<unsigned long long>(z, 8);
	carve<int32_t>(z, P), carve<float>(z, (size_t)P * GN_IN), carve<float>(z, (size_t)P * GN_OUT);
	carve<float4>(z, (size_t)P * GV * 6), carve<float>(z, (size_t)tcap * 16);
	carve<float4>(z, W.n_items), carve<float4>(z, W.n_items), carve<float>(z, 3 * (size_t)W.npix),
		carve<float>(z, 3 * (size_t)W.npix);
	need = (size_t)z;
	void *mem = nullptr;
	if (are_status st = pool_alloc(sc, need, &mem)) return st;
	z = (char *)mem;
	for (int q = 0; q < 2; ++q)
		W.qa[q] = carve<float4>(z, P), W.qb[q] = carve<float4>(z, P), W.qc[q] = carve<float4>(z, P),
		W.qd[q] = carve<float4>(z, P);
	W.hit = carve<float4>(z, P);
	W.acc_s = carve<float4>(z, P), W.acc_c = carve<float4>(z, P), W.acc_q = carve<float4>(z, P);
	W.cnt = carve<unsigned>(z, 64);
	W.stat = carve<unsigned long long>(z, 8);
	G.gidx = carve<int32_t>(z, P);
	G.gfeat = carve<float>(z, (size_t)P * GN_IN);
	G.gout = carve<float>(z, (size_t)P * GN_OUT);
	G.vrec = carve<float4>(z, (size_t)P * GV * 6);
	G.tbuf = carve<float>(z, (size_t)tcap * 16);
	W.item_s = carve<float4>(z, W.n_items);
	W.item_q = carve<float4>(z, W.n_items);
	float *d_rgb = carve<float>(z, 3 * (size_t)W.npix);
	float *d_var = carve<float>(z, 3 * (size_t)W.npix);
	G.tcount = W.cnt + 7;

	cudaStream_t s = sc->stream;
	const bool dev_out = (p.flags & ARE_FLAG_DEVICE_OUTPUT) != 0;
	cudaEvent_t ev0, ev1;
	cudaEventCreate(&ev0);
	cudaEventCreate(&ev1);
	// per graph iteration: before intersect, after intersect, after inference, after shade;
	// then two around each batch of training steps
	cudaEvent_t kev[4 * GUIDED_ITERS + 2];
	for (auto &e : kev) cudaEventCreate(&e);
	double kms[4] = { 0.0, 0.0, 0.0, 0.0 };
	cudaGraph_t graph = nullptr;
	cudaGraphExec_t exec = nullptr;
	int64_t iterations = 0, train_steps = 0;
	int64_t launches[4] = { 0, 0, 0, 0 };
	unsigned init[8] = { (unsigned)std::min<int64_t>(P, W.n_items), 0u, 0u, (unsigned)std::min<int64_t>(P, W.n_items),
		0u, 0u, 0u, 0u };
	cudaGetLastError();
	cudaEventRecord(ev0, s);
	are_status st = cuda_status(cudaMemcpyAsync(W.cnt, init, sizeof init, cudaMemcpyHostToDevice, s), "counters");
	if (!st) st = cuda_status(cudaMemsetAsync(W.stat, 0, 64, s), "stats");
	if (!st) {
		k_init<<<grid_of((const void *)k_init, sc->n_sms), BLOCK, 0, s>>>(W, (int)init[0]);
		++launches[ARE_KERNEL_OTHER];
		st = cuda_status(cudaGetLastError(), "k_init");
	}
	const bool linear = sc->linear;
	const void *isect_fn = linear ? (const void *)k_intersect_select<true> : (const void *)k_intersect_select<false>;
	const int g_int = grid_of(isect_fn, sc->n_sms);
	const int g_sh = grid_of((const void *)k_shade_guided, sc->n_sms);
	const DevScene S = sc->dev;
	// the network runs on the compact list, its length read on the device
	if (!st) st = cuda_status(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "capture");
	if (!st) {
		for (int it = 0; it < GUIDED_ITERS; ++it) {
			int par = it & 1;
			cudaMemsetAsync(W.cnt + 6, 0, 4, s);
			cudaEventRecordWithFlags(kev[4 * it + 0], s, cudaEventRecordExternal);
			if (linear)
				k_intersect_select<true><<<g_int, BLOCK, 0, s>>>(S, W, G, par);
			else
				k_intersect_select<false><<<g_int, BLOCK, 0, s>>>(S, W, G, par);
			cudaEventRecordWithFlags(kev[4 * it + 1], s, cudaEventRecordExternal);
			net->infer(G.gfeat, P, G.gout, s, W.cnt + 6, W.cnt + 4, true);
			cudaEventRecordWithFlags(kev[4 * it + 2], s, cudaEventRecordExternal);
			k_shade_guided<<<g_sh, BLOCK, 0, s>>>(S, W, G, par);
			cudaEventRecordWithFlags(kev[4 * it + 3], s, cudaEventRecordExternal);
		}
		st = cuda_status(cudaStreamEndCapture(s, &graph), "capture end");
	}
	if (!st) st = cuda_status(cudaGraphInstantiate(&exec, graph, 0), "instantiate");
	const int64_t max_launches = (int64_t)(W.n_items / std::max(1, P) + 2) * (int64_t)p.max_depth * W.chunk + 16;
	unsigned *hc = sc->host_counters;
	bool pending_loss = false, pending_train = false;
	unsigned pending_n = 1;
	// a step needs a quarter batch: fewer samples make a noisy gradient
	const unsigned tmin = std::max(256u, tcap / 4);
	for (int64_t g = 0; !st; ++g) {
		st = cuda_status(cudaGraphLaunch(exec, s), "graph launch");
		if (st) break;
		cudaMemcpyAsync(hc, W.cnt, 8 * sizeof(unsigned), cudaMemcpyDeviceToHost, s);
		st = cuda_status(cudaStreamSynchronize(s), "guided iteration");
		if (st) break;
		iterations += GUIDED_ITERS;
		launches[ARE_KERNEL_INTERSECT] += GUIDED_ITERS;
		launches[ARE_KERNEL_GENERATE] += GUIDED_ITERS;  // inference
		launches[ARE_KERNEL_SHADE] += GUIDED_ITERS;     // shade (+ training samples, accumulate, next camera ray)
		for (int it = 0; it < GUIDED_ITERS; ++it) {
			static const int kind[3] = { ARE_KERNEL_INTERSECT, ARE_KERNEL_GENERATE, ARE_KERNEL_SHADE };
			for (int k = 0; k < 3; ++k) {
				float ms = 0.f;
				if (cudaEventElapsedTime(&ms, kev[4 * it + k], kev[4 * it + k + 1]) == cudaSuccess) kms[kind[k]] += ms;
			}
		}
		if (pending_train) {
			float ms = 0.f;
			if (cudaEventElapsedTime(&ms, kev[4 * GUIDED_ITERS], kev[4 * GUIDED_ITERS + 1]) == cudaSuccess)
				kms[ARE_KERNEL_OTHER] += ms;
			pending_train = false;
		}
		const unsigned have = std::min(hc[7], tcap);
		if (pending_loss) {
			// the loss of the step enqueued after the previous launch is complete now
			net->loss_log.push_back(*reinterpret_cast<float *>(&hc[16]) / (float)pending_n);
			pending_loss = false;
		}
		if (gp->train && have >= tmin) {
			// `train` Adam steps on what was collected (up to one batch), then collect again
			net->weight_clip = gp->weight_clip > 0.f ? gp->weight_clip : 1e30f;
			cudaEventRecord(kev[4 * GUIDED_ITERS], s);
			for (int k = 0; k < gp->train && !st; ++k) {
				st = net->train_step(G.tbuf, (int)have, -1.0f, gp->lr, s, W.cnt + 4);
				++train_steps;
				launches[ARE_KERNEL_OTHER] += 7;
			}
			cudaEventRecord(kev[4 * GUIDED_ITERS + 1], s);
			pending_train = true;  // timed once the next launch's read-back has synchronised
			cudaMemcpyAsync(hc + 16, net->grad + GN_PARAMS, 4, cudaMemcpyDeviceToHost, s);
			pending_loss = true;
			pending_n = have;
			cudaMemsetAsync(G.tcount, 0, 4, s);
		}
		if (hc[0] == 0) break;
		if (g > max_launches) {
			set_error("render did not converge");
			st = ARE_ERR_INTERNAL;
		}
	}
	if (!st) {
		k_resolve<<<std::max(1, std::min(4096, (W.npix + BLOCK - 1) / BLOCK)), BLOCK, 0, s>>>(
			W, dev_out ? rgb : d_rgb, var ? (dev_out ? var : d_var) : nullptr, (p.flags & ARE_FLAG_CLAMP_OUTPUT) != 0);
		++launches[ARE_KERNEL_OTHER];
		st = cuda_status(cudaGetLastError(), "k_resolve");
	}
	cudaEventRecord(ev1, s);
	unsigned long long hstat[4] = { 0, 0, 0, 0 };
	unsigned herr = 0;
	if (!st) {
		cudaMemcpyAsync(hstat, W.stat, sizeof hstat, cudaMemcpyDeviceToHost, s);
		cudaMemcpyAsync(&herr, W.cnt + 4, sizeof herr, cudaMemcpyDeviceToHost, s);
		if (!dev_out) {
			cudaMemcpyAsync(rgb, d_rgb, 3 * sizeof(float) * W.npix, cudaMemcpyDeviceToHost, s);
			if (var) cudaMemcpyAsync(var, d_var, 3 * sizeof(float) * W.npix, cudaMemcpyDeviceToHost, s);
		}
		st = cuda_status(cudaStreamSynchronize(s), "guided render");
	}
	if (!st && pending_loss) net->loss_log.push_back(*reinterpret_cast<float *>(&hc[16]) / (float)pending_n);
	float ms = 0.f;
	cudaEventElapsedTime(&ms, ev0, ev1);
	if (exec) cudaGraphExecDestroy(exec);
	if (graph) cudaGraphDestroy(graph);
	cudaEventDestroy(ev0);
	cudaEventDestroy(ev1);
	if (!st && pending_train) {
		float tms = 0.f;
		if (cudaEventElapsedTime(&tms, kev[4 * GUIDED_ITERS], kev[4 * GUIDED_ITERS + 1]) == cudaSuccess)
			kms[ARE_KERNEL_OTHER] += tms;
	}
	for (auto &e : kev) cudaEventDestroy(e);
	cudaStreamSynchronize(s);
	pool_free(sc, mem);
	if (!st && herr) {
		set_error("device error word " + std::to_string(herr));
		st = ARE_ERR_INTERNAL;
	}
	if (stats) {
		*stats = are_render_stats{};
		stats->samples = (int64_t)hstat[1];
		stats->segments = (int64_t)hstat[0];
		stats->iterations = iterations;
		stats->device_ms = ms;
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
