// guide_host.h — host-side owner of a path-guiding network (the opaque
// are_guide of the C ABI): FP32 master parameters, Adam moments, the FP16
// weight images the kernels load, and the training buffers.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "aurora_gb300.h"

namespace are_core {

// per-sample tensors of one training batch, FP16 [samples][features]
struct GuideTrainBufs {
	__half *h0;     // encoded inputs [cap][256]
	__half *h[4];   // hidden outputs h1..h4 [cap][64]
	__half *d[4];   // gradients at h1..h4 pre-activations [cap][64]
	__half *d5;     // output gradients [cap][48]
};

struct GuideNet {
	int device = 0, n_sms = 0;
	cudaStream_t stream = nullptr;
	bool own_stream = false;
	float *params = nullptr, *adam_m = nullptr, *adam_v = nullptr;
	float *grad = nullptr;  // GN_PARAMS gradients, then loss sum, then an overflow flag
	__half *tc_img = nullptr;  // FP16 weights of the tensor-core kernels (core-matrix layout): forward, then backward
	unsigned *err_word = nullptr;  // device error bits of inference outside a render
	void *train_mem = nullptr;
	int train_cap = 0;
	GuideTrainBufs bufs{};
	std::vector<void *> allocs;
	int64_t steps = 0;
	float loss_scale = 8.0f;     // gradients are carried in FP16 times this factor
	float weight_clip = 1e30f;   // cap on a sample's normalised weight
	uint32_t first_wait_limit = 0xffffffffu;  // polls of each warpgroup's first MMA wait in inference and training (capped)
	std::vector<float> loss_log; // losses of Adam steps taken inside renders

	~GuideNet();
	are_status init(uint64_t seed);
	are_status set_params(const float *host);
	are_status pack();
	are_status ensure_train(int n);
	// n_dev: optional device row count (rows = min(n, *n_dev)), read when the kernel runs
	// d_err: device error word to OR failures into (default: err_word)
	// mixture_out: write the packed vMF mixture (pack_mixture_fast) instead of the raw outputs
	are_status infer(const float *d_feat, int n, float *d_out, cudaStream_t s, const unsigned *n_dev = nullptr,
		unsigned *d_err = nullptr, bool mixture_out = false);
	// wmean < 0: normalise the weights by their batch mean computed on the device
	// d_err: device error word to OR failures into (default: err_word); a failed step is not applied
	are_status gradient(const float *d_samples, int n, float wmean, cudaStream_t s, unsigned *d_err = nullptr);
	are_status train_step(const float *d_samples, int n, float wmean, float lr, cudaStream_t s, unsigned *d_err = nullptr);
};

size_t guide_infer_smem();

are_status render_guided(struct ::are_scene *sc, GuideNet *net, const are_camera *cam, const are_render_params *prm,
	const are_guide_params *gp, float *rgb, float *var, are_render_stats *stats);
// the megakernel schedule of render_guided (guided_mega.cu), parameters validated by render_guided
are_status render_guided_mega(struct ::are_scene *sc, GuideNet *net, const are_camera *cam, const are_render_params &p,
	const are_guide_params *gp, float *rgb, float *var, are_render_stats *stats);

}  // namespace are_core
