// output.cu — the step after accumulation: FP32 RGB -> 8-bit RGB on the GPU,
// and the image files the reference writes and reads.
//
//   are_tonemap    8-bit quantisation of a linear FP32 image, byte-identical
//                  to the reference's writers:
//                    ARE_TONEMAP_GAMMA   experiments/rt.cpp:377-392 writePPM:
//                                        clamp to [0,1], powf(c, 1/gamma) * 255
//                                        in FP32, truncated (gamma 2.2 there)
//                    ARE_TONEMAP_LINEAR  src/texture.cpp:362-395 save_texture:
//                                        clamp(c * 255.0, 0, 255) in FP64, truncated
//   are_write_ppm  P6 file, header "P6\n<w> <h>\n255\n" as both writers
//   are_write_pfm  FP32 RGB Portable Float Map (little-endian, bottom row first)
//   are_read_ppm   P6 reader of src/texture.cpp:9-50 (texel = byte / 255.0)
//
// The quantiser on the device does not evaluate pow: both modes are monotone
// maps from a float to a byte, so the host finds, for every byte q, the
// smallest float whose byte is >= q (bisection over the ordered bit patterns
// of [0, 1], evaluating the reference's own formula in the reference's own
// precision), and the kernel counts the thresholds at or below each value
// (binary search in shared memory).  The bytes therefore equal the reference
// formula's bytes on this host for every input, including the values right
// at a step.  The kernel is a streaming pass: 12 bytes read and 3 written
// per pixel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "aurora_gb300.h"
#include "scene.h"

namespace are_core {

namespace {

constexpr int TM_BLOCK = 256;

// thr[q] for q = 1..255 (thr[0] unused); a value v maps to #{q : v >= thr[q]}
__global__ void __launch_bounds__(TM_BLOCK) k_tonemap(const float *__restrict__ in, int64_t n, const float *__restrict__ thr,
	float nan_value, uint8_t *__restrict__ out) {
	__shared__ float s_thr[256];
	s_thr[threadIdx.x] = threadIdx.x == 0 ? -INFINITY : thr[threadIdx.x];
	__syncthreads();
	auto q8 = [&](float v) -> uint32_t {
		if (v != v) v = nan_value;
		// largest q with s_thr[q] <= v (s_thr is non-decreasing, s_thr[0] = -inf)
		uint32_t q = 0;
#pragma unroll
		for (uint32_t step = 128; step; step >>= 1)
			if (s_thr[q + step] <= v) q += step;
		return q;
	};
	const bool vec = ((reinterpret_cast<uintptr_t>(in) & 15) == 0) && ((reinterpret_cast<uintptr_t>(out) & 3) == 0);
	const int64_t stride = (int64_t)gridDim.x * blockDim.x;
	const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (vec) {
		const int64_t n4 = n >> 2;
		const float4 *in4 = reinterpret_cast<const float4 *>(in);
		uint32_t *out4 = reinterpret_cast<uint32_t *>(out);
		for (int64_t i = t0; i < n4; i += stride) {
			float4 v = in4[i];
			out4[i] = q8(v.x) | (q8(v.y) << 8) | (q8(v.z) << 16) | (q8(v.w) << 24);
		}
		for (int64_t i = (n4 << 2) + t0; i < n; i += stride) out[i] = (uint8_t)q8(in[i]);
	} else {
		for (int64_t i = t0; i < n; i += stride) out[i] = (uint8_t)q8(in[i]);
	}
}

// the reference formulas, evaluated on the host in the reference's precision
uint8_t byte_gamma(float c, float inv_gamma) {
	c = std::fmax(0.0f, std::fmin(1.0f, c));  // rt.cpp:72-76 Color::clamp
	return (uint8_t)(std::pow(c, inv_gamma) * 255);
}
uint8_t byte_linear(float c) {
	double v = (double)c * 255.0;  // texture.cpp:381, image stored as FP64
	v = v < 0.0 ? 0.0 : (v > 255.0 ? 255.0 : v);
	return (uint8_t)v;
}

float from_bits(uint32_t b) {
	float f;
	std::memcpy(&f, &b, 4);
	return f;
}

// thresholds of a monotone float -> byte map on [0, 1]; false if the map is
// not monotone around a threshold
template <class F>
bool thresholds(F byte_of, float *thr) {
	const uint32_t one = 0x3f800000u;
	if (byte_of(0.0f) != 0 || byte_of(1.0f) != 255) return false;
	for (int q = 1; q < 256; ++q) {
		uint32_t lo = 0, hi = one;  // byte_of(lo) < q <= byte_of(hi)
		while (hi - lo > 1) {
			uint32_t mid = lo + (hi - lo) / 2;
			if (byte_of(from_bits(mid)) >= q)
				hi = mid;
			else
				lo = mid;
		}
		thr[q] = from_bits(hi);
		// the map must be monotone near the step for a threshold to describe it
		for (uint32_t d = 1; d <= 64; ++d) {
			if (hi >= d && byte_of(from_bits(hi - d)) >= q) return false;
			if (hi + d <= one && byte_of(from_bits(hi + d)) < q) return false;
		}
	}
	thr[0] = -INFINITY;
	for (int q = 2; q < 256; ++q)
		if (thr[q] < thr[q - 1]) return false;
	return true;
}

struct TableKey {
	int mode;
	float gamma;
	int device;
};

struct Table {
	TableKey key;
	float *d_thr;
};

std::mutex g_tables_mu;
std::vector<Table> g_tables;

// device copy of the threshold table of (mode, gamma) on the current device, built once
are_status table_for(int mode, float gamma, const float **out) {
	int device = 0;
	if (are_status st = cuda_status(cudaGetDevice(&device), "cudaGetDevice")) return st;
	std::lock_guard<std::mutex> lock(g_tables_mu);
	for (const Table &t : g_tables)
		if (t.key.mode == mode && t.key.device == device && (mode != ARE_TONEMAP_GAMMA || t.key.gamma == gamma)) {
			*out = t.d_thr;
			return ARE_OK;
		}
	float thr[256];
	bool ok;
	if (mode == ARE_TONEMAP_GAMMA) {
		const float inv = 1 / gamma;  // rt.cpp:384 writes 1 / 2.2f
		ok = thresholds([inv](float c) { return byte_gamma(c, inv); }, thr);
	} else {
		ok = thresholds(byte_linear, thr);
	}
	if (!ok) {
		set_error("tonemap: the quantiser is not monotone for these parameters");
		return ARE_ERR_INVALID_ARGUMENT;
	}
	float *d = nullptr;
	if (are_status st = cuda_status(cudaMalloc(&d, sizeof thr), "cudaMalloc(tonemap table)")) return st;
	if (are_status st = cuda_status(cudaMemcpy(d, thr, sizeof thr, cudaMemcpyHostToDevice), "tonemap table")) {
		cudaFree(d);
		return st;
	}
	g_tables.push_back(Table{ TableKey{ mode, gamma, device }, d });
	*out = d;
	return ARE_OK;
}

are_status bad(const std::string &m) {
	set_error(m);
	return ARE_ERR_INVALID_ARGUMENT;
}

are_status io_error(const std::string &m) {
	set_error(m);
	return ARE_ERR_IO;
}

}  // namespace

are_status tonemap(const float *rgb, int64_t n, const are_tonemap_params *p, uint8_t *out) {
	if (!p) return bad("null tonemap params");
	if (p->mode != ARE_TONEMAP_GAMMA && p->mode != ARE_TONEMAP_LINEAR) return bad("unknown tonemap mode");
	if (p->mode == ARE_TONEMAP_GAMMA && !(p->gamma >= 0.1f && p->gamma <= 10.0f)) return bad("gamma must be in [0.1, 10]");
	if (n < 0) return bad("negative value count");
	if (n == 0) return ARE_OK;
	if (!rgb || !out) return bad("null image or output");
	const float *thr = nullptr;
	if (are_status st = table_for(p->mode, p->gamma, &thr)) return st;
	int device = 0, n_sms = 1;
	cudaGetDevice(&device);
	cudaDeviceGetAttribute(&n_sms, cudaDevAttrMultiProcessorCount, device);
	const float nan_value = p->mode == ARE_TONEMAP_GAMMA ? 1.0f : 0.0f;  // fmin(1, NaN) = 1 in rt.cpp's clamp
	const int64_t blocks_needed = (n / 4 + TM_BLOCK - 1) / TM_BLOCK + 1;
	const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)n_sms * 8, blocks_needed));
	cudaStream_t s = cudaStreamPerThread;
	cudaGetLastError();
	if (p->flags & ARE_FLAG_DEVICE_OUTPUT) {
		k_tonemap<<<grid, TM_BLOCK, 0, s>>>(rgb, n, thr, nan_value, out);
		if (are_status st = cuda_status(cudaGetLastError(), "k_tonemap")) return st;
		return cuda_status(cudaStreamSynchronize(s), "tonemap");
	}
	// host image: staged through one device buffer (values, then bytes)
	void *mem = nullptr;
	const size_t in_bytes = ((size_t)n * 4 + 255) & ~(size_t)255;
	if (are_status st = cuda_status(cudaMalloc(&mem, in_bytes + (size_t)n), "cudaMalloc(tonemap)")) return st;
	float *d_in = (float *)mem;
	uint8_t *d_out = (uint8_t *)mem + in_bytes;
	are_status st = cuda_status(cudaMemcpyAsync(d_in, rgb, (size_t)n * 4, cudaMemcpyHostToDevice, s), "tonemap upload");
	if (!st) {
		k_tonemap<<<grid, TM_BLOCK, 0, s>>>(d_in, n, thr, nan_value, d_out);
		st = cuda_status(cudaGetLastError(), "k_tonemap");
	}
	if (!st) st = cuda_status(cudaMemcpyAsync(out, d_out, (size_t)n, cudaMemcpyDeviceToHost, s), "tonemap download");
	if (!st) st = cuda_status(cudaStreamSynchronize(s), "tonemap");
	cudaStreamSynchronize(s);
	cudaFree(mem);
	return st;
}

are_status write_ppm(const char *path, const uint8_t *rgb8, int w, int h) {
	if (!path || !rgb8 || w <= 0 || h <= 0) return bad("bad PPM arguments");
	FILE *f = std::fopen(path, "wb");
	if (!f) return io_error(std::string("cannot open ") + path);
	bool ok = std::fprintf(f, "P6\n%d %d\n255\n", w, h) > 0;
	ok = ok && std::fwrite(rgb8, 1, (size_t)w * h * 3, f) == (size_t)w * h * 3;
	ok = (std::fclose(f) == 0) && ok;
	return ok ? ARE_OK : io_error(std::string("cannot write ") + path);
}

are_status write_pfm(const char *path, const float *rgb, int w, int h) {
	if (!path || !rgb || w <= 0 || h <= 0) return bad("bad PFM arguments");
	FILE *f = std::fopen(path, "wb");
	if (!f) return io_error(std::string("cannot open ") + path);
	const uint32_t probe = 1;
	uint8_t first;
	std::memcpy(&first, &probe, 1);
	const bool little = first == 1;  // the scale's sign gives the byte order
	bool ok = std::fprintf(f, "PF\n%d %d\n%s\n", w, h, little ? "-1.0" : "1.0") > 0;
	for (int y = h - 1; ok && y >= 0; --y)  // PFM stores the bottom row first
		ok = std::fwrite(rgb + (size_t)y * w * 3, sizeof(float), (size_t)w * 3, f) == (size_t)w * 3;
	ok = (std::fclose(f) == 0) && ok;
	return ok ? ARE_OK : io_error(std::string("cannot write ") + path);
}

are_status read_ppm(const char *path, int *w_out, int *h_out, float *texels) {
	if (!path || !w_out || !h_out) return bad("bad PPM arguments");
	FILE *f = std::fopen(path, "rb");
	if (!f) return io_error(std::string("cannot open ") + path);
	struct Close {
		FILE *f;
		~Close() { std::fclose(f); }
	} close_guard{ f };
	// texture.cpp:18-29: "P6", then width, height and a maximum of 255, then one whitespace byte
	char format[3] = { 0, 0, 0 };
	if (std::fscanf(f, "%2s", format) != 1 || std::strcmp(format, "P6") != 0)
		return bad(std::string("unsupported PPM format in ") + path);
	int w = 0, h = 0, maxval = 0;
	if (std::fscanf(f, "%d %d %d", &w, &h, &maxval) != 3 || maxval != 255 || w <= 0 || h <= 0 ||
		(int64_t)w * h > (int64_t)1 << 28)
		return bad(std::string("invalid PPM header in ") + path);
	std::fgetc(f);
	*w_out = w, *h_out = h;
	if (!texels) return ARE_OK;  // size query
	std::vector<uint8_t> px((size_t)w * h * 3);
	if (std::fread(px.data(), 1, px.size(), f) != px.size())
		return io_error(std::string("unexpected end of pixel data in ") + path);
	for (size_t i = 0; i < px.size(); ++i) texels[i] = (float)((double)px[i] / 255.0);  // texture.cpp:41-43
	return ARE_OK;
}

}  // namespace are_core
