// are_render — command-line renderer over the C++ host layer: one of the
// built-in workloads (or rt.cpp's own scene) -> PPM (rt.cpp writePPM's
// quantisation) and optionally the linear FP32 image as PFM.
//
//   are_render [--config cornell|spheres|mesh|occluded|legacy] [--width W]
//              [--height H] [--spp S] [--depth D] [--seed N] [--gamma G]
//              [--out image.ppm] [--pfm image.pfm]
//
// Prints one line: samples, device milliseconds and Msamples/s.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "aurora_gb300.hpp"

namespace {

int config_id(const std::string &name) {
	if (name == "spheres") return ARE_CONFIG_RANDOM_SPHERES;
	if (name == "cornell") return ARE_CONFIG_CORNELL;
	if (name == "mesh") return ARE_CONFIG_MESH;
	if (name == "occluded") return ARE_CONFIG_CORNELL_OCCLUDED;
	if (name == "legacy") return ARE_CONFIG_LEGACY_RT;
	return -1;
}

int usage() {
	std::fprintf(stderr,
		"usage: are_render [--config cornell|spheres|mesh|occluded|legacy] [--width W] [--height H] [--spp S]\n"
		"                  [--depth D] [--seed N] [--gamma G] [--out image.ppm] [--pfm image.pfm]\n");
	return 2;
}

}  // namespace

int main(int argc, char **argv) {
	std::string config = "cornell", out = "out.ppm", pfm;
	int width = 0, height = 0, spp = 0, depth = 0;
	long long seed = -1;
	float gamma = 2.2f;
	for (int i = 1; i < argc; ++i) {
		std::string a = argv[i];
		if (i + 1 >= argc) return usage();
		const char *v = argv[++i];
		if (a == "--config") config = v;
		else if (a == "--width") width = std::atoi(v);
		else if (a == "--height") height = std::atoi(v);
		else if (a == "--spp") spp = std::atoi(v);
		else if (a == "--depth") depth = std::atoi(v);
		else if (a == "--seed") seed = std::atoll(v);
		else if (a == "--gamma") gamma = (float)std::atof(v);
		else if (a == "--out") out = v;
		else if (a == "--pfm") pfm = v;
		else return usage();
	}
	const int id = config_id(config);
	if (id < 0) return usage();
	try {
		are_config *cfg = nullptr;
		are_gb300::check(are_config_build(id, 42, 0, &cfg));
		are_camera cam{};
		are_render_params par{};
		are_gb300::check(are_config_defaults(cfg, &cam, &par));
		are_gb300::Scene scene(*are_config_desc(cfg));
		are_config_free(cfg);
		if (width > 0) par.width = width;
		if (height > 0) par.height = height;
		if (spp > 0) par.spp = spp;
		if (depth > 0) par.max_depth = depth;
		if (seed >= 0) par.seed = (uint64_t)seed;
		are_render_stats st{};
		are_gb300::Image im = are_gb300::render(scene, cam, par, &st);
		are_gb300::write_ppm(out, im, ARE_TONEMAP_GAMMA, gamma);
		if (!pfm.empty()) are_gb300::write_pfm(pfm, im);
		std::printf("%s %dx%d %d spp: %lld samples in %.3f ms (%.1f Msamples/s) -> %s\n", config.c_str(), im.width,
			im.height, par.spp, (long long)st.samples, st.device_ms,
			st.device_ms > 0 ? (double)st.samples / (st.device_ms * 1e3) : 0.0, out.c_str());
	} catch (const are_gb300::Error &e) {
		std::fprintf(stderr, "are_render: %s\n", e.what());
		return 1;
	}
	return 0;
}
