// rt_dropin.cpp — the drop-in binding of INTEGRATION.md, compiled (TEST
// INFRASTRUCTURE, built by tests/test_dropin.py where the reference tree is
// present).
//
// experiments/rt.cpp is #included from the reference tree unchanged, with its
// own render() (rt.cpp:337-374) renamed so that the render() body shown in
// written by the test into the file RT_DROPIN_RENDER names —
// takes its place; main (rt.cpp:395-403) is renamed too and restated below
// with the image size and the output file from the command line.  Linked
// against libaurora_gb300.so it is the reference's program rendering through
// the GPU core; linked against tests/harness/abi_recorder.cpp it records the
// scene descriptor, camera and parameters the binding hands to the C ABI.
#include <cstdlib>
#include <iostream>
#include <map>
#include <random>
#include <vector>

#include "aurora_gb300.h"

#define render rt_reference_render
#define main rt_reference_main
#include "experiments/rt.cpp"
#undef main
#undef render

#include RT_DROPIN_RENDER

int main(int argc, char **argv) {
	const char *out = argc > 1 ? argv[1] : "out_dropin.ppm";
	const int w = argc > 2 ? std::atoi(argv[2]) : 512, h = argc > 3 ? std::atoi(argv[3]) : 512;
	Scene scene;
	Viewport vp(w, h);
	render(scene, Vec3(0, 0, 4), Vec3(0, 0, 0), Vec3(0, 1, 0), 50.f, vp);
	writePPM(vp, out);
	return 0;
}
