// abi_recorder.cpp — a recording stand-in for four entry points of the C ABI
// (TEST INFRASTRUCTURE, linked into tests/harness/rt_dropin.cpp by
// tests/test_dropin.py): it writes what a caller hands to are_scene_create and
// are_render to the file named by ARE_RECORD_PATH, so a test can compare the
// descriptor a binding builds with the one the GPU tests render.
//
// File layout (little endian): int32 n_triangles, float triangles[9n],
// float uv[6n], int32 triangle_mat[n], int32 n_materials,
// are_material[n_materials], int32 n_textures, are_texture[n_textures],
// int32 background, float bg_a[3], int32 triangle_test, are_camera,
// are_render_params.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "aurora_gb300.h"

struct are_scene {
	std::vector<unsigned char> bytes;
};

template <class T>
static void put(std::vector<unsigned char> &b, const T *p, size_t n) {
	const unsigned char *c = reinterpret_cast<const unsigned char *>(p);
	b.insert(b.end(), c, c + sizeof(T) * n);
}

extern "C" {

const char *are_last_error(void) { return ""; }

are_status are_scene_create(const are_scene_desc *d, are_scene **out) {
	are_scene *s = new are_scene();
	const int32_t n = d->n_triangles;
	put(s->bytes, &n, 1);
	put(s->bytes, d->triangles, 9 * (size_t)n);
	std::vector<float> uv(6 * (size_t)n, -1.0f);
	if (d->triangle_uv) uv.assign(d->triangle_uv, d->triangle_uv + 6 * (size_t)n);
	put(s->bytes, uv.data(), uv.size());
	put(s->bytes, d->triangle_mat, (size_t)n);
	put(s->bytes, &d->n_materials, 1);
	put(s->bytes, d->materials, (size_t)d->n_materials);
	put(s->bytes, &d->n_textures, 1);
	put(s->bytes, d->textures, (size_t)d->n_textures);
	put(s->bytes, &d->background, 1);
	put(s->bytes, d->bg_a, 3);
	put(s->bytes, &d->triangle_test, 1);
	*out = s;
	return ARE_OK;
}

are_status are_render(are_scene *s, const are_camera *cam, const are_render_params *p, float *rgb, float *, are_render_stats *) {
	put(s->bytes, cam, 1);
	put(s->bytes, p, 1);
	const char *path = std::getenv("ARE_RECORD_PATH");
	if (!path) return ARE_ERR_INVALID_ARGUMENT;
	FILE *f = std::fopen(path, "wb");
	if (!f) return ARE_ERR_IO;
	std::fwrite(s->bytes.data(), 1, s->bytes.size(), f);
	std::fclose(f);
	for (int64_t i = 0; i < 3 * (int64_t)p->width * p->height; ++i) rgb[i] = 0.0f;
	return ARE_OK;
}

are_status are_scene_destroy(are_scene *s) {
	delete s;
	return ARE_OK;
}

}  // extern "C"
