/*
 * ref_rt_harness.cpp — TEST INFRASTRUCTURE ONLY.
 *
 * Compiles the reference's experiments/rt.cpp unchanged (it is #included from
 * the reference tree, never copied) and exports its hot-path functions with C
 * linkage so the oracle can be checked against the reference itself:
 *   Tri::intersect (rt.cpp:123-138), intersect() (rt.cpp:209-218),
 *   CheckerTexture::at (rt.cpp:98-101), Vec3::rotateToHemisphere
 *   (rt.cpp:50-55), render() (rt.cpp:337-374), writePPM (rt.cpp:377-392),
 *   and the Scene built by Scene::Scene (rt.cpp:153-167).
 *
 * Two changes of environment, no change of code: `main` is renamed so the
 * file links into a library, and std::random_device (rt.cpp:348-351, which
 * makes every run different) is replaced by a source returning a fixed seed,
 * so render() becomes reproducible.
 */
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <random>
#include <vector>

namespace std {
struct are_fixed_random_device {
	unsigned operator()();
};
} // namespace std
static unsigned g_fixed_seed = 0;
unsigned std::are_fixed_random_device::operator()() {
	return g_fixed_seed;
}

#define random_device are_fixed_random_device
#define main rt_reference_main
#include "experiments/rt.cpp"
#undef main
#undef random_device

static int texture_kind(const Texture *t, float *a, float *b, float *scale) {
	if (auto s = dynamic_cast<const SolidTexture *>(t)) {
		a[0] = s->c.r, a[1] = s->c.g, a[2] = s->c.b;
		b[0] = b[1] = b[2] = 0;
		*scale = 0;
		return 0;
	}
	auto c = dynamic_cast<const CheckerTexture *>(t);
	a[0] = c->a.r, a[1] = c->a.g, a[2] = c->a.b;
	b[0] = c->b.r, b[1] = c->b.g, b[2] = c->b.b;
	*scale = c->scale;
	return 1;
}

extern "C" {

int ref_scene_size(void) {
	Scene s;
	return (int)s.tris.size();
}

/* Per triangle: verts[9], uv[6] (uv0..uv2 .x/.y), mat[1], reflect_ratio[1],
 * tint[3], tex_kind[1], tex_a[3], tex_b[3], tex_scale[1] -> 28 floats. */
int ref_scene_export(float *out, int cap) {
	Scene s;
	int n = (int)s.tris.size();
	if (cap < n)
		return -1;
	for (int i = 0; i < n; ++i) {
		const Tri &t = s.tris[i];
		float *o = out + 28 * i;
		const Vec3 *v[3] = { &t.v0, &t.v1, &t.v2 };
		for (int k = 0; k < 3; ++k)
			o[3 * k] = v[k]->x, o[3 * k + 1] = v[k]->y, o[3 * k + 2] = v[k]->z;
		const Vec3 *uv[3] = { &t.uv0, &t.uv1, &t.uv2 };
		for (int k = 0; k < 3; ++k)
			o[9 + 2 * k] = uv[k]->x, o[9 + 2 * k + 1] = uv[k]->y;
		o[15] = (float)t.mat;
		o[16] = t.reflect_ratio;
		o[17] = t.metal_tint.r, o[18] = t.metal_tint.g, o[19] = t.metal_tint.b;
		o[20] = (float)texture_kind(t.tex, o + 21, o + 24, o + 27);
	}
	return n;
}

/* rays: n x 6 (o, d); hits: n x 4 (t, tri as int bits, u, v), t = 1e30 and
 * tri = -1 on a miss exactly as HitRec's defaults (rt.cpp:203-206). */
void ref_intersect(const float *rays, int64_t n, float *hits) {
	Scene s;
	for (int64_t i = 0; i < n; ++i) {
		const float *r = rays + 6 * i;
		HitRec h = intersect(s, Vec3(r[0], r[1], r[2]), Vec3(r[3], r[4], r[5]));
		float *o = hits + 4 * i;
		int32_t id = h.tri;
		o[0] = h.t;
		std::memcpy(&o[1], &id, 4);
		o[2] = h.u;
		o[3] = h.v;
	}
}

/* Tri::intersect on caller-provided triangles (tris: m x 9), linear scan
 * with rt.cpp's strict '<' rule, for random triangle soups. */
void ref_intersect_soup(const float *tris, int m, const float *rays, int64_t n, float *hits) {
	SolidTexture tex(Color(1, 1, 1));
	std::vector<Tri> soup;
	soup.reserve(m);
	for (int j = 0; j < m; ++j) {
		const float *t = tris + 9 * j;
		soup.emplace_back(Vec3(t[0], t[1], t[2]), Vec3(t[3], t[4], t[5]), Vec3(t[6], t[7], t[8]), Vec3(), Vec3(), Vec3(),
			&tex);
	}
	for (int64_t i = 0; i < n; ++i) {
		const float *r = rays + 6 * i;
		Vec3 o(r[0], r[1], r[2]), d(r[3], r[4], r[5]);
		HitRec best;
		for (int j = 0; j < m; ++j) {
			float t, u, v;
			if (soup[j].intersect(o, d, t, u, v) && t < best.t)
				best = { j, t, u, v };
		}
		float *out = hits + 4 * i;
		int32_t id = best.tri;
		out[0] = best.t;
		std::memcpy(&out[1], &id, 4);
		out[2] = best.u;
		out[3] = best.v;
	}
}

void ref_checker_at(const float *a, const float *b, float scale, float u, float v, float *out) {
	CheckerTexture c(Color(a[0], a[1], a[2]), Color(b[0], b[1], b[2]), scale);
	Color r = c.at(u, v);
	out[0] = r.r, out[1] = r.g, out[2] = r.b;
}

void ref_rotate_to_hemisphere(const float *n, float u, float v, float *out) {
	Vec3 r = Vec3(0, 0, 1).rotateToHemisphere(Vec3(n[0], n[1], n[2]), u, v);
	out[0] = r.x, out[1] = r.y, out[2] = r.z;
}

/* render() on the reference scene with rd() fixed to `seed`; rgb: w*h*3. */
void ref_render(unsigned seed, int w, int h, float *rgb) {
	g_fixed_seed = seed;
	Scene scene;
	Viewport vp(w, h);
	std::streambuf *old = std::cerr.rdbuf(nullptr);
	render(scene, Vec3(0, 0, 4), Vec3(0, 0, 0), Vec3(0, 1, 0), 50.f, vp);
	std::cerr.rdbuf(old);
	std::cerr.clear();
	for (int i = 0; i < w * h; ++i)
		rgb[3 * i] = vp.pixels[i].r, rgb[3 * i + 1] = vp.pixels[i].g, rgb[3 * i + 2] = vp.pixels[i].b;
}

/* writePPM of a caller image. */
int ref_write_ppm(const float *rgb, int w, int h, const char *path) {
	Viewport vp(w, h);
	for (int i = 0; i < w * h; ++i)
		vp.pixels[i] = Color(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
	writePPM(vp, path);
	return 0;
}

} // extern "C"
