/*
 * ref_lib_harness.cpp — TEST INFRASTRUCTURE ONLY.
 *
 * Links the reference library's own sources (src/basic/*.cpp,
 * src/object/*.cpp, src/material/*.cpp, src/texture.cpp, compiled from the
 * reference tree) and exports the scene-API math the oracle and the host
 * adapter restate:
 *   are::Triangle ctor checks and FP64 Möller–Trumbore (src/object/triangle.cpp:9-121),
 *   are::reflect / are::refract (src/basic/vec3.cpp:182-199),
 *   are::Plane::intersect_ray (src/basic/plane.cpp:13-27),
 *   are::Texture PPM load + pixel (src/texture.cpp:9-50, 77-83).
 *
 * The library declares Triangle::trace_texture (include/object/triangle.h:31)
 * but never defines it; a definition returning an empty texture is supplied
 * here so the translation units link.
 */
#include <basic/plane.h>
#include <basic/ray.h>
#include <basic/vec3.h>
#include <cstdint>
#include <material/diffuse.h>
#include <material/reflective.h>
#include <object/object_set.h>
#include <object/triangle.h>
#include <stdexcept>
#include <texture.h>

namespace are {
Texture Triangle::trace_texture(const ObjectSet &, const Point3 &) const {
	return Texture();
}
} // namespace are

extern "C" {

/* 0 = constructed, 1 = the constructor threw std::invalid_argument. */
int ref_lib_triangle_check(const double *Q, const double *u, const double *v) {
	are::Diffuse m;
	are::Texture t;
	try {
		are::Triangle tri(are::Vec3(Q[0], Q[1], Q[2]), are::Vec3(u[0], u[1], u[2]), are::Vec3(v[0], v[1], v[2]), &m, &t);
	} catch (const std::invalid_argument &) {
		return 1;
	}
	return 0;
}

/* FP64 Triangle::intersect_ray on m triangles (Q,u,v: m x 9 doubles), first
 * hit in index order with the smallest distance; the hit point is returned,
 * as the reference exposes no t. rays: n x 6 doubles; out: n x 4 (id, p). */
void ref_lib_triangles_intersect(const double *tris, int m, const double *rays, int64_t n, double *out) {
	are::Diffuse mat;
	are::Texture tex;
	std::vector<are::Triangle *> ts;
	for (int j = 0; j < m; ++j) {
		const double *t = tris + 9 * j;
		ts.push_back(new are::Triangle(are::Vec3(t[0], t[1], t[2]), are::Vec3(t[3], t[4], t[5]),
			are::Vec3(t[6], t[7], t[8]), &mat, &tex));
	}
	for (int64_t i = 0; i < n; ++i) {
		const double *r = rays + 6 * i;
		are::Ray ray(are::Vec3(r[0], r[1], r[2]), are::Vec3(r[3], r[4], r[5]));
		double best = 1e300;
		int id = -1;
		are::Point3 bp;
		for (int j = 0; j < m; ++j) {
			are::Point3 p;
			if (ts[j]->intersect_ray(ray, p)) {
				double dist = (p - ray.Q).length();
				if (dist < best) {
					best = dist;
					id = j;
					bp = p;
				}
			}
		}
		out[4 * i] = id;
		out[4 * i + 1] = bp.x();
		out[4 * i + 2] = bp.y();
		out[4 * i + 3] = bp.z();
	}
	for (auto *t : ts)
		delete t;
}

void ref_lib_reflect(const double *v, const double *n, double *out) {
	are::Vec3 r = are::reflect(are::Vec3(v[0], v[1], v[2]), are::Vec3(n[0], n[1], n[2]));
	out[0] = r.x(), out[1] = r.y(), out[2] = r.z();
}

void ref_lib_refract(const double *uv, const double *n, double eta, double *out) {
	are::Vec3 r = are::refract(are::Vec3(uv[0], uv[1], uv[2]), are::Vec3(n[0], n[1], n[2]), eta);
	out[0] = r.x(), out[1] = r.y(), out[2] = r.z();
}

int ref_lib_plane_intersect(const double *p, const double *nrm, const double *o, const double *d, double *hit) {
	are::Plane pl(are::Vec3(p[0], p[1], p[2]), are::Vec3(nrm[0], nrm[1], nrm[2]));
	are::Ray ray(are::Vec3(o[0], o[1], o[2]), are::Vec3(d[0], d[1], d[2]));
	are::Point3 h;
	if (!pl.intersect_ray(ray, h))
		return 0;
	hit[0] = h.x(), hit[1] = h.y(), hit[2] = h.z();
	return 1;
}

/* Loads a PPM through are::Texture and copies its texels (w*h*3 doubles,
 * row-major from the top, as pixel(x,y) indexes image_[y][x]).  Returns 0 on
 * success, 1 if the loader threw, 2 if cap is too small. */
int ref_lib_texture_load(const char *path, int *w, int *h, double *rgb, int64_t cap) {
	try {
		are::Texture t{ std::string(path) };
		*w = t.width_;
		*h = t.height_;
		if ((int64_t)t.width_ * t.height_ * 3 > cap)
			return 2;
		for (int y = 0; y < t.height_; ++y)
			for (int x = 0; x < t.width_; ++x) {
				are::Color3 &c = t.pixel(x, y);
				double *o = rgb + 3 * ((int64_t)y * t.width_ + x);
				o[0] = c.x(), o[1] = c.y(), o[2] = c.z();
			}
	} catch (const std::runtime_error &) {
		return 1;
	}
	return 0;
}

} // extern "C"
