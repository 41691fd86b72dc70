/* aurora_gb300_are.hpp — scenes of the reference library (are::ObjectSet)
 * into the core's scene builder.
 *
 * Header-only; include it where the reference's include/ directory is on the
 * include path (it includes <object/object_set.h>).  are::ObjectSet is a
 * vector of are::Triangle pointers (include/object/object_set.h:10-12); a
 * triangle exposes its vertices Q, Q + u, Q + v through get_vertices()
 * (include/object/triangle.h:31-32, src/object/triangle.cpp:41-45) but keeps
 * its Material and Texture private (include/object/triangle.h:36-39), so the
 * caller says which material and texture each triangle was made with: either
 * a core material index per triangle (add_object_set), or the are::Material
 * and are::Texture pointers it constructed the triangle with
 * (add_object_set_bound), which the adapter turns into core materials and
 * image textures itself: an are::Texture's texels through its public
 * width_, height_ and pixel(x, y) (include/texture.h:20-29,
 * src/texture.cpp:77-83), are::Reflective(r) as a metal of reflect_ratio r,
 * any other material (are::Diffuse) as lambertian.  The reference computes
 * in FP64; vertices and texels are rounded to FP32 here, the precision of
 * the core.
 */
#ifndef AURORA_GB300_ARE_HPP
#define AURORA_GB300_ARE_HPP

#include <material/reflective.h>
#include <object/object_set.h>
#include <texture.h>

#include <map>
#include <string>
#include <utility>
#include <vector>

#include "aurora_gb300.hpp"

namespace are_gb300 {

// Adds every triangle of `set` to `b` with material material_of(triangle);
// returns the number added.  A null triangle pointer or a triangle without
// three vertices is refused (Error, ARE_ERR_INVALID_ARGUMENT) before anything
// is added, as are::Triangle's constructor refuses bad input by throwing.
template <class MaterialOf>
int add_object_set(SceneBuilder &b, const are::ObjectSet &set, MaterialOf material_of) {
	for (size_t i = 0; i < set.triangles.size(); ++i) {
		const are::Triangle *t = set.triangles[i];
		if (!t || t->get_vertices().size() != 3)
			throw Error(ARE_ERR_INVALID_ARGUMENT, "are::ObjectSet triangle " + std::to_string(i) + " is null or malformed");
	}
	for (const are::Triangle *t : set.triangles) {
		const auto &v = t->get_vertices();
		b.triangle(Vec3{ v[0].x(), v[0].y(), v[0].z() }, Vec3{ v[1].x(), v[1].y(), v[1].z() },
			Vec3{ v[2].x(), v[2].y(), v[2].z() }, material_of(*t));
	}
	return (int)set.triangles.size();
}

// Every triangle with the same material.
inline int add_object_set(SceneBuilder &b, const are::ObjectSet &set, int material) {
	return add_object_set(b, set, [material](const are::Triangle &) { return material; });
}

// An are::Texture's texels as an image texture of `b` (row-major from the top, texel (x, y) =
// tex.pixel(x, y), the reference's [y][x] addressing); returns its index.  pixel() is not const in
// the reference, hence the non-const reference.  A texture without texels is refused.
inline int add_texture(SceneBuilder &b, are::Texture &tex, int filter = ARE_FILTER_NEAREST) {
	if (tex.width_ <= 0 || tex.height_ <= 0)
		throw Error(ARE_ERR_INVALID_ARGUMENT, "are::Texture without texels (width or height <= 0)");
	std::vector<float> rgb(3 * (size_t)tex.width_ * tex.height_);
	for (int y = 0; y < tex.height_; ++y)
		for (int x = 0; x < tex.width_; ++x) {
			const are::Color3 &c = tex.pixel(x, y);
			float *o = &rgb[3 * ((size_t)y * tex.width_ + x)];
			o[0] = (float)c.x(), o[1] = (float)c.y(), o[2] = (float)c.z();
		}
	return b.image(tex.width_, tex.height_, rgb.data(), filter);
}

// A material of the reference library with albedo texture `texture`: are::Reflective(r)
// (include/material/reflective.h) becomes a mirror metal (fuzz 0) of reflect_ratio r, any other
// (are::Diffuse, include/material/diffuse.h) lambertian.
inline int add_material(SceneBuilder &b, const are::Material &m, int texture) {
	if (auto *r = dynamic_cast<const are::Reflective *>(&m)) return b.metal(texture, 0.0f, (float)r->reflectivity_);
	return b.lambertian(texture);
}

// The materials and textures add_object_set_bound made, by the reference's pointers: the caller can
// keep one across several object sets so shared materials and textures are added once.
struct ObjectSetMaps {
	std::map<are::Texture *, int> textures;
	std::map<std::pair<const are::Material *, are::Texture *>, int> materials;
};

// Adds every triangle of `set` with the material and texture it was constructed with:
// binding(triangle) returns that std::pair<const are::Material *, are::Texture *> (are::Triangle keeps
// them private).  Each distinct texture becomes one image texture (add_texture), each distinct pair
// one core material (add_material); a triangle's texture coordinates are (0, 0) at Q, (1, 0) at
// Q + u and (0, 1) at Q + v.  A null triangle, material or texture is refused before anything is
// added.  Returns the number of triangles added.
template <class Binding>
int add_object_set_bound(SceneBuilder &b, const are::ObjectSet &set, Binding binding, ObjectSetMaps &maps,
	int filter = ARE_FILTER_NEAREST) {
	std::vector<std::pair<const are::Material *, are::Texture *>> bound(set.triangles.size());
	for (size_t i = 0; i < set.triangles.size(); ++i) {
		const are::Triangle *t = set.triangles[i];
		if (!t || t->get_vertices().size() != 3)
			throw Error(ARE_ERR_INVALID_ARGUMENT, "are::ObjectSet triangle " + std::to_string(i) + " is null or malformed");
		bound[i] = binding(*t);
		if (!bound[i].first || !bound[i].second)
			throw Error(ARE_ERR_INVALID_ARGUMENT, "are::ObjectSet triangle " + std::to_string(i) + " has no material or texture");
	}
	static const float uv[6] = { 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 1.0f };
	for (size_t i = 0; i < set.triangles.size(); ++i) {
		auto tex = maps.textures.find(bound[i].second);
		if (tex == maps.textures.end()) tex = maps.textures.emplace(bound[i].second, add_texture(b, *bound[i].second, filter)).first;
		auto mat = maps.materials.find(bound[i]);
		if (mat == maps.materials.end()) mat = maps.materials.emplace(bound[i], add_material(b, *bound[i].first, tex->second)).first;
		const auto &v = set.triangles[i]->get_vertices();
		b.triangle(Vec3{ v[0].x(), v[0].y(), v[0].z() }, Vec3{ v[1].x(), v[1].y(), v[1].z() },
			Vec3{ v[2].x(), v[2].y(), v[2].z() }, mat->second, uv);
	}
	return (int)set.triangles.size();
}

}  // namespace are_gb300

// The reference declares are::Triangle::trace_texture
// (include/object/triangle.h:29-30) but never defines it, so a program that
// constructs are::Triangles does not link.  Define ARE_GB300_DEFINE_TRACE_TEXTURE
// before including this header in exactly one translation unit to supply a
// definition that returns an empty texture (the patch renderer that would use
// it is not part of this path).
#ifdef ARE_GB300_DEFINE_TRACE_TEXTURE
are::Texture are::Triangle::trace_texture(const are::ObjectSet &, const are::Point3 &) const { return are::Texture(); }
#endif

#endif
