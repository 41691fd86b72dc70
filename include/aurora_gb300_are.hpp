/* aurora_gb300_are.hpp — scenes of the reference library (are::ObjectSet)
 * into the core's scene builder.
 *
 * Header-only; include it where the reference's include/ directory is on the
 * include path (it includes <object/object_set.h>).  are::ObjectSet is a
 * vector of are::Triangle pointers (include/object/object_set.h:10-12); a
 * triangle exposes its vertices Q, Q + u, Q + v through get_vertices()
 * (include/object/triangle.h:31-32, src/object/triangle.cpp:41-45) but keeps
 * its Material and Texture private, so the caller maps each triangle to a
 * core material index (for instance in the order it created them).  The
 * reference computes in FP64; vertices are rounded to FP32 here, the
 * precision of the core's primitive tests.
 */
#ifndef AURORA_GB300_ARE_HPP
#define AURORA_GB300_ARE_HPP

#include <object/object_set.h>

#include <string>

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
