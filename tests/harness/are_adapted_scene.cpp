// are_adapted_scene.cpp — a scene built with the reference library's own types
// (are::ObjectSet of are::Triangle, are::Diffuse, are::Reflective, are::Texture
// filled through pixel()), turned into the core's scene descriptor by
// include/aurora_gb300_are.hpp's add_object_set_bound, and written out (TEST
// INFRASTRUCTURE: built against the reference's headers and compiled sources
// by tests/golden/make_adapted_scene.py and tests/test_are_adapter.py).
//
// The scene: a box room of 2-triangle walls (a checker texture of 8 x 8
// texels on the floor, a gradient texture on the back wall, plain colours
// elsewhere), a reflective block and a sky-gradient background as the light.
//
// Output (little endian): int32 n, float triangles[9n], float uv[6n],
// int32 mat[n], int32 n_materials, are_material[], int32 n_textures,
// are_texture[], int64 n_texels, float texels[3 n_texels].
#define ARE_GB300_DEFINE_TRACE_TEXTURE
#include <material/diffuse.h>
#include <material/reflective.h>

#include <cstdio>
#include <map>
#include <utility>
#include <vector>

#include "aurora_gb300_are.hpp"

struct Binding {
	std::map<const are::Triangle *, std::pair<const are::Material *, are::Texture *>> of;
	std::pair<const are::Material *, are::Texture *> operator()(const are::Triangle &t) const { return of.at(&t); }
};

static void quad(are::ObjectSet &set, Binding &bind, are::Point3 Q, are::Vec3 u, are::Vec3 v, are::Material *m,
	are::Texture *t) {
	// two triangles (Q, u, v) and (Q + u + v, -u, -v): the texture's (0, 0) corner at Q and at the far corner
	are::Triangle *a = new are::Triangle(Q, u, v, m, t);
	are::Triangle *b = new are::Triangle(Q + u + v, u * -1.0, v * -1.0, m, t);
	set.triangles.push_back(a);
	set.triangles.push_back(b);
	bind.of[a] = { m, t };
	bind.of[b] = { m, t };
}

int main(int argc, char **argv) {
	if (argc < 2) return 2;
	are::Diffuse diffuse;
	are::Reflective mirror(0.8);
	are::Texture checker(8, 8, are::Color3(0.9, 0.9, 0.9)), ramp(16, 4, are::Color3(0, 0, 0));
	are::Texture white(1, 1, are::Color3(0.73, 0.73, 0.73)), red(1, 1, are::Color3(0.65, 0.05, 0.05));
	are::Texture steel(1, 1, are::Color3(0.8, 0.85, 0.9));
	for (int y = 0; y < 8; ++y)
		for (int x = 0; x < 8; ++x)
			if ((x + y) % 2) checker.pixel(x, y) = are::Color3(0.1, 0.2, 0.6);
	for (int y = 0; y < 4; ++y)
		for (int x = 0; x < 16; ++x) ramp.pixel(x, y) = are::Color3(x / 15.0, 0.3 + 0.1 * y, 1.0 - x / 15.0);
	are::ObjectSet set;
	Binding bind;
	const double S = 4.0;
	quad(set, bind, are::Point3(0, 0, 0), are::Vec3(S, 0, 0), are::Vec3(0, 0, S), &diffuse, &checker);   // floor
	quad(set, bind, are::Point3(0, 0, S), are::Vec3(S, 0, 0), are::Vec3(0, S, 0), &diffuse, &ramp);      // back
	quad(set, bind, are::Point3(0, 0, 0), are::Vec3(0, 0, S), are::Vec3(0, S, 0), &diffuse, &red);       // left
	quad(set, bind, are::Point3(S, 0, 0), are::Vec3(0, S, 0), are::Vec3(0, 0, S), &diffuse, &white);     // right
	// a reflective block, four sides and a top
	const double x0 = 1.2, x1 = 2.4, z0 = 1.6, z1 = 2.8, h = 1.5;
	quad(set, bind, are::Point3(x0, 0, z0), are::Vec3(x1 - x0, 0, 0), are::Vec3(0, h, 0), &mirror, &steel);
	quad(set, bind, are::Point3(x0, 0, z1), are::Vec3(0, h, 0), are::Vec3(x1 - x0, 0, 0), &mirror, &steel);
	quad(set, bind, are::Point3(x0, 0, z0), are::Vec3(0, h, 0), are::Vec3(0, 0, z1 - z0), &mirror, &steel);
	quad(set, bind, are::Point3(x1, 0, z0), are::Vec3(0, 0, z1 - z0), are::Vec3(0, h, 0), &mirror, &steel);
	quad(set, bind, are::Point3(x0, h, z0), are::Vec3(0, 0, z1 - z0), are::Vec3(x1 - x0, 0, 0), &diffuse, &white);
	are_gb300::SceneBuilder b;
	are_gb300::ObjectSetMaps maps;
	const int n = are_gb300::add_object_set_bound(b, set, bind, maps);
	const are_scene_desc d = b.desc();
	FILE *f = std::fopen(argv[1], "wb");
	if (!f) return 3;
	std::fwrite(&n, 4, 1, f);
	std::fwrite(d.triangles, 4, 9 * (size_t)n, f);
	std::fwrite(d.triangle_uv, 4, 6 * (size_t)n, f);
	std::fwrite(d.triangle_mat, 4, (size_t)n, f);
	std::fwrite(&d.n_materials, 4, 1, f);
	std::fwrite(d.materials, sizeof(are_material), (size_t)d.n_materials, f);
	std::fwrite(&d.n_textures, 4, 1, f);
	std::fwrite(d.textures, sizeof(are_texture), (size_t)d.n_textures, f);
	std::fwrite(&d.n_texels, 8, 1, f);
	std::fwrite(d.texels, 4, 3 * (size_t)d.n_texels, f);
	std::fclose(f);
	std::printf("%d triangles, %zu textures, %zu materials\n", n, maps.textures.size(), maps.materials.size());
	for (auto *t : set.triangles) delete t;
	return 0;
}
