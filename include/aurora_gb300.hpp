/* aurora_gb300.hpp — C++17 host layer over the C ABI of aurora_gb300.h.
 *
 * Owning handles (move-only, destroyed with the object), a scene builder in
 * the reference's vocabulary (spheres, quads, triangles, lambertian / metal /
 * dielectric / light materials, solid / checker / image textures), and the
 * output step: render to an Image, quantise and write PPM (rt.cpp writePPM,
 * experiments/rt.cpp:377-392) or PFM.  Errors become are_gb300::Error
 * exceptions carrying the status and are_last_error(), as the reference's
 * library reports bad input by throwing (src/object/triangle.cpp:13-36).
 *
 * Image textures are copied into the scene descriptor by value, so a texture
 * can be copied and destroyed freely (are::Texture owns raw row pointers and
 * has no copy constructor, src/texture.cpp:68-75).
 */
#ifndef AURORA_GB300_HPP
#define AURORA_GB300_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "aurora_gb300.h"

namespace are_gb300 {

struct Error : std::runtime_error {
	are_status status;
	Error(are_status s, const std::string &what) : std::runtime_error(what), status(s) {}
};

inline void check(are_status s) {
	if (s != ARE_OK) throw Error(s, std::string(are_status_string(s)) + ": " + are_last_error());
}

struct Vec3 {
	double x = 0, y = 0, z = 0;
};

// A scene on the device; created from a descriptor, which it copies.
class Scene {
public:
	explicit Scene(const are_scene_desc &desc) { check(are_scene_create(&desc, &h_)); }
	~Scene() {
		if (h_) are_scene_destroy(h_);
	}
	Scene(Scene &&o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
	Scene &operator=(Scene &&o) noexcept {
		if (this != &o) {
			if (h_) are_scene_destroy(h_);
			h_ = std::exchange(o.h_, nullptr);
		}
		return *this;
	}
	Scene(const Scene &) = delete;
	Scene &operator=(const Scene &) = delete;
	are_scene *get() const { return h_; }

private:
	are_scene *h_ = nullptr;
};

// Flat arrays of the descriptor, filled in the reference's vocabulary.
class SceneBuilder {
public:
	int solid(float r, float g, float b) {
		are_texture t{};
		t.type = ARE_TEX_SOLID;
		t.a[0] = r, t.a[1] = g, t.a[2] = b;
		return push_texture(t);
	}
	// rt.cpp:85-102 CheckerTexture: ((floor(u s) + floor(v s)) % 2 == 0) ? a : b
	int checker(const float a[3], const float b[3], float scale) {
		are_texture t{};
		t.type = ARE_TEX_CHECKER;
		t.scale = scale;
		for (int k = 0; k < 3; ++k) t.a[k] = a[k], t.b[k] = b[k];
		return push_texture(t);
	}
	// width x height RGB texels, row-major from the top (are::Texture::pixel(x, y))
	// texels row-major from the top, as are::Texture::pixel(x, y); filter ARE_FILTER_NEAREST or _BILINEAR
	int image(int width, int height, const float *rgb, int filter = ARE_FILTER_NEAREST) {
		are_texture t{};
		t.type = ARE_TEX_IMAGE;
		t.filter = filter;
		t.width = width, t.height = height;
		t.texel_offset = (int32_t)(texels_.size() / 3);
		texels_.insert(texels_.end(), rgb, rgb + (size_t)width * height * 3);
		return push_texture(t);
	}
	int lambertian(int texture) { return push_material(ARE_MAT_LAMBERTIAN, texture); }
	int metal(int texture, float fuzz, float reflect_ratio = 1.0f) {
		int m = push_material(ARE_MAT_METAL, texture);
		mats_[m].fuzz = fuzz;
		mats_[m].reflect_ratio = reflect_ratio;
		for (int k = 0; k < 3; ++k) mats_[m].tint[k] = 1.0f;
		return m;
	}
	int dielectric(float ior) {
		int m = push_material(ARE_MAT_DIELECTRIC, solid(1, 1, 1));
		mats_[m].ior = ior;
		return m;
	}
	int light(float r, float g, float b) {
		int m = push_material(ARE_MAT_DIFFUSE_LIGHT, solid(0, 0, 0));
		mats_[m].emit[0] = r, mats_[m].emit[1] = g, mats_[m].emit[2] = b;
		return m;
	}
	void sphere(Vec3 c, double radius, int material) {
		spheres_.insert(spheres_.end(), { (float)c.x, (float)c.y, (float)c.z, (float)radius });
		sphere_mat_.push_back(material);
	}
	// parallelogram Q + a u + b v, a, b in [0, 1]
	void quad(Vec3 Q, Vec3 u, Vec3 v, int material) {
		quads_.insert(quads_.end(), { (float)Q.x, (float)Q.y, (float)Q.z, (float)u.x, (float)u.y, (float)u.z, (float)v.x,
										(float)v.y, (float)v.z });
		quad_mat_.push_back(material);
	}
	// are::Triangle(Q, u, v, ...) has the vertices Q, Q + u, Q + v (src/object/triangle.cpp:42-45)
	void triangle(Vec3 a, Vec3 b, Vec3 c, int material) {
		tris_.insert(tris_.end(), { (float)a.x, (float)a.y, (float)a.z, (float)b.x, (float)b.y, (float)b.z, (float)c.x,
									  (float)c.y, (float)c.z });
		tri_mat_.push_back(material);
		if (!tri_uv_.empty()) tri_uv_.insert(tri_uv_.end(), 6, 0.0f);
	}
	// a triangle with per-vertex texture coordinates uv = (u0, v0, u1, v1, u2, v2) (rt.cpp:139-142 bary2uv);
	// triangles added without them get (0, 0) at every vertex
	void triangle(Vec3 a, Vec3 b, Vec3 c, int material, const float uv[6]) {
		triangle(a, b, c, material);
		tri_uv_.resize(6 * tri_mat_.size(), 0.0f);  // the earlier triangles' (0, 0)s, then this one's six
		for (int k = 0; k < 6; ++k) tri_uv_[tri_uv_.size() - 6 + k] = uv[k];
	}
	void background(int kind, const float a[3], const float b[3]) {
		bg_kind_ = kind;
		for (int k = 0; k < 3; ++k) bg_a_[k] = a[k], bg_b_[k] = b[k];
	}
	void triangle_test(int t) { tri_test_ = t; }

	are_scene_desc desc() const {
		are_scene_desc d{};
		d.n_spheres = (int32_t)sphere_mat_.size();
		d.spheres = spheres_.data();
		d.sphere_mat = sphere_mat_.data();
		d.n_quads = (int32_t)quad_mat_.size();
		d.quads = quads_.data();
		d.quad_mat = quad_mat_.data();
		d.n_triangles = (int32_t)tri_mat_.size();
		d.triangles = tris_.data();
		d.triangle_mat = tri_mat_.data();
		d.triangle_uv = tri_uv_.empty() ? nullptr : tri_uv_.data();
		d.n_materials = (int32_t)mats_.size();
		d.materials = mats_.data();
		d.n_textures = (int32_t)texs_.size();
		d.textures = texs_.data();
		d.n_texels = (int64_t)(texels_.size() / 3);
		d.texels = texels_.empty() ? nullptr : texels_.data();
		d.background = bg_kind_;
		for (int k = 0; k < 3; ++k) d.bg_a[k] = bg_a_[k], d.bg_b[k] = bg_b_[k];
		d.triangle_test = tri_test_;
		return d;
	}
	Scene build() const { return Scene(desc()); }

private:
	int push_texture(const are_texture &t) {
		texs_.push_back(t);
		return (int)texs_.size() - 1;
	}
	int push_material(int type, int texture) {
		are_material m{};
		m.type = type;
		m.texture = texture;
		m.reflect_ratio = 1.0f;
		mats_.push_back(m);
		return (int)mats_.size() - 1;
	}
	std::vector<float> spheres_, quads_, tris_, texels_, tri_uv_;
	std::vector<int32_t> sphere_mat_, quad_mat_, tri_mat_;
	std::vector<are_material> mats_;
	std::vector<are_texture> texs_;
	int bg_kind_ = ARE_BG_CONSTANT;
	float bg_a_[3] = { 0, 0, 0 }, bg_b_[3] = { 0, 0, 0 };
	int tri_test_ = ARE_TRI_WATERTIGHT;
};

// Linear FP32 RGB, row-major from the top (rt.cpp's Viewport).
struct Image {
	int width = 0, height = 0;
	std::vector<float> rgb;
};

inline Image render(const Scene &scene, const are_camera &camera, const are_render_params &params,
	are_render_stats *stats = nullptr, std::vector<float> *variance = nullptr) {
	Image im;
	im.width = params.width, im.height = params.height;
	im.rgb.resize((size_t)params.width * params.height * 3);
	if (variance) variance->resize(im.rgb.size());
	are_render_params p = params;
	p.flags &= ~ARE_FLAG_DEVICE_OUTPUT;
	check(are_render(scene.get(), &camera, &p, im.rgb.data(), variance ? variance->data() : nullptr, stats));
	return im;
}

// 8-bit RGB of an image: ARE_TONEMAP_GAMMA is rt.cpp writePPM's quantisation
inline std::vector<uint8_t> tonemap(const Image &im, int mode = ARE_TONEMAP_GAMMA, float gamma = 2.2f) {
	std::vector<uint8_t> out(im.rgb.size());
	are_tonemap_params tp{};
	tp.mode = mode;
	tp.gamma = gamma;
	check(are_tonemap(im.rgb.data(), (int64_t)im.rgb.size(), &tp, out.data()));
	return out;
}

inline void write_ppm(const std::string &path, const Image &im, int mode = ARE_TONEMAP_GAMMA, float gamma = 2.2f) {
	std::vector<uint8_t> b = tonemap(im, mode, gamma);
	check(are_write_ppm(path.c_str(), b.data(), im.width, im.height));
}

inline void write_pfm(const std::string &path, const Image &im) {
	check(are_write_pfm(path.c_str(), im.rgb.data(), im.width, im.height));
}

inline Image read_ppm(const std::string &path) {
	Image im;
	check(are_read_ppm(path.c_str(), &im.width, &im.height, nullptr));
	im.rgb.resize((size_t)im.width * im.height * 3);
	check(are_read_ppm(path.c_str(), &im.width, &im.height, im.rgb.data()));
	return im;
}

}  // namespace are_gb300

#endif /* AURORA_GB300_HPP */
