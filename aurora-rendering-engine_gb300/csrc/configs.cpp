// configs.cpp — seeded synthetic scenes for the benchmark and parity tests.
//
// Every scene is a pure function of (config, seed): random numbers come from
// SplitMix64 (Steele, Lea, Flood 2014) and geometry is computed in double,
// so the same descriptor is produced on every host.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "scene.h"

struct are_config {
	std::vector<float> spheres, quads, tris, tri_uv;
	std::vector<int32_t> sphere_mat, quad_mat, tri_mat;
	std::vector<are_material> mats;
	std::vector<are_texture> texs;
	std::vector<float> texels;
	are_scene_desc desc{};
	are_camera cam{};
	are_render_params params{};

	int texture(int type, const float a[3], const float b[3] = nullptr, float scale = 1.0f, int mapping = 0,
		const float *center = nullptr) {
		are_texture t{};
		t.type = type;
		t.mapping = mapping;
		t.scale = scale;
		for (int k = 0; k < 3; ++k) {
			t.a[k] = a[k];
			t.b[k] = b ? b[k] : 0.0f;
			t.center[k] = center ? center[k] : 0.0f;
		}
		texs.push_back(t);
		return (int)texs.size() - 1;
	}
	int material(int type, int tex, float fuzz = 0.0f, float ior = 1.5f, const float *emit = nullptr) {
		are_material m{};
		m.type = type;
		m.texture = tex;
		m.fuzz = fuzz;
		m.ior = ior;
		if (emit)
			for (int k = 0; k < 3; ++k) m.emit[k] = emit[k];
		mats.push_back(m);
		return (int)mats.size() - 1;
	}
	int lambertian(float r, float g, float b) {
		float c[3] = { r, g, b };
		return material(ARE_MAT_LAMBERTIAN, texture(ARE_TEX_SOLID, c));
	}
	void sphere(double x, double y, double z, double r, int m) {
		spheres.insert(spheres.end(), { (float)x, (float)y, (float)z, (float)r });
		sphere_mat.push_back(m);
	}
	void quad(const double Q[3], const double u[3], const double v[3], int m) {
		for (int k = 0; k < 3; ++k) quads.push_back((float)Q[k]);
		for (int k = 0; k < 3; ++k) quads.push_back((float)u[k]);
		for (int k = 0; k < 3; ++k) quads.push_back((float)v[k]);
		quad_mat.push_back(m);
	}
	void finish() {
		are_scene_desc &d = desc;
		d.n_spheres = (int32_t)sphere_mat.size();
		d.spheres = spheres.data();
		d.sphere_mat = sphere_mat.data();
		d.n_quads = (int32_t)quad_mat.size();
		d.quads = quads.data();
		d.quad_mat = quad_mat.data();
		d.n_triangles = (int32_t)tri_mat.size();
		d.triangles = tris.data();
		d.triangle_uv = tri_uv.empty() ? nullptr : tri_uv.data();
		d.triangle_mat = tri_mat.data();
		d.n_materials = (int32_t)mats.size();
		d.materials = mats.data();
		d.n_textures = (int32_t)texs.size();
		d.textures = texs.data();
		d.n_texels = (int64_t)texels.size() / 3;
		d.texels = texels.empty() ? nullptr : texels.data();
	}
};

namespace are_core {
namespace {

struct SplitMix {
	uint64_t s;
	uint64_t next() {
		uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
		z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
		z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
		return z ^ (z >> 31);
	}
	double u() { return (double)(next() >> 11) * 0x1.0p-53; }
	double u(double lo, double hi) { return lo + (hi - lo) * u(); }
};

void set_cam(are_camera &c, double fx, double fy, double fz, double tx, double ty, double tz, double vfov,
	double aperture, double focus) {
	c.lookfrom[0] = (float)fx, c.lookfrom[1] = (float)fy, c.lookfrom[2] = (float)fz;
	c.lookat[0] = (float)tx, c.lookat[1] = (float)ty, c.lookat[2] = (float)tz;
	c.vup[0] = 0.f, c.vup[1] = 1.f, c.vup[2] = 0.f;
	c.vfov_deg = (float)vfov;
	c.aperture = (float)aperture;
	c.focus_dist = (float)focus;
}

void set_params(are_render_params &p, int w, int h, int spp, int depth, uint64_t seed, float t_min) {
	p = are_render_params{};
	p.width = w, p.height = h, p.spp = spp, p.max_depth = depth;
	p.seed = seed;
	p.rr_depth = 3;
	p.t_min = t_min;
	p.estimator = ARE_EST_PATH;
}

// Random spheres: ground r=1000 lambertian 0.5; 22x22 grid of r=0.2 spheres
// centred at (a+U, 0.2, b+U); materials p=.8 lambertian (albedo U^3 * U^3),
// p=.15 metal (albedo U(.5,1), fuzz U(0,.5)), p=.05 dielectric 1.5; three r=1
// spheres.  Camera (13,2,3) -> origin, vfov 20, aperture .1, focus 10.
void random_spheres(are_config &c, uint64_t seed) {
	SplitMix r{ seed };
	c.sphere(0, -1000, 0, 1000, c.lambertian(0.5f, 0.5f, 0.5f));
	for (int a = -11; a < 11; ++a)
		for (int b = -11; b < 11; ++b) {
			double choose = r.u();
			double x = a + r.u(), z = b + r.u();
			int m;
			if (choose < 0.8) {
				float alb[3];
				for (int k = 0; k < 3; ++k) alb[k] = (float)r.u();
				for (int k = 0; k < 3; ++k) alb[k] *= (float)r.u();
				m = c.lambertian(alb[0], alb[1], alb[2]);
			} else if (choose < 0.95) {
				float alb[3];
				for (int k = 0; k < 3; ++k) alb[k] = (float)r.u(0.5, 1.0);
				m = c.material(ARE_MAT_METAL, c.texture(ARE_TEX_SOLID, alb), (float)r.u(0.0, 0.5));
			} else {
				float w[3] = { 1.f, 1.f, 1.f };
				m = c.material(ARE_MAT_DIELECTRIC, c.texture(ARE_TEX_SOLID, w), 0.0f, 1.5f);
			}
			c.sphere(x, 0.2, z, 0.2, m);
		}
	float w[3] = { 1.f, 1.f, 1.f };
	c.sphere(0, 1, 0, 1.0, c.material(ARE_MAT_DIELECTRIC, c.texture(ARE_TEX_SOLID, w), 0.0f, 1.5f));
	c.sphere(-4, 1, 0, 1.0, c.lambertian(0.4f, 0.2f, 0.1f));
	float mc[3] = { 0.7f, 0.6f, 0.5f };
	c.sphere(4, 1, 0, 1.0, c.material(ARE_MAT_METAL, c.texture(ARE_TEX_SOLID, mc), 0.0f));
	c.desc.background = ARE_BG_SKY_GRADIENT;
	for (int k = 0; k < 3; ++k) c.desc.bg_a[k] = 1.0f;
	c.desc.bg_b[0] = 0.5f, c.desc.bg_b[1] = 0.7f, c.desc.bg_b[2] = 1.0f;
	c.desc.triangle_test = ARE_TRI_WATERTIGHT;
	set_cam(c.cam, 13, 2, 3, 0, 0, 0, 20, 0.1, 10.0);
	set_params(c.params, 400, 225, 32, 50, 1, 1e-3f);
}

void rot_y(double deg, const double in[3], double out[3]) {
	double t = deg * 3.14159265358979323846 / 180.0, c = std::cos(t), s = std::sin(t);
	out[0] = c * in[0] + s * in[2];
	out[1] = in[1];
	out[2] = -s * in[0] + c * in[2];
}

// axis-aligned box [0,size] rotated about +y by deg, then translated
void box(are_config &c, const double size[3], double deg, const double tr[3], int m) {
	double e[3][3] = { { size[0], 0, 0 }, { 0, size[1], 0 }, { 0, 0, size[2] } };
	const int face[6][3] = { // corner offset mask (x,y,z), first edge, second edge
		{ 0, 0, 1 }, { 2, 0, 1 }, { 1, 2, 1 }, { 0, 2, 1 }, { 0, 0, 2 }, { 4, 0, 2 } };
	for (const auto &f : face) {
		double Q[3] = { 0, 0, 0 };
		if (f[0] & 2) Q[2] = size[2];
		if (f[0] & 1) Q[0] = size[0];
		if (f[0] & 4) Q[1] = size[1];
		double Qr[3], ur[3], vr[3];
		rot_y(deg, Q, Qr);
		rot_y(deg, e[f[1]], ur);
		rot_y(deg, e[f[2]], vr);
		for (int k = 0; k < 3; ++k) Qr[k] += tr[k];
		c.quad(Qr, ur, vr, m);
	}
}

// Cornell box of side 555: red wall x=0, green wall x=555, white floor,
// ceiling and back wall, a 130 x 105 light facing down below the ceiling,
// and two rotated boxes.  Camera (278,278,-800) -> (278,278,0), vfov 40.
void cornell(are_config &c, bool occluded) {
	int red = c.lambertian(0.65f, 0.05f, 0.05f);
	int white = c.lambertian(0.73f, 0.73f, 0.73f);
	int green = c.lambertian(0.12f, 0.45f, 0.15f);
	float e[3] = { 15.f, 15.f, 15.f }, k0[3] = { 0.f, 0.f, 0.f };
	int light = c.material(ARE_MAT_DIFFUSE_LIGHT, c.texture(ARE_TEX_SOLID, k0), 0.0f, 1.0f, e);
	auto q = [&](double qx, double qy, double qz, double ux, double uy, double uz, double vx, double vy, double vz,
				 int m) {
		double Q[3] = { qx, qy, qz }, u[3] = { ux, uy, uz }, v[3] = { vx, vy, vz };
		c.quad(Q, u, v, m);
	};
	q(555, 0, 0, 0, 555, 0, 0, 0, 555, green);
	q(0, 0, 0, 0, 555, 0, 0, 0, 555, red);
	q(0, 0, 0, 555, 0, 0, 0, 0, 555, white);
	q(555, 555, 555, -555, 0, 0, 0, 0, -555, white);
	q(0, 0, 555, 555, 0, 0, 0, 555, 0, white);
	q(343, 554, 332, -130, 0, 0, 0, 0, -105, light);  // normal -y
	double tall[3] = { 165, 330, 165 }, t1[3] = { 265, 0, 295 };
	double shrt[3] = { 165, 165, 165 }, t2[3] = { 130, 0, 65 };
	box(c, tall, 15.0, t1, white);
	box(c, shrt, -18.0, t2, white);
	if (occluded) q(128, 534, 129.5, 300, 0, 0, 0, 0, 300, white);
	c.desc.background = ARE_BG_CONSTANT;
	c.desc.triangle_test = ARE_TRI_WATERTIGHT;
	set_cam(c.cam, 278, 278, -800, 278, 278, 0, 40, 0.0, 10.0);
	set_params(c.params, 600, 600, 1024, occluded ? 16 : 50, 1, 1e-3f);
}

// ---- displaced geodesic icosphere --------------------------------------------

uint32_t hash3(int32_t x, int32_t y, int32_t z, uint64_t seed) {
	uint64_t h = seed ^ ((uint64_t)(uint32_t)x * 0x9E3779B97F4A7C15ULL) ^ ((uint64_t)(uint32_t)y * 0xC2B2AE3D27D4EB4FULL) ^
		((uint64_t)(uint32_t)z * 0x165667B19E3779F9ULL);
	h = (h ^ (h >> 30)) * 0xBF58476D1CE4E5B9ULL;
	h = (h ^ (h >> 27)) * 0x94D049BB133111EBULL;
	return (uint32_t)((h ^ (h >> 31)) >> 32);
}

// value noise: hashed lattice values in [-1,1], smoothstep-weighted trilinear blend
double value_noise(double x, double y, double z, uint64_t seed) {
	double fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
	int32_t ix = (int32_t)fx, iy = (int32_t)fy, iz = (int32_t)fz;
	double tx = x - fx, ty = y - fy, tz = z - fz;
	auto sm = [](double t) { return t * t * (3.0 - 2.0 * t); };
	double sx = sm(tx), sy = sm(ty), sz = sm(tz);
	double v[2][2][2];
	for (int a = 0; a < 2; ++a)
		for (int b = 0; b < 2; ++b)
			for (int cc = 0; cc < 2; ++cc) v[a][b][cc] = hash3(ix + a, iy + b, iz + cc, seed) * (2.0 / 4294967295.0) - 1.0;
	auto lerp = [](double p, double q, double t) { return p + (q - p) * t; };
	double x00 = lerp(v[0][0][0], v[1][0][0], sx), x10 = lerp(v[0][1][0], v[1][1][0], sx);
	double x01 = lerp(v[0][0][1], v[1][0][1], sx), x11 = lerp(v[0][1][1], v[1][1][1], sx);
	return lerp(lerp(x00, x10, sy), lerp(x01, x11, sy), sz);
}

double fbm3(double x, double y, double z, uint64_t seed) {
	double amp = 1.0, f = 1.0, s = 0.0, norm = 0.0;
	for (int o = 0; o < 3; ++o) {  // 3 octaves, lacunarity 2, gain 0.5
		s += amp * value_noise(x * f, y * f, z * f, seed + 1000003ULL * o);
		norm += amp;
		amp *= 0.5;
		f *= 2.0;
	}
	return s / norm;
}

void icosphere(are_config &c, int n, const double ctr[3], double radius, uint64_t seed, int mat) {
	const double phi = (1.0 + std::sqrt(5.0)) / 2.0;
	double V[12][3] = { { -1, phi, 0 }, { 1, phi, 0 }, { -1, -phi, 0 }, { 1, -phi, 0 }, { 0, -1, phi }, { 0, 1, phi },
		{ 0, -1, -phi }, { 0, 1, -phi }, { phi, 0, -1 }, { phi, 0, 1 }, { -phi, 0, -1 }, { -phi, 0, 1 } };
	// faces: all vertex triples that are pairwise at edge length 2, wound outward
	std::vector<std::array<int, 3>> F;
	auto d2 = [&](int a, int b) {
		double s = 0;
		for (int k = 0; k < 3; ++k) s += (V[a][k] - V[b][k]) * (V[a][k] - V[b][k]);
		return s;
	};
	for (int a = 0; a < 12; ++a)
		for (int b = a + 1; b < 12; ++b)
			for (int cc = b + 1; cc < 12; ++cc)
				if (std::fabs(d2(a, b) - 4) < 1e-9 && std::fabs(d2(a, cc) - 4) < 1e-9 && std::fabs(d2(b, cc) - 4) < 1e-9) {
					double e1[3], e2[3], nn[3];
					for (int k = 0; k < 3; ++k) e1[k] = V[b][k] - V[a][k], e2[k] = V[cc][k] - V[a][k];
					nn[0] = e1[1] * e2[2] - e1[2] * e2[1];
					nn[1] = e1[2] * e2[0] - e1[0] * e2[2];
					nn[2] = e1[0] * e2[1] - e1[1] * e2[0];
					if (nn[0] * V[a][0] + nn[1] * V[a][1] + nn[2] * V[a][2] < 0)
						F.push_back({ a, cc, b });
					else
						F.push_back({ a, b, cc });
				}
	// vertex at lattice (i, j, k) of face (A, B, C), i + j + k = n: terms are
	// added in the fixed order A, B, C, so a point on an edge shared by two
	// faces gets bit-identical coordinates from both (x + 0 == x, a + b == b + a).
	auto vert = [&](const std::array<int, 3> &f, int i, int j, int k, float out[3]) {
		double p[3];
		for (int m = 0; m < 3; ++m) {
			double a = i * V[f[0]][m], b = j * V[f[1]][m], cc = k * V[f[2]][m];
			// order-independent sum of the non-zero terms
			double t[3] = { a, b, cc };
			std::sort(t, t + 3);
			p[m] = (t[0] + t[1]) + t[2];
		}
		double l = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
		for (int m = 0; m < 3; ++m) p[m] /= l;
		double disp = 1.0 + 0.05 * fbm3(p[0] * 4.0, p[1] * 4.0, p[2] * 4.0, seed);
		for (int m = 0; m < 3; ++m) out[m] = (float)(ctr[m] + radius * disp * p[m]);
	};
	c.tris.reserve(c.tris.size() + 9 * (size_t)20 * n * n);
	for (const auto &f : F) {
		for (int i = 0; i < n; ++i)
			for (int j = 0; j < n - i; ++j) {
				int k = n - i - j;
				float a[3], b[3], cc[3], d[3];
				vert(f, i, j, k, a);
				vert(f, i + 1, j, k - 1, b);
				vert(f, i, j + 1, k - 1, cc);
				c.tris.insert(c.tris.end(), { a[0], a[1], a[2], b[0], b[1], b[2], cc[0], cc[1], cc[2] });
				c.tri_mat.push_back(mat);
				if (i + j < n - 1) {
					vert(f, i + 1, j + 1, k - 2, d);
					c.tris.insert(c.tris.end(), { b[0], b[1], b[2], d[0], d[1], d[2], cc[0], cc[1], cc[2] });
					c.tri_mat.push_back(mat);
				}
			}
	}
}

// Displaced icosphere (frequency n -> 20 n^2 triangles) with a spherical
// checker (scale 10) on a 2-triangle ground, lit by a sphere light.
void mesh(are_config &c, uint64_t seed, int freq) {
	double ctr[3] = { 0.0, 1.0, 0.0 };
	float ca[3] = { 0.85f, 0.85f, 0.8f }, cb[3] = { 0.15f, 0.2f, 0.35f }, cf[3] = { (float)ctr[0], (float)ctr[1], (float)ctr[2] };
	int chk = c.material(ARE_MAT_LAMBERTIAN, c.texture(ARE_TEX_CHECKER, ca, cb, 10.0f, ARE_MAP_SPHERICAL, cf));
	icosphere(c, freq, ctr, 1.0, seed, chk);
	int ground = c.lambertian(0.5f, 0.5f, 0.5f);
	const float g = 20.0f;
	c.tris.insert(c.tris.end(), { -g, 0.f, -g, g, 0.f, g, g, 0.f, -g });
	c.tris.insert(c.tris.end(), { -g, 0.f, -g, -g, 0.f, g, g, 0.f, g });
	c.tri_mat.push_back(ground);
	c.tri_mat.push_back(ground);
	float e[3] = { 12.f, 12.f, 12.f }, k0[3] = { 0.f, 0.f, 0.f };
	c.sphere(3.0, 5.0, 2.0, 1.0, c.material(ARE_MAT_DIFFUSE_LIGHT, c.texture(ARE_TEX_SOLID, k0), 0.f, 1.f, e));
	c.desc.background = ARE_BG_CONSTANT;
	for (int k = 0; k < 3; ++k) c.desc.bg_a[k] = 0.02f;
	c.desc.triangle_test = ARE_TRI_WATERTIGHT;
	set_cam(c.cam, 0.0, 1.6, 4.5, 0.0, 0.9, 0.0, 35, 0.0, 4.5);
	set_params(c.params, 1920, 1080, 256, 16, 1, 1e-4f);
}

// One scene of the uneven batch: `count` spheres on a jittered square grid
// sized to the count (side ceil(sqrt(count)) over 22 units, radius 0.4 of a
// cell), materials drawn as in random_spheres, on the same ground sphere and
// camera; resolution and samples per pixel drawn from the seed.
void sphere_field(are_config &c, uint64_t seed, int count) {
	SplitMix r{ seed * 0x9E3779B97F4A7C15ULL + 17 };
	c.sphere(0, -1000, 0, 1000, c.lambertian(0.5f, 0.5f, 0.5f));
	int side = (int)std::ceil(std::sqrt((double)count));
	double cell = 22.0 / side, rad = 0.4 * cell;
	int placed = 0;
	for (int a = 0; a < side && placed < count; ++a)
		for (int b = 0; b < side && placed < count; ++b, ++placed) {
			double choose = r.u();
			double x = -11.0 + (a + 0.2 + 0.6 * r.u()) * cell, z = -11.0 + (b + 0.2 + 0.6 * r.u()) * cell;
			int m;
			if (choose < 0.8) {
				float alb[3];
				for (int k = 0; k < 3; ++k) alb[k] = (float)r.u();
				for (int k = 0; k < 3; ++k) alb[k] *= (float)r.u();
				m = c.lambertian(alb[0], alb[1], alb[2]);
			} else if (choose < 0.95) {
				float alb[3];
				for (int k = 0; k < 3; ++k) alb[k] = (float)r.u(0.5, 1.0);
				m = c.material(ARE_MAT_METAL, c.texture(ARE_TEX_SOLID, alb), (float)r.u(0.0, 0.5));
			} else {
				float w[3] = { 1.f, 1.f, 1.f };
				m = c.material(ARE_MAT_DIELECTRIC, c.texture(ARE_TEX_SOLID, w), 0.0f, 1.5f);
			}
			c.sphere(x, rad, z, rad, m);
		}
	c.desc.background = ARE_BG_SKY_GRADIENT;
	for (int k = 0; k < 3; ++k) c.desc.bg_a[k] = 1.0f;
	c.desc.bg_b[0] = 0.5f, c.desc.bg_b[1] = 0.7f, c.desc.bg_b[2] = 1.0f;
	c.desc.triangle_test = ARE_TRI_WATERTIGHT;
	set_cam(c.cam, 13, 2, 3, 0, 0, 0, 20, 0.1, 10.0);
	static const int res[3][2] = { { 256, 256 }, { 640, 360 }, { 1280, 720 } };
	static const int spps[3] = { 16, 64, 256 };
	int ri = (int)(r.u() * 3.0), si = (int)(r.u() * 3.0);
	set_params(c.params, res[std::min(ri, 2)][0], res[std::min(ri, 2)][1], spps[std::min(si, 2)], 50, seed, 1e-3f);
}

// rt.cpp's own scene (experiments/rt.cpp:153-185), as data: five wall quads
// and two boxes, each quad split into two triangles with the fixed per-vertex
// uv of pushQuad, every triangle MAT_METAL with reflect_ratio 0.9.
void legacy_rt(are_config &c) {
	float red[3] = { 0.8f, 0.15f, 0.15f }, green[3] = { 0.15f, 0.8f, 0.15f }, white[3] = { 0.8f, 0.8f, 0.8f };
	float ck_a[3] = { 0.9f, 0.9f, 0.9f }, ck_b[3] = { 0.1f, 0.1f, 0.1f }, meta[3] = { 0.93f, 0.95f, 1.0f };
	int t_red = c.texture(ARE_TEX_SOLID, red), t_green = c.texture(ARE_TEX_SOLID, green);
	int t_white = c.texture(ARE_TEX_SOLID, white), t_ck = c.texture(ARE_TEX_CHECKER, ck_a, ck_b, 8.0f);
	int t_meta = c.texture(ARE_TEX_SOLID, meta);
	auto metal = [&](int tex, const float tint[3]) {
		are_material m{};
		m.type = ARE_MAT_METAL;
		m.texture = tex;
		m.reflect_ratio = 0.90f;
		for (int k = 0; k < 3; ++k) m.tint[k] = tint[k];
		c.mats.push_back(m);
		return (int)c.mats.size() - 1;
	};
	float no_tint[3] = { 0, 0, 0 }, box_tint[3] = { 0.92f, 0.94f, 1.0f };
	auto push_quad = [&](const float p[12], int m) {
		const float *v0 = p, *v1 = p + 3, *v2 = p + 6, *v3 = p + 9;
		const float *tri[2][3] = { { v0, v1, v2 }, { v0, v2, v3 } };
		const float uv[2][6] = { { 0, 0, 1, 0, 1, 1 }, { 0, 0, 1, 1, 0, 1 } };
		for (int t = 0; t < 2; ++t) {
			for (int k = 0; k < 3; ++k)
				for (int a = 0; a < 3; ++a) c.tris.push_back(tri[t][k][a]);
			c.tri_uv.insert(c.tri_uv.end(), uv[t], uv[t] + 6);
			c.tri_mat.push_back(m);
		}
	};
	auto quad12 = [&](std::initializer_list<float> l, int m) {
		float p[12];
		std::copy(l.begin(), l.end(), p);
		push_quad(p, m);
	};
	quad12({ -1, -1, -1, -1, 1, -1, -1, 1, 1, -1, -1, 1 }, metal(t_red, no_tint));
	quad12({ 1, -1, 1, 1, 1, 1, 1, 1, -1, 1, -1, -1 }, metal(t_green, no_tint));
	quad12({ -1, -1, 1, 1, -1, 1, 1, -1, -1, -1, -1, -1 }, metal(t_ck, no_tint));
	quad12({ -1, 1, 1, -1, 1, -1, 1, 1, -1, 1, 1, 1 }, metal(t_white, no_tint));
	quad12({ -1, -1, -1, 1, -1, -1, 1, 1, -1, -1, 1, -1 }, metal(t_white, no_tint));
	auto push_box = [&](float cx, float cy, float cz, float r, int m) {
		float X[2] = { cx - r, cx + r }, Y[2] = { cy - r, cy + r }, Z[2] = { cz - r, cz + r };
		quad12({ X[0], Y[0], Z[0], X[1], Y[0], Z[0], X[1], Y[1], Z[0], X[0], Y[1], Z[0] }, m);
		quad12({ X[0], Y[0], Z[1], X[1], Y[0], Z[1], X[1], Y[1], Z[1], X[0], Y[1], Z[1] }, m);
		quad12({ X[0], Y[0], Z[0], X[0], Y[1], Z[0], X[0], Y[1], Z[1], X[0], Y[0], Z[1] }, m);
		quad12({ X[1], Y[0], Z[0], X[1], Y[1], Z[0], X[1], Y[1], Z[1], X[1], Y[0], Z[1] }, m);
		quad12({ X[0], Y[1], Z[0], X[1], Y[1], Z[0], X[1], Y[1], Z[1], X[0], Y[1], Z[1] }, m);
		quad12({ X[0], Y[0], Z[0], X[1], Y[0], Z[0], X[1], Y[0], Z[1], X[0], Y[0], Z[1] }, m);
	};
	push_box(-0.5f, -0.9f, 0.4f, 0.15f, metal(t_white, box_tint));
	push_box(0.0f, -0.9f, 0.4f, 0.10f, metal(t_meta, box_tint));
	c.desc.background = ARE_BG_CONSTANT;
	c.desc.bg_a[0] = 0.06f, c.desc.bg_a[1] = 0.09f, c.desc.bg_a[2] = 0.14f;
	c.desc.triangle_test = ARE_TRI_REFERENCE_MT;
	set_cam(c.cam, 0, 0, 4, 0, 0, 0, 50, 0.0, 1.0);
	set_params(c.params, 512, 512, 1, 2, 1, 1e-5f);
	c.params.estimator = ARE_EST_LEGACY_RT;
	c.params.flags = ARE_FLAG_NO_JITTER | ARE_FLAG_CLAMP_OUTPUT;
	c.params.rr_depth = 0;
}

}  // namespace

are_status config_build(int32_t config, uint64_t seed, int32_t freq, are_config **out) {
	if (!out) {
		set_error("output pointer is null");
		return ARE_ERR_INVALID_ARGUMENT;
	}
	*out = nullptr;
	std::unique_ptr<are_config> c(new (std::nothrow) are_config());
	if (!c) return ARE_ERR_OUT_OF_MEMORY;
	try {
		switch (config) {
		case ARE_CONFIG_RANDOM_SPHERES: random_spheres(*c, seed); break;
		case ARE_CONFIG_CORNELL: cornell(*c, false); break;
		case ARE_CONFIG_CORNELL_OCCLUDED: cornell(*c, true); break;
		case ARE_CONFIG_MESH:
			if (freq < 0 || freq > 2000) {
				set_error("mesh frequency must be in [0, 2000]");
				return ARE_ERR_INVALID_ARGUMENT;
			}
			mesh(*c, seed, freq ? freq : 316);
			break;
		case ARE_CONFIG_LEGACY_RT: legacy_rt(*c); break;
		case ARE_CONFIG_SPHERE_FIELD:
			if (freq < 1 || freq > 4000000) {
				set_error("sphere count must be in [1, 4000000]");
				return ARE_ERR_INVALID_ARGUMENT;
			}
			sphere_field(*c, seed, freq);
			break;
		default: set_error("unknown config " + std::to_string(config)); return ARE_ERR_INVALID_ARGUMENT;
		}
	} catch (const std::bad_alloc &) {
		set_error("out of host memory building config");
		return ARE_ERR_OUT_OF_MEMORY;
	}
	c->finish();
	*out = c.release();
	return ARE_OK;
}

}  // namespace are_core

extern "C" {

ARE_API const are_scene_desc *are_config_desc(const are_config *cfg) { return cfg ? &cfg->desc : nullptr; }

ARE_API are_status are_config_defaults(const are_config *cfg, are_camera *camera, are_render_params *params) {
	if (!cfg) {
		are_core::set_error("null config");
		return ARE_ERR_INVALID_ARGUMENT;
	}
	if (camera) *camera = cfg->cam;
	if (params) *params = cfg->params;
	return ARE_OK;
}

ARE_API void are_config_free(are_config *cfg) { delete cfg; }

}  // extern "C"
