"""The adapter from the reference library's scene container
(include/aurora_gb300_are.hpp).  A program built against the reference's own
headers and sources (compiled into oracle/_ref) fills an are::ObjectSet with
are::Triangles, the adapter turns it into the core's scene descriptor, and
the descriptor holds the reference's vertices Q, Q + u, Q + v
(src/object/triangle.cpp:41-45) rounded to float, with the materials the
caller assigned; a null triangle is refused.  Runs where the reference tree
is present; skipped elsewhere (the GPU hosts have no reference tree)."""
import subprocess

import numpy as np
import pytest

from common import REPO
from oracle.build import REF_OUT, REF_ROOT

pytestmark = pytest.mark.skipif(
    not (REF_ROOT / "include" / "object" / "object_set.h").exists() or not (REF_OUT / "libref_lib.so").exists(),
    reason="reference tree or its compiled library (oracle/_ref) not present")

TRIS = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0],
                 [0.1, 0.2, 0.3, 0.7, -0.3, 0.05, -0.2, 0.9, 1.0 / 3.0],
                 [278.0, 554.0, 332.0, -130.0, 0.0, 0.0, 0.0, 0.0, -105.0]], np.float64)

PROGRAM = r"""
#include <material/diffuse.h>

#include <cstdio>

#include "aurora_gb300_are.hpp"

int main() {
	are::Diffuse mat;
	are::Texture tex(2, 2, are::Color3(0.5, 0.5, 0.5));
	are::ObjectSet set;
	const double q[3][9] = { %s };
	for (const auto &t : q)
		set.triangles.push_back(new are::Triangle(are::Point3(t[0], t[1], t[2]), are::Vec3(t[3], t[4], t[5]),
			are::Vec3(t[6], t[7], t[8]), &mat, &tex));
	are_gb300::SceneBuilder b;
	const int white = b.lambertian(b.solid(.73f, .73f, .73f)), red = b.lambertian(b.solid(.65f, .05f, .05f));
	int k = 0;
	const int n = are_gb300::add_object_set(b, set, [&](const are::Triangle &) { return (k++ %% 2) ? red : white; });
	const are_scene_desc d = b.desc();
	std::printf("%%d %%d\n", n, d.n_triangles);
	for (int i = 0; i < 9 * d.n_triangles; ++i) std::printf("%%a\n", (double)d.triangles[i]);
	for (int i = 0; i < d.n_triangles; ++i) std::printf("%%d\n", d.triangle_mat[i]);
	set.triangles.push_back(nullptr);
	try {
		are_gb300::add_object_set(b, set, white);
		std::printf("accepted\n");
	} catch (const are_gb300::Error &e) {
		std::printf("refused %%d %%d\n", (int)e.status, b.desc().n_triangles);
	}
	for (auto *t : set.triangles) delete t;
	return 0;
}
"""


def test_object_set_to_scene_descriptor(tmp_path):
    src = tmp_path / "adapter.cpp"
    src.write_text(PROGRAM % ", ".join("{ " + ", ".join(repr(float(x)) for x in t) + " }" for t in TRIS))
    exe = tmp_path / "adapter"
    subprocess.run(["g++", "-std=c++20", "-O1", "-Wall", "-Werror", "-I", str(REF_ROOT / "include"), "-I",
                    str(REPO / "include"), str(src), "-o", str(exe), str(REF_OUT / "libref_lib.so"),
                    f"-Wl,-rpath,{REF_OUT}"], check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    n, nt = map(int, out[0].split())
    assert n == nt == len(TRIS)
    got = np.array([float.fromhex(x) for x in out[1:1 + 9 * nt]], np.float64).reshape(nt, 9)
    Q, u, v = TRIS[:, 0:3], TRIS[:, 3:6], TRIS[:, 6:9]
    want = np.concatenate([Q, Q + u, Q + v], 1).astype(np.float32).astype(np.float64)  # FP64 sums, rounded once
    assert np.array_equal(got, want)
    mats = [int(x) for x in out[1 + 9 * nt:1 + 10 * nt]]
    assert mats == [0, 1, 0]  # white, red, white: the caller's mapping, in the set's order
    assert out[1 + 10 * nt] == f"refused 1 {nt}"  # ARE_ERR_INVALID_ARGUMENT, nothing added


def test_trace_texture_definition_compiles(tmp_path):
    """The opt-in definition of the member the reference declares but never
    defines compiles against the reference's headers."""
    src = tmp_path / "stub.cpp"
    src.write_text('#define ARE_GB300_DEFINE_TRACE_TEXTURE\n#include "aurora_gb300_are.hpp"\n')
    subprocess.run(["g++", "-std=c++20", "-Wall", "-Werror", "-c", "-I", str(REF_ROOT / "include"), "-I",
                    str(REPO / "include"), str(src), "-o", str(tmp_path / "stub.o")], check=True, capture_output=True,
                   text=True)


def test_bound_object_set_with_materials_and_textures(tmp_path):
    """add_object_set_bound: each triangle's are::Material and are::Texture
    (which are::Triangle keeps private, so the caller names them) become core
    materials and image textures — texels read through are::Texture::pixel,
    are::Reflective(0.8) a metal of reflect_ratio 0.8, are::Diffuse
    lambertian — and the result is the committed fixture the GPU test renders
    (tests/golden/are_adapted_scene.npz)."""
    from tests.golden.make_adapted_scene import build_and_run, read
    from common import GOLDEN, are
    out = tmp_path / "scene.bin"
    log = build_and_run(out, tmp_path)
    assert log.startswith("18 triangles, 5 textures, 5 materials")
    d = read(out)
    z = np.load(GOLDEN / "are_adapted_scene.npz")
    for k in ("triangles", "triangle_uv", "triangle_mat", "texels"):
        assert np.array_equal(d[k], z[k]), k
    assert d["materials"].tobytes() == z["materials"].tobytes() and d["textures"].tobytes() == z["textures"].tobytes()
    assert np.array_equal(d["triangle_uv"], np.tile([0, 0, 1, 0, 0, 1], (18, 1)).astype(np.float32))
    # the floor's checker, texel (x, y) = pixel(x, y), row-major from the top
    t0 = d["textures"][d["materials"][d["triangle_mat"][0]]["texture"]]
    assert (t0["type"], t0["width"], t0["height"]) == (are.TEX_IMAGE, 8, 8)
    tex = d["texels"][t0["texel_offset"]:t0["texel_offset"] + 64].reshape(8, 8, 3)
    for y in range(8):
        for x in range(8):
            want = (0.1, 0.2, 0.6) if (x + y) % 2 else (0.9, 0.9, 0.9)
            assert np.array_equal(tex[y, x], np.float32(want)), (x, y)
    kinds = sorted((int(m["type"]), round(float(m["reflect_ratio"]), 6)) for m in d["materials"])
    assert kinds == [(are.MAT_LAMBERTIAN, 1.0)] * 4 + [(are.MAT_METAL, 0.8)]
