"""Image files of the reference's output step, host side: the PPM writer
(experiments/rt.cpp:377-392, src/texture.cpp:362-395) against the golden
bytes of the reference's own writePPM, the PPM reader of
src/texture.cpp:9-50, and the FP32 PFM writer.  No GPU needed."""
import numpy as np
import pytest

from common import GOLDEN, are


def test_ppm_bytes_match_reference_writeppm(lib, oracle, tmp_path):
    g = np.load(GOLDEN / "rt_kat.npz")
    img = g["ppm_img"]  # (h, w, 3) written by rt.cpp writePPM
    rgb8 = oracle.quantize(img, 0, 2.2)
    p = tmp_path / "o.ppm"
    are.write_ppm(p, rgb8)
    assert p.read_bytes() == bytes(g["ppm_bytes"])


def test_texture_quantisation_matches_save_texture_formula(oracle):
    v = np.array([-1.0, -0.0, 0.0, 1 / 255, 0.5, 254.9999 / 255, 1.0, 2.0, np.inf, -np.inf, np.nan], np.float32)
    q = oracle.quantize(v, 1)
    d = np.where(np.isnan(v), 0.0, v.astype(np.float64))
    ref = np.clip(d * 255.0, 0, 255).astype(np.uint8)
    assert np.array_equal(q, ref)


def test_ppm_read_back(lib, tmp_path):
    rng = np.random.default_rng(3)
    rgb8 = rng.integers(0, 256, (9, 13, 3), dtype=np.uint8)
    p = tmp_path / "t.ppm"
    are.write_ppm(p, rgb8)
    tex = are.read_ppm(p)
    assert tex.shape == (9, 13, 3)
    assert np.array_equal(tex, (rgb8.astype(np.float64) / 255.0).astype(np.float32))


def test_ppm_reader_rejects_what_the_reference_rejects(lib, tmp_path):
    bad_magic = tmp_path / "a.ppm"
    bad_magic.write_bytes(b"P3\n1 1\n255\n\x00\x00\x00")
    bad_max = tmp_path / "b.ppm"
    bad_max.write_bytes(b"P6\n1 1\n65535\n\x00\x00\x00\x00\x00\x00")
    short = tmp_path / "c.ppm"
    short.write_bytes(b"P6\n2 2\n255\n\x00\x00\x00")
    for p, status in ((bad_magic, 1), (bad_max, 1), (short, 7), (tmp_path / "missing.ppm", 7)):
        with pytest.raises(are.AreError) as e:
            are.read_ppm(p)
        assert e.value.status == status, (p, e.value)


def test_pfm_layout(lib, tmp_path):
    rng = np.random.default_rng(4)
    img = rng.random((5, 7, 3), dtype=np.float32)
    p = tmp_path / "o.pfm"
    are.write_pfm(p, img)
    data = p.read_bytes()
    header = b"PF\n7 5\n-1.0\n"
    assert data[:len(header)] == header
    body = np.frombuffer(data[len(header):], "<f4").reshape(5, 7, 3)
    assert np.array_equal(body[::-1], img)  # bottom row first


def test_writers_reject_bad_arguments(lib, tmp_path):
    with pytest.raises(are.AreError):
        are.write_ppm(tmp_path / "no_such_dir" / "x.ppm", np.zeros((1, 1, 3), np.uint8))
    L = are.load()
    assert L.are_write_ppm(b"x.ppm", None, 1, 1) == 1
    assert L.are_write_pfm(b"x.pfm", None, 0, 1) == 1


def test_cpp_header_compiles_cleanly(tmp_path):
    import shutil
    import subprocess

    from common import REPO

    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    src = tmp_path / "use.cpp"
    src.write_text('#include "aurora_gb300.hpp"\nint main() { are_gb300::SceneBuilder b; '
                   'int m = b.lambertian(b.solid(1, 1, 1)); b.sphere({0, 0, 0}, 1, m); '
                   'return b.desc().n_spheres == 1 ? 0 : 1; }\n')
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", str(REPO / "include"),
                        str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_cli_usage(lib):
    import subprocess

    cli = are.LIB_PATH.parent / "are_render"
    assert cli.exists(), "build() makes the command-line renderer"
    r = subprocess.run([str(cli), "--config", "nonsense"], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
