"""The drop-in binding of INTEGRATION.md, compiled against the reference's
own program.

tests/harness/rt_dropin.cpp includes experiments/rt.cpp from the reference
tree with its render() (rt.cpp:337-374) renamed, and puts in its place the
render() body that INTEGRATION.md shows a maintainer (extracted from the
document here, so the document is what gets compiled).  Two links:

* against tests/harness/abi_recorder.cpp, which records what the binding hands
  to the C ABI: the descriptor must be the one the GPU parity tests render
  for rt.cpp's scene (the same triangles, uv, materials and textures; the
  reference's MT triangle test and background), with rt.cpp's camera and the
  legacy estimator's parameters;
* against the CUDA core's libaurora_gb300.so: the reference's program links
  and runs through the library (without a GPU, are_scene_create reports that
  no device is present and the program still writes its image).

Needs the reference tree (it is not copied into this repository), so it is
skipped where the tree is absent.
"""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from common import GOLDEN, REPO, are, legacy_scene_from_export
from oracle.build import REF_ROOT

RT_CPP = REF_ROOT / "experiments" / "rt.cpp"
pytestmark = pytest.mark.skipif(not RT_CPP.exists() or not shutil.which("g++"), reason="reference tree or g++ absent")


def integration_render_body() -> str:
    text = (REPO / "INTEGRATION.md").read_text()
    blocks = re.findall(r"```cpp\n(.*?)```", text, flags=re.S)
    body = [b for b in blocks if "void render(const Scene &scene" in b]
    assert body, "INTEGRATION.md has no render() binding block"
    return body[0]


@pytest.fixture(scope="module")
def built(tmp_path_factory):
    d = tmp_path_factory.mktemp("dropin")
    inc = d / "render_body.inc"
    inc.write_text(integration_render_body())
    common = ["g++", "-std=c++20", "-O1", "-w", f"-DRT_DROPIN_RENDER=\"{inc}\"", "-I", str(REF_ROOT),
              "-I", str(REPO / "include"), str(REPO / "tests" / "harness" / "rt_dropin.cpp")]
    rec = d / "rt_dropin_record"
    r = subprocess.run(common + [str(REPO / "tests" / "harness" / "abi_recorder.cpp"), "-o", str(rec)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    lib = are.LIB_PATH
    core = d / "rt_dropin_core"
    r = subprocess.run(common + ["-L", str(lib.parent), "-laurora_gb300", f"-Wl,-rpath,{lib.parent}", "-o", str(core)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return d, rec, core


def read_record(path):
    b = path.read_bytes()
    off = 0

    def take(dtype, count):
        nonlocal off
        a = np.frombuffer(b, dtype=dtype, count=count, offset=off)
        off += a.nbytes
        return a

    n = int(take(np.int32, 1)[0])
    rec = {"triangles": take(np.float32, 9 * n).reshape(n, 9), "uv": take(np.float32, 6 * n).reshape(n, 6),
           "triangle_mat": take(np.int32, n)}
    nm = int(take(np.int32, 1)[0])
    rec["materials"] = take(are.MATERIAL_DTYPE, nm)
    nt = int(take(np.int32, 1)[0])
    rec["textures"] = take(are.TEXTURE_DTYPE, nt)
    rec["background"] = int(take(np.int32, 1)[0])
    rec["bg_a"] = take(np.float32, 3)
    rec["triangle_test"] = int(take(np.int32, 1)[0])
    cam = are.Camera.from_buffer_copy(b[off:off + C_sizeof(are.Camera)])
    off += C_sizeof(are.Camera)
    par = are.RenderParams.from_buffer_copy(b[off:off + C_sizeof(are.RenderParams)])
    return rec, cam.to_dict(), par.to_dict()


def C_sizeof(t):
    import ctypes
    return ctypes.sizeof(t)


def per_triangle(mats, texs, mat_idx):
    """(material type, reflect ratio, tint, texture type, a, b, scale) of each triangle."""
    out = []
    for m in mat_idx:
        mt = mats[m]
        t = texs[mt["texture"]]
        out.append((int(mt["type"]), float(mt["reflect_ratio"]), tuple(np.round(mt["tint"], 6)), int(t["type"]),
                    tuple(np.round(t["a"], 6)), tuple(np.round(t["b"], 6)),
                    float(t["scale"]) if int(t["type"]) == are.TEX_CHECKER else 0.0))
    return out


def test_binding_hands_the_tested_scene_to_the_core(built):
    d, rec_bin, _ = built
    path = d / "record.bin"
    r = subprocess.run([str(rec_bin), str(d / "rec.ppm"), "64", "48"], capture_output=True, text=True,
                       env=dict(os.environ, ARE_RECORD_PATH=str(path)))
    assert r.returncode == 0, r.stderr
    rec, cam, par = read_record(path)
    # the scene the GPU tests render for rt.cpp's estimator (tests/test_gpu_legacy.py)
    ref = legacy_scene_from_export(np.load(GOLDEN / "rt_scene.npy"))
    assert np.array_equal(rec["triangles"], ref.triangles)
    assert np.array_equal(rec["uv"], ref.triangle_uv)
    assert per_triangle(rec["materials"], rec["textures"], rec["triangle_mat"]) == \
        per_triangle(ref.materials, ref.textures, ref.triangle_mat)
    assert rec["background"] == are.BG_CONSTANT and np.allclose(rec["bg_a"], (0.06, 0.09, 0.14))
    assert rec["triangle_test"] == are.TRI_REFERENCE_MT
    # rt.cpp's camera (rt.cpp:399) and the legacy estimator's parameters
    _, lcam, lpar = are.build_config(are.CONFIG_LEGACY_RT)
    for k in ("lookfrom", "lookat", "vup"):
        assert np.allclose(cam[k], lcam[k])
    assert cam["vfov_deg"] == lcam["vfov_deg"] and cam["aperture"] == 0.0
    assert (par["width"], par["height"], par["spp"]) == (64, 48, 1)
    assert par["estimator"] == are.EST_LEGACY_RT and par["max_depth"] == lpar["max_depth"]
    assert par["t_min"] == lpar["t_min"]
    assert par["flags"] == lpar["flags"] | are.FLAG_LEGACY_MT19937


def test_reference_program_links_and_runs_through_the_core(built):
    d, _, core = built
    out = d / "core.ppm"
    r = subprocess.run([str(core), str(out), "32", "24"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert out.exists() and out.read_bytes().startswith(b"P6")
    if are.load().are_device_count() == 0:
        assert "no CUDA device" in r.stderr
