"""The C ABI without a GPU: exports, status strings, descriptor validation,
the synthetic scene generators."""
import ctypes as C

import numpy as np
import pytest

from common import REPO, are


def test_library_exports_every_declared_symbol(lib):
    names = are.exported_symbols()
    assert len(names) >= 13
    for n in names:
        assert hasattr(lib, n), n


def test_header_declares_only_extern_c_are_names():
    import re
    hdr = (REPO / "include" / "aurora_gb300.h").read_text()
    assert 'extern "C"' in hdr
    for n in re.findall(r"ARE_API\s+[\w\s\*]+?\b(\w+)\s*\(", hdr):
        assert n.startswith("are_"), n


def test_status_strings(lib):
    assert lib.are_status_string(0) == b"ok"
    assert lib.are_status_string(1) == b"invalid argument"
    assert lib.are_version() >= 10000


def _create(lib, s):
    d, keep = are.desc_struct(s)
    h = C.c_void_p()
    st = lib.are_scene_create(C.byref(d), C.byref(h))
    if st == 0:
        lib.are_scene_destroy(h)
    return st, lib.are_last_error().decode()


@pytest.mark.parametrize("case", ["null_tri_material", "zero_edge", "collinear", "bad_sphere", "bad_texture",
                                  "bad_image", "bad_mat_type", "degenerate_quad", "bad_bvh_width",
                                  "wide_device_build", "bad_filter", "bad_accel"])
def test_descriptor_validation(lib, case):
    """Mirrors are::Triangle's constructor checks (src/object/triangle.cpp:9-46)
    and are::Texture's size check (src/texture.cpp:52-55); validation runs
    before any device work, so it is testable without a GPU."""
    s = are.SceneArrays()
    m = s.material(are.MAT_LAMBERTIAN, albedo=(0.5, 0.5, 0.5))
    if case == "null_tri_material":
        s.add_triangles([0, 0, 0, 1, 0, 0, 0, 1, 0], 5)
    elif case == "zero_edge":
        s.add_triangles([0, 0, 0, 0, 0, 0, 0, 1, 0], m)
    elif case == "collinear":
        s.add_triangles([0, 0, 0, 1, 0, 0, 2, 0, 0], m)
    elif case == "bad_sphere":
        s.add_spheres([0, 0, 0, -1], m)
    elif case == "bad_texture":
        s.materials["texture"][0] = 9
    elif case == "bad_image":
        s.texture(are.TEX_IMAGE, width=4, height=4, texel_offset=0)
    elif case == "bad_mat_type":
        s.materials["type"][0] = 17
    elif case == "degenerate_quad":
        s.add_quads([0, 0, 0, 1, 0, 0, 2, 0, 0], m)
    elif case == "bad_bvh_width":
        s.bvh_width = 3
    elif case == "wide_device_build":  # the device build's tree is traversed two-wide only
        s.bvh_width, s.bvh_build = 4, are.BVH_DEVICE
    elif case == "bad_accel":
        s.accel = 5
    elif case == "bad_filter":
        s.texels = np.ones((4, 3), np.float32)
        t = s.texture(are.TEX_IMAGE, width=2, height=2, texel_offset=0)
        s.textures["filter"][t] = 7
    st, msg = _create(lib, s)
    assert st == 1, (case, st, msg)
    assert msg


def test_first_bad_triangle_is_reported_in_large_scenes(lib):
    """Above 2^16 triangles the checks run on several threads; the message
    still names the lowest-numbered bad triangle, as a serial scan would."""
    n = 100_000
    base = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32)
    tris = np.tile(base, (n, 1)) + np.repeat(np.arange(n, dtype=np.float32) * 0.01, 9).reshape(n, 9)
    tris[99_999, 4] = np.nan                        # non-finite vertex
    tris[90_000, 3:6] = tris[90_000, 0:3]           # zero edge vector
    tris[41_000, 6:9] = 2 * tris[41_000, 3:6] - tris[41_000, 0:3]  # collinear edges
    s = are.SceneArrays()
    m = s.material(are.MAT_LAMBERTIAN, albedo=(0.5, 0.5, 0.5))
    s.add_triangles(tris.reshape(-1), m)
    st, msg = _create(lib, s)
    assert st == 1 and "triangle 41000" in msg and "collinear" in msg, (st, msg)


def test_scene_create_without_device_is_an_error(lib):
    if lib.are_device_count() > 0:
        pytest.skip("a device is present")
    s, _, _ = are.build_config(are.CONFIG_CORNELL)
    st, msg = _create(lib, s)
    assert st == 4 and "device" in msg


def test_render_rejects_bad_arguments_before_device_work(lib):
    cam = are.Camera()
    p = are.RenderParams()
    st = lib.are_render(None, C.byref(cam), C.byref(p), None, None, None)
    assert st == 1


@pytest.mark.parametrize("cfg,n_prims", [(are.CONFIG_RANDOM_SPHERES, 488), (are.CONFIG_CORNELL, 18),
                                         (are.CONFIG_CORNELL_OCCLUDED, 19), (are.CONFIG_LEGACY_RT, 34)])
def test_configs_are_deterministic(cfg, n_prims):
    a, cam, par = are.build_config(cfg, seed=42)
    b, _, _ = are.build_config(cfg, seed=42)
    assert a.n_prims == n_prims
    for k in ("spheres", "quads", "triangles"):
        assert np.array_equal(getattr(a, k), getattr(b, k))
    assert np.array_equal(a.materials, b.materials)


def test_random_spheres_distribution():
    s, cam, par = are.build_config(are.CONFIG_RANDOM_SPHERES, seed=42)
    assert (par["width"], par["height"], par["spp"], par["max_depth"]) == (400, 225, 32, 50)
    assert cam["vfov_deg"] == 20 and abs(cam["aperture"] - 0.1) < 1e-7 and cam["focus_dist"] == 10
    small = s.spheres[1:485]
    assert np.all(small[:, 3] == np.float32(0.2)) and np.all(small[:, 1] == np.float32(0.2))
    t = s.materials["type"][s.sphere_mat[1:485]]
    frac = [(t == k).mean() for k in (0, 1, 2)]
    assert abs(frac[0] - 0.8) < 0.06 and abs(frac[1] - 0.15) < 0.05 and abs(frac[2] - 0.05) < 0.03
    fuzz = s.materials["fuzz"][s.sphere_mat[1:485]][t == 1]
    assert fuzz.min() >= 0 and fuzz.max() <= 0.5


def test_cornell_geometry():
    s, cam, par = are.build_config(are.CONFIG_CORNELL)
    assert (par["width"], par["height"], par["spp"], par["max_depth"]) == (600, 600, 1024, 50)
    light = s.materials["type"] == are.MAT_DIFFUSE_LIGHT
    lq = s.quads[light[s.quad_mat]]
    assert len(lq) == 1
    n = np.cross(lq[0, 3:6], lq[0, 6:9])
    assert n[1] < 0 and abs(np.linalg.norm(n) - 130 * 105) < 1e-3  # faces down, 130 x 105
    assert np.all(s.materials["emit"][light] == 15)


def test_mesh_triangle_count_and_watertight_edges():
    s, cam, par = are.build_config(are.CONFIG_MESH, mesh_frequency=9)
    assert len(s.triangles) == 20 * 81 + 2
    # every interior edge of the displaced icosphere is shared by exactly two triangles
    tri = s.triangles[:-2].reshape(-1, 3, 3)
    keys = {}
    for t in tri:
        vs = [tuple(v) for v in t]
        for a, b in ((0, 1), (1, 2), (2, 0)):
            e = tuple(sorted((vs[a], vs[b])))
            keys[e] = keys.get(e, 0) + 1
    assert set(keys.values()) == {2}
    assert s.triangle_test == are.TRI_WATERTIGHT


def test_ctypes_structs_match_the_header():
    """Every C struct of include/aurora_gb300.h has the size its ctypes mirror
    assumes (a mismatch lets the library write past the Python object)."""
    import subprocess
    import tempfile
    from pathlib import Path
    structs = {"are_material": are.MATERIAL_DTYPE.itemsize, "are_texture": are.TEXTURE_DTYPE.itemsize,
               "are_scene_desc": C.sizeof(are.SceneDesc), "are_camera": C.sizeof(are.Camera),
               "are_render_params": C.sizeof(are.RenderParams), "are_render_stats": C.sizeof(are.RenderStats),
               "are_guide_params": C.sizeof(are.GuideParams), "are_batch_options": C.sizeof(are.BatchOptions)}
    src = '#include "aurora_gb300.h"\n#include <stdio.h>\nint main(void){\n' + "".join(
        f'printf("%zu\\n", sizeof({k}));\n' for k in structs) + "return 0;}\n"
    with tempfile.TemporaryDirectory() as td:
        c = Path(td) / "s.c"
        c.write_text(src)
        exe = Path(td) / "s"
        subprocess.run(["gcc", "-I", str(REPO / "include"), str(c), "-o", str(exe)], check=True)
        sizes = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert dict(zip(structs, sizes)) == structs


def test_reference_arm_scene_files_match_the_builder(lib):
    """The benchmark's reference arm reads its scenes from oracle/scenes/*.npz
    (so it never loads the CUDA core); they must be the scenes the core's
    builder makes, array for array."""
    from oracle.scenes import load
    for name, cfg in (("cornell_box", are.CONFIG_CORNELL), ("random_spheres", are.CONFIG_RANDOM_SPHERES)):
        s, cam, par = load(name)
        ref, rcam, rpar = are.build_config(cfg)
        assert cam == rcam and par == rpar
        for k in ("spheres", "sphere_mat", "quads", "quad_mat", "triangles", "triangle_mat"):
            assert np.array_equal(getattr(s, k), getattr(ref, k)), (name, k)
        assert s.materials.tobytes() == ref.materials.tobytes() and s.textures.tobytes() == ref.textures.tobytes()
        assert (s.background, s.bg_a, s.bg_b, s.triangle_test) == (ref.background, tuple(ref.bg_a), tuple(ref.bg_b),
                                                                    ref.triangle_test)
