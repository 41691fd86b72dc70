"""Pin the oracle to the reference (CPU only).

Where oracle/_ref exists (built from the reference's own sources), the oracle
is compared with the reference directly; everywhere, it is compared with the
committed fixtures that tests/golden/make_golden.py recorded from the
reference.  Bit-exact for closest-hit ids, t, u, v and texture/frame values.
"""
import numpy as np
import pytest

from common import GOLDEN, REF_T_MAX, REF_T_MIN, are, hit_ids, legacy_scene_from_export, random_rays
from oracle.orc import RefLib, RefRT

needs_ref = pytest.mark.skipif(not RefRT.available(), reason="reference tree not built here (oracle/_ref)")


def rays8(r6, t_min=REF_T_MIN, t_max=REF_T_MAX):
    r = np.empty((len(r6), 8), np.float32)
    r[:, 0:3], r[:, 3], r[:, 4:7], r[:, 7] = r6[:, 0:3], t_min, r6[:, 3:6], t_max
    return r


def same_hits(a, b):
    """Reference misses are (t=1e30, -1); the oracle's are (inf, -1)."""
    ia, ib = hit_ids(a), hit_ids(b)
    assert np.array_equal(ia, ib), f"{(ia != ib).sum()} id mismatches"
    m = ia >= 0
    assert np.array_equal(a[m][:, [0, 2, 3]].view(np.uint32), b[m][:, [0, 2, 3]].view(np.uint32))


@pytest.fixture(scope="module")
def rt_scene():
    return legacy_scene_from_export(np.load(GOLDEN / "rt_scene.npy"))


def test_golden_scene_matches_config(lib):
    """The library's built-in copy of rt.cpp's scene equals the reference's."""
    exp = np.load(GOLDEN / "rt_scene.npy")
    s, cam, par = are.build_config(are.CONFIG_LEGACY_RT)
    assert np.array_equal(s.triangles, exp[:, 0:9])
    assert np.array_equal(s.triangle_uv, exp[:, 9:15])
    m = s.materials[s.triangle_mat]
    assert np.all(m["type"] == are.MAT_METAL) and np.all(exp[:, 15] == 1)
    assert np.array_equal(m["reflect_ratio"], exp[:, 16]) and np.array_equal(m["tint"], exp[:, 17:20])
    t = s.textures[m["texture"]]
    assert np.array_equal(t["type"], exp[:, 20].astype(np.int32))
    assert np.array_equal(t["a"], exp[:, 21:24])
    ck = t["type"] == are.TEX_CHECKER
    assert np.array_equal(t["b"][ck], exp[ck, 24:27]) and np.all(t["scale"][ck] == exp[ck, 27])
    assert cam["lookfrom"] == [0, 0, 4] and cam["vfov_deg"] == 50 and par["width"] == 512


def test_intersect_matches_golden(oracle, rt_scene):
    g = np.load(GOLDEN / "rt_intersect.npz")
    ctx = oracle.prepare(rt_scene, accel=0)
    same_hits(g["hits"], oracle.intersect(ctx, rays8(g["rays6"])))


def test_documented_tie_break(oracle, rt_scene):
    """(0,0,4) -> (0,0,-1) hits the back wall's shared diagonal: the first
    triangle (id 8) wins at t = 5 with u = 0, v = 0.5 (rt.cpp:213)."""
    ctx = oracle.prepare(rt_scene, accel=0)
    h = oracle.intersect(ctx, rays8(np.array([[0, 0, 4, 0, 0, -1]], np.float32)))
    assert hit_ids(h)[0] == 8 and h[0, 0] == 5.0 and h[0, 2] == 0.0 and h[0, 3] == 0.5


def test_soups_match_golden(oracle):
    g = np.load(GOLDEN / "rt_soup.npz")
    for k in range(8):
        s = are.SceneArrays()
        s.triangle_test = are.TRI_REFERENCE_MT
        s.material()
        s.add_triangles(g[f"tris{k}"], 0)
        ctx = oracle.prepare(s, accel=0)
        same_hits(g[f"hits{k}"], oracle.intersect(ctx, rays8(g[f"rays{k}"])))


@needs_ref
def test_intersect_10m_rays_against_reference(oracle, rt_scene, nthreads):
    """10M seeded rays: oracle closest hit == the reference's intersect()."""
    ref = RefRT()
    ctx = oracle.prepare(rt_scene, accel=0)
    for chunk in range(5):
        r = random_rays(2_000_000, 10_000 + chunk)
        h_ref = ref.intersect(np.concatenate([r[:, 0:3], r[:, 4:7]], 1))
        same_hits(h_ref, oracle.intersect(ctx, r, nthreads))


def test_oracle_bvh_equals_linear(oracle, lib, nthreads):
    """The oracle's own BVH returns the linear scan's answer (smallest t,
    lower id on ties) on every workload scene."""
    for cfg, kw in [(are.CONFIG_RANDOM_SPHERES, dict(lo=-12, hi=12, t_min=1e-3, camera=(13, 2, 3))),
                    (are.CONFIG_CORNELL, dict(lo=0, hi=555, t_min=1e-3, camera=(278, 278, -800))),
                    (are.CONFIG_CORNELL_OCCLUDED, dict(lo=0, hi=555, t_min=1e-3, camera=(278, 278, -800))),
                    (are.CONFIG_MESH, dict(lo=-1.5, hi=2.5, t_min=1e-4, camera=(0, 1.6, 4.5)))]:
        s, _, _ = are.build_config(cfg, mesh_frequency=12)
        r = random_rays(100_000, 5 + cfg, t_max=np.inf, **kw)
        a = oracle.intersect(oracle.prepare(s, accel=0), r, nthreads)
        b = oracle.intersect(oracle.prepare(s, accel=1), r, nthreads)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), cfg


def test_checker_and_frame_match_golden(oracle):
    g = np.load(GOLDEN / "rt_kat.npz")
    s = are.SceneArrays()
    s.texture(are.TEX_CHECKER, a=g["checker_a"], b=g["checker_b"], scale=float(g["checker_scale"]))
    ctx = oracle.prepare(s, accel=0)
    import ctypes as C
    f = C.POINTER(C.c_float)
    out = np.zeros(3, np.float32)
    p = np.zeros(3, np.float32)
    for (u, v), want in zip(g["checker_uv"], g["checker_out"]):
        oracle.lib.orc_texture_eval_f32(ctx.h, 0, float(u), float(v), p.ctypes.data_as(f), out.ctypes.data_as(f))
        assert np.array_equal(out, want), (u, v)
    for n, (u, v), want in zip(g["hemi_n"], g["hemi_uv"], g["hemi_out"]):
        n = np.ascontiguousarray(n)
        oracle.lib.orc_hemisphere_f32(n.ctypes.data_as(f), float(u), float(v), out.ctypes.data_as(f))
        assert np.array_equal(out, want), (n, u, v)


def test_ppm_quantisation_matches_golden(oracle):
    import ctypes as C
    g = np.load(GOLDEN / "rt_kat.npz")
    img = np.ascontiguousarray(g["ppm_img"].reshape(-1))
    out = np.zeros(img.size, np.uint8)
    oracle.lib.orc_ppm_quantize(img.ctypes.data_as(C.POINTER(C.c_float)), img.size, 2.2,
                                out.ctypes.data_as(C.POINTER(C.c_uint8)))
    ppm = g["ppm_bytes"]
    header = b"P6\n5 7\n255\n"
    assert bytes(ppm[:len(header)]) == header
    assert np.array_equal(ppm[len(header):], out)


def test_reflect_refract_match_golden(oracle):
    import ctypes as C
    g = np.load(GOLDEN / "lib_kat.npz")
    d = C.POINTER(C.c_double)
    o = np.zeros(3)
    for v, n, eta, rf, rr in zip(g["v"], g["n"], g["eta"], g["reflect"], g["refract"]):
        v, n = np.ascontiguousarray(v), np.ascontiguousarray(n)
        oracle.lib.orc_reflect_f64(v.ctypes.data_as(d), n.ctypes.data_as(d), o.ctypes.data_as(d))
        assert np.allclose(o, rf, rtol=0, atol=1e-15)
        oracle.lib.orc_refract_f64(v.ctypes.data_as(d), n.ctypes.data_as(d), float(eta), o.ctypes.data_as(d))
        assert np.allclose(o, rr, rtol=0, atol=1e-14, equal_nan=True)


@pytest.mark.skipif(not RefLib.available(), reason="reference library not built here (oracle/_ref)")
def test_reference_library_fixtures_reproduce():
    """The fixtures recorded from the reference library reproduce when the
    library is rebuilt (guards the fixtures themselves)."""
    import ctypes as C
    g = np.load(GOLDEN / "lib_kat.npz")
    lib = RefLib()
    d = C.POINTER(C.c_double)
    hits = np.zeros((len(g["rays"]), 4))
    tris, rays = np.ascontiguousarray(g["tris"]), np.ascontiguousarray(g["rays"])
    lib.lib.ref_lib_triangles_intersect(tris.ctypes.data_as(d), len(tris), rays.ctypes.data_as(d), len(rays),
                                        hits.ctypes.data_as(d))
    assert np.array_equal(hits, g["hits"])


def test_mt19937_known_answer(oracle):
    """std::mt19937 default-seeded: the 10000th output is 4123659995 ([rand.predef])."""
    import ctypes as C
    out = np.zeros(10000, np.uint32)
    can = np.zeros(10000, np.float32)
    oracle.lib.orc_mt19937(5489, 10000, out.ctypes.data_as(C.POINTER(C.c_uint32)),
                           can.ctypes.data_as(C.POINTER(C.c_float)))
    assert out[-1] == 4123659995
    assert np.array_equal(can, np.minimum(out.astype(np.float32) / np.float32(2 ** 32), np.nextafter(np.float32(1), 0)))


def test_reference_estimator_matches_reference_render(oracle):
    """rt.cpp's whole estimator (trace + computeAO + per-row mt19937, rt.cpp:221-374)
    restated in the oracle reproduces the reference's render bit for bit."""
    from oracle.orc import render_legacy
    g = np.load(GOLDEN / "rt_render.npz")
    s, cam, par = are.build_config(are.CONFIG_LEGACY_RT)
    par = dict(par, width=int(g["width"]), height=int(g["height"]))
    img = render_legacy(oracle, oracle.prepare(s, accel=0), cam, par, rng_mode=1, mt_seed=int(g["seed"]))
    diff = img != g["rgb"]
    # transcendental functions of another libm may differ by an ulp: allow a handful of pixels
    assert diff.mean() < 0.002, diff.mean()
    assert np.abs(img - g["rgb"]).max() < 0.05


@needs_ref
def test_reference_estimator_full_frame_bitexact(oracle):
    from oracle.orc import render_legacy
    ref = RefRT().render(3, 512, 512)
    s, cam, par = are.build_config(are.CONFIG_LEGACY_RT)
    img = render_legacy(oracle, oracle.prepare(s, accel=0), cam, par, rng_mode=1, mt_seed=3)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))


def test_oracle_estimator_matches_the_references_committed_render(oracle):
    """The oracle's restatement of rt.cpp's estimator against
    experiments/out_diffuse.ppm, the reference's own committed render (its
    seed unknown, so 32x32-pixel block means within 1.5 levels)."""
    from oracle.orc import render_legacy
    g = np.load(GOLDEN / "rt_out_diffuse.npz")
    s, cam, par = are.build_config(are.CONFIG_LEGACY_RT)
    img = render_legacy(oracle, oracle.prepare(s, accel=0), cam, par, rng_mode=1, mt_seed=11)
    q = oracle.quantize(img, 0, 2.2).reshape(int(g["height"]), int(g["width"]), 3).astype(np.float64)
    b = int(g["block"])
    d = np.abs(q.reshape(q.shape[0] // b, b, q.shape[1] // b, b, 3).mean((1, 3)) - g["means"])
    assert d.max() < 1.5 and d.mean() < 0.2, (d.max(), d.mean())
