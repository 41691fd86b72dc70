"""Closest-hit parity on the GPU: the CUDA core through the C ABI
(are_intersect) against the oracle and the reference's recorded hits.
Bit-exact: primitive id, t, u and v."""
import numpy as np
import pytest

from common import GOLDEN, REF_T_MAX, REF_T_MIN, are, hit_ids, legacy_scene_from_export, random_rays

pytestmark = pytest.mark.gpu


def rays8(r6, t_min=REF_T_MIN, t_max=REF_T_MAX):
    r = np.empty((len(r6), 8), np.float32)
    r[:, 0:3], r[:, 3], r[:, 4:7], r[:, 7] = r6[:, 0:3], t_min, r6[:, 3:6], t_max
    return r


def assert_bitexact(a, b, what=""):
    ia, ib = hit_ids(a), hit_ids(b)
    bad = np.nonzero(ia != ib)[0]
    assert len(bad) == 0, f"{what}: {len(bad)} id mismatches, first {bad[:5]}: {a[bad[:3]]} vs {b[bad[:3]]}"
    m = ia >= 0
    assert np.array_equal(a[m][:, [0, 2, 3]].view(np.uint32), b[m][:, [0, 2, 3]].view(np.uint32)), what
    assert np.all(np.isinf(a[~m][:, 0])) and np.all(np.isinf(b[~m][:, 0]))


def ref_to_core(h):
    """The reference reports misses as t = 1e30 (rt.cpp:205); the core as +inf."""
    h = h.copy()
    h[hit_ids(h) < 0, 0] = np.inf
    h[hit_ids(h) < 0, 2:] = 0
    return h


def test_reference_scene_matches_reference_hits(gpu_lib):
    """rt.cpp's own scene: the GPU's Möller–Trumbore closest hit equals the
    hits recorded from the reference's intersect(), including the
    first-index tie on the back wall's diagonal."""
    g = np.load(GOLDEN / "rt_intersect.npz")
    sc = are.Scene(legacy_scene_from_export(np.load(GOLDEN / "rt_scene.npy")))
    h, ms = sc.intersect(rays8(g["rays6"]))
    assert_bitexact(ref_to_core(g["hits"]), h, "rt.cpp scene")
    assert hit_ids(h)[0] == 8 and h[0, 0] == 5.0


def test_reference_soups(gpu_lib):
    g = np.load(GOLDEN / "rt_soup.npz")
    for k in range(8):
        s = are.SceneArrays()
        s.triangle_test = are.TRI_REFERENCE_MT
        s.material()
        s.add_triangles(g[f"tris{k}"], 0)
        h, _ = are.Scene(s).intersect(rays8(g[f"rays{k}"]))
        assert_bitexact(ref_to_core(g[f"hits{k}"]), h, f"soup {k}")


def test_ten_million_rays_reference_scene(gpu_lib, oracle, nthreads):
    """10M seeded rays on rt.cpp's scene, GPU vs the oracle (itself pinned
    bit-exact to the reference's intersect())."""
    s = legacy_scene_from_export(np.load(GOLDEN / "rt_scene.npy"))
    sc = are.Scene(s)
    ctx = oracle.prepare(s, accel=0)
    for chunk in range(5):
        r = random_rays(2_000_000, 10_000 + chunk)
        h, ms = sc.intersect(r)
        assert_bitexact(oracle.intersect(ctx, r, nthreads), h, f"chunk {chunk}")


@pytest.mark.parametrize("cfg,kw", [
    (are.CONFIG_RANDOM_SPHERES, dict(lo=-12, hi=12, t_min=1e-3, camera=(13, 2, 3))),
    (are.CONFIG_CORNELL, dict(lo=0, hi=555, t_min=1e-3, camera=(278, 278, -800))),
    (are.CONFIG_CORNELL_OCCLUDED, dict(lo=0, hi=555, t_min=1e-3, camera=(278, 278, -800))),
    (are.CONFIG_MESH, dict(lo=-1.5, hi=2.5, t_min=1e-4, camera=(0, 1.6, 4.5))),
], ids=["random_spheres", "cornell", "cornell_occluded", "mesh_2M"])
def test_workload_scenes_ten_million_rays(gpu_lib, oracle, nthreads, cfg, kw):
    """Every workload scene at its full size (the mesh with all 1,997,123
    triangles): 10M seeded rays, every closest hit (id, t, u, v) equal to the
    oracle's bit for bit.  Spheres (robust quadratic), quads and watertight
    triangles through the SAH BVH or the linear scan, against the oracle's
    linear scan / median BVH."""
    s, _, _ = are.build_config(cfg)
    sc = are.Scene(s)
    ctx = oracle.prepare(s)
    for part in range(5):  # 5 x 2M rays, to bound host memory
        r = random_rays(2_000_000, 50 + 10 * cfg + part, t_max=np.inf, **kw)
        h, ms = sc.intersect(r)
        assert_bitexact(oracle.intersect(ctx, r, nthreads), h, f"config {cfg} part {part}")
    if cfg == are.CONFIG_MESH:
        info = sc.info()
        assert info["prims"] == 1_997_123 and info["depth"] <= 60


def test_quads_through_the_bvh(gpu_lib, oracle, nthreads):
    """Three Cornell boxes side by side: more quads than the linear shared-memory
    scan takes, so quads go through the BVH."""
    s, _, _ = are.build_config(are.CONFIG_CORNELL)
    q = s.quads
    big = are.SceneArrays(materials=s.materials, textures=s.textures)
    for k in range(3):
        qq = q.copy()
        qq[:, 0] += 600.0 * k
        big.add_quads(qq, s.quad_mat)
    assert big.n_prims > 48
    sc = are.Scene(big)
    r = random_rays(1_000_000, 8, lo=0, hi=1700, t_min=1e-3, t_max=np.inf, camera=(900, 278, -800))
    h, _ = sc.intersect(r)
    assert_bitexact(oracle.intersect(oracle.prepare(big), r, nthreads), h, "quads via BVH")


def test_ray_extent_and_empty_scene(gpu_lib, oracle):
    s, _, _ = are.build_config(are.CONFIG_CORNELL)
    r = random_rays(20_000, 7, lo=0, hi=555, t_min=1e-3, t_max=np.inf, camera=(278, 278, -800))
    r[:, 7] = np.linspace(1.0, 2000.0, len(r), dtype=np.float32)  # finite t_max per ray
    r[::7, 3] = 100.0                                               # larger t_min on some
    h, _ = are.Scene(s).intersect(r)
    assert_bitexact(oracle.intersect(oracle.prepare(s, accel=0), r), h, "t range")
    e = are.SceneArrays()
    e.material()
    h, _ = are.Scene(e).intersect(r)
    assert np.all(hit_ids(h) == -1) and np.all(np.isinf(h[:, 0]))


def test_negative_t_min_rays(gpu_lib, oracle):
    """Rays whose interval starts behind the origin: warps holding such a ray
    take the per-lane scan (hits at t <= 0 and ties between +0 and -0 keep the
    (t, global id) order); the others the warp-cooperative one.  Both equal the
    oracle bit for bit."""
    s, _, _ = are.build_config(are.CONFIG_CORNELL)
    r = random_rays(50_000, 17, lo=0, hi=555, t_min=1e-3, t_max=np.inf, frac_camera=0.0)  # origins in the room
    r[: len(r) // 2 : 97, 3] = -300.0  # sparse in the first half, none in the second
    h, _ = are.Scene(s).intersect(r)
    assert_bitexact(oracle.intersect(oracle.prepare(s, accel=0), r), h, "negative t_min")
    assert (h[: len(r) // 2 : 97, 0] < 0).any()  # some hits behind the origin were found


def test_device_pointer_path(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    s, _, _ = are.build_config(are.CONFIG_RANDOM_SPHERES)
    sc = are.Scene(s)
    r = random_rays(100_000, 3, lo=-12, hi=12, t_min=1e-3, t_max=np.inf, camera=(13, 2, 3))
    dr = torch.from_numpy(r).cuda()
    dh = torch.empty((len(r), 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    sc.intersect_device(dr.data_ptr(), len(r), dh.data_ptr())
    assert_bitexact(oracle.intersect(oracle.prepare(s), r), dh.cpu().numpy(), "device ptrs")


@pytest.mark.parametrize("cfg,kw", [(are.CONFIG_RANDOM_SPHERES, dict(lo=-12, hi=12, camera=(13, 2, 3))),
                                    (are.CONFIG_SPHERE_FIELD, dict(lo=-12, hi=12, camera=(13, 2, 3)))])
def test_bvh_widths_give_the_same_answers(gpu_lib, oracle, nthreads, cfg, kw):
    """The binary and the 4-wide tree over the same scene: every closest hit
    bit-identical (and equal to the oracle's), and the rendered image too."""
    import dataclasses
    s, cam, par = are.build_config(cfg, seed=7, mesh_frequency=20_000 if cfg == are.CONFIG_SPHERE_FIELD else 0)
    s2, s4 = (are.Scene(dataclasses.replace(s, bvh_width=w)) for w in (2, 4))
    r = random_rays(500_000, 31, t_min=1e-3, t_max=np.inf, **kw)
    h2, _ = s2.intersect(r)
    h4, _ = s4.intersect(r)
    assert np.array_equal(h2.view(np.uint32), h4.view(np.uint32))
    idx = np.arange(0, len(r), 25)
    assert_bitexact(oracle.intersect(oracle.prepare(s), r[idx], nthreads), h4[idx], "4-wide")
    par = dict(par, width=96, height=54, spp=8, chunk=2)
    a, va, sa = s2.render(cam, par)
    b, vb, sb = s4.render(cam, par)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.array_equal(va.view(np.uint32), vb.view(np.uint32))
    assert sa["error_word"] == sb["error_word"] == 0
