"""Edge cases of are_render on both schedules (megakernel, wavefront): an
empty scene, a one-pixel frame, paths of a single segment, and scenes on
either side of the linear-scan limit (48 primitives: the warp-cooperative
scan of staged primitives; 49: the BVH).  Closest hits bit-exact against the
oracle; images between the schedules bit for bit and against the oracle's
same-seed render."""
import numpy as np
import pytest

from common import are, hit_ids, random_rays

pytestmark = pytest.mark.gpu

SCHEDULES = (are.SCHEDULE_MEGAKERNEL, are.SCHEDULE_WAVEFRONT)
LINEAR_MAX = 48  # core.h


def render_both(sc, cam, par):
    """Both schedules with the same chunk: the same image and statistics."""
    out = [sc.render(cam, dict(par, schedule=s)) for s in SCHEDULES]
    (a, va, sa), (b, vb, sb) = out
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.array_equal(va.view(np.uint32), vb.view(np.uint32))
    assert sa["samples"] == sb["samples"] and sa["segments"] == sb["segments"]
    assert sa["error_word"] == sb["error_word"] == 0
    return a, va, sa


def test_empty_scene_is_the_background(gpu_lib):
    s = are.SceneArrays()
    s.material()
    s.bg_a = (0.25, 0.5, 0.75)
    cam = dict(lookfrom=(0, 0, 0), lookat=(0, 0, -1), vup=(0, 1, 0), vfov_deg=60.0, aperture=0.0, focus_dist=1.0)
    par = dict(width=17, height=9, spp=8, max_depth=8, seed=3, rr_depth=3, t_min=1e-3, chunk=2)
    img, var, st = render_both(are.Scene(s), cam, par)
    assert st["samples"] == 17 * 9 * 8 and st["segments"] == st["samples"]  # one miss per path
    assert np.allclose(img, np.asarray(s.bg_a, np.float32), rtol=1e-6, atol=0)
    assert np.all(var <= 1e-12)


def test_one_pixel_frame(gpu_lib, oracle, nthreads):
    s, cam, par = are.build_config(are.CONFIG_CORNELL)
    par = dict(par, width=1, height=1, spp=256, chunk=16)
    img, var, st = render_both(are.Scene(s), cam, par)
    m, v, st_cpu = oracle.render(oracle.prepare(s), cam, par, nthreads=nthreads)
    assert st["samples"] == st_cpu["samples"] == 256
    assert np.all(np.abs(img - m) <= 5 * np.sqrt(var + v) + 1e-6)


def test_single_segment_paths(gpu_lib, oracle, nthreads):
    """max_depth 1: a path is its camera ray; the image is the emission seen
    directly, the same rays and hits as the oracle's."""
    s, cam, par = are.build_config(are.CONFIG_CORNELL)
    par = dict(par, width=40, height=40, spp=16, max_depth=1, chunk=4)
    img, var, st = render_both(are.Scene(s), cam, par)
    m, v, st_cpu = oracle.render(oracle.prepare(s), cam, par, nthreads=nthreads)
    assert st["segments"] == st["samples"] == st_cpu["samples"] == 40 * 40 * 16
    assert img.max() > 0  # the light is in view
    assert np.allclose(img, m, rtol=1e-5, atol=1e-6)


def random_scene(n: int, seed: int) -> are.SceneArrays:
    """n primitives in a unit box around the origin (quads, spheres and
    watertight triangles in turn), a white diffuse material and a light."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = are.SceneArrays()
    white = s.material(albedo=(0.7, 0.7, 0.7))
    lamp = s.material(are.MAT_DIFFUSE_LIGHT, emit=(4.0, 4.0, 4.0))
    s.background = are.BG_SKY_GRADIENT
    s.bg_a, s.bg_b = (1.0, 1.0, 1.0), (0.5, 0.7, 1.0)
    for k in range(n):
        c = rng.uniform(-1, 1, 3)
        mat = lamp if k % 11 == 0 else white
        if k % 3 == 0:
            s.add_quads(np.concatenate([c, rng.normal(size=3) * 0.3, rng.normal(size=3) * 0.3]), mat)
        elif k % 3 == 1:
            s.add_spheres([*c, rng.uniform(0.05, 0.2)], mat)
        else:
            s.add_triangles(np.concatenate([c, c + rng.normal(size=3) * 0.3, c + rng.normal(size=3) * 0.3]), mat)
    return s


@pytest.mark.parametrize("n", [LINEAR_MAX, LINEAR_MAX + 1])
def test_linear_scan_limit(gpu_lib, oracle, nthreads, n):
    s = random_scene(n, 40 + n)
    assert s.n_prims == n
    sc = are.Scene(s)
    r = random_rays(200_000, n, lo=-1.5, hi=1.5, t_min=1e-4, t_max=np.inf, camera=(0, 0, 4))
    h, _ = sc.intersect(r)
    ref = oracle.intersect(oracle.prepare(s, accel=0), r, nthreads)
    ih, ir = hit_ids(h), hit_ids(ref)
    assert np.array_equal(ih, ir)
    m = ih >= 0
    assert m.mean() > 0.03  # ~15k hits of 200k rays among small primitives
    assert np.array_equal(h[m][:, [0, 2, 3]].view(np.uint32), ref[m][:, [0, 2, 3]].view(np.uint32))
    cam = dict(lookfrom=(0, 0, 4), lookat=(0, 0, 0), vup=(0, 1, 0), vfov_deg=45.0, aperture=0.0, focus_dist=4.0)
    par = dict(width=48, height=32, spp=32, max_depth=8, seed=5, rr_depth=3, t_min=1e-4, chunk=8)
    img, var, st = render_both(sc, cam, par)
    mc, vc, _ = oracle.render(oracle.prepare(s), cam, par, nthreads=nthreads)
    sd = np.sqrt(var + vc)
    out = (sd > 0) & (np.abs(img - mc) > 4 * sd)
    assert out.mean() < 0.01, out.mean()


def test_scene_churn_reuses_pooled_memory(gpu_lib):
    """Create, render and destroy a scene again and again (as a caller that
    rebuilds its scene every frame): scene arrays and render workspaces come
    from the device's memory pool, so after the first cycle the device's free
    memory stays where it is — nothing leaks and nothing is allocated anew."""
    torch = pytest.importorskip("torch")
    s, cam, par = are.build_config(are.CONFIG_RANDOM_SPHERES)
    par = dict(par, width=160, height=90, spp=4)

    def cycle(seed):
        sc = are.Scene(s)
        img, _, st = sc.render(cam, dict(par, seed=seed), with_var=False)
        sc.close()
        assert st["error_word"] == 0 and np.isfinite(img).all()

    torch.cuda.init()
    cycle(0)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for k in range(1, 21):
        cycle(k)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    # the cached blocks go back to the driver on request
    are.trim_memory(-1)
    torch.cuda.synchronize()
    free2, _ = torch.cuda.mem_get_info()
    assert free2 > free1
    with pytest.raises(are.AreError):
        are.trim_memory(1000)


def textured_quad(filt):
    """A 5x4 random image texture on a lambertian quad under a constant white
    sky: with roulette off and two segments per path, a pixel's radiance is
    exactly the texture at its camera ray's hit (albedo x sky)."""
    rng = np.random.Generator(np.random.PCG64(9))
    s = are.SceneArrays()
    s.bg_a = (1.0, 1.0, 1.0)
    s.texels = rng.uniform(0.0, 1.0, (5 * 4, 3)).astype(np.float32)
    t = s.texture(are.TEX_IMAGE, width=5, height=4, texel_offset=0, filter=filt)
    s.add_quads([-1, -1, 0, 2, 0, 0, 0, 2, 0], s.material(are.MAT_LAMBERTIAN, texture=t))
    cam = dict(lookfrom=(0, 0, 3), lookat=(0, 0, 0), vup=(0, 1, 0), vfov_deg=40.0, aperture=0.0, focus_dist=3.0)
    par = dict(width=48, height=48, spp=1, max_depth=2, seed=1, rr_depth=-1, t_min=1e-4,
               flags=are.FLAG_NO_JITTER, chunk=1)
    return s, cam, par


def test_image_texture_filters(gpu_lib, oracle, nthreads):
    """Nearest (are::Texture::pixel) and bilinear (src/texture.cpp:310-330's
    weights) texel lookups: the GPU's image equals the oracle's, and the two
    filters give different images."""
    out = {}
    for filt in (are.FILTER_NEAREST, are.FILTER_BILINEAR):
        s, cam, par = textured_quad(filt)
        img, _, st = render_both(are.Scene(s), cam, par)
        ref, _, _ = oracle.render(oracle.prepare(s), cam, par, nthreads=nthreads)
        assert st["error_word"] == 0
        assert np.allclose(img, ref, rtol=1e-5, atol=1e-6), np.abs(img - ref).max()
        out[filt] = img
    hit = out[are.FILTER_NEAREST] < 0.999  # pixels on the quad (the sky is exactly 1)
    assert hit.mean() > 0.3
    assert not np.allclose(out[are.FILTER_NEAREST][hit], out[are.FILTER_BILINEAR][hit], atol=1e-3)


def test_adapted_reference_scene_against_the_oracle(gpu_lib, oracle, nthreads):
    """A scene made of the reference library's own types (are::Triangle,
    are::Diffuse, are::Reflective, are::Texture images filled through
    pixel()), converted by include/aurora_gb300_are.hpp (the committed
    fixture tests/golden/are_adapted_scene.npz), rendered on the GPU and by
    the oracle with the same random numbers: per-pixel 3-sigma agreement."""
    from common import ADAPTED_CAMERA, adapted_scene, binomial_bound, same_seed_agreement, sigma_test
    s = adapted_scene()
    par = dict(width=160, height=120, spp=64, max_depth=16, seed=3, rr_depth=3, t_min=1e-4, estimator=are.EST_PATH)
    m_gpu, v_gpu, st = are.Scene(s).render(ADAPTED_CAMERA, par)
    m_cpu, v_cpu, _ = oracle.render(oracle.prepare(s), ADAPTED_CAMERA, par, nthreads=nthreads)
    assert st["error_word"] == 0 and st["samples"] == 160 * 120 * 64
    frac, _ = sigma_test(m_gpu, v_gpu, m_cpu, v_cpu)
    same, close = same_seed_agreement(m_gpu, m_cpu)
    assert frac <= binomial_bound(m_gpu.size), frac
    assert close >= 0.98, close
    assert m_gpu.mean() > 0.05  # the room is lit and visible
