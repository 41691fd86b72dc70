"""Image parity on the GPU: the path tracer (are_render; megakernel and
wavefront schedules) against the oracle's CPU render of the same estimator.

* same seed: both sides consume the same random numbers, so the images agree
  to float rounding except where an ulp-level difference in a transcendental
  sends one path elsewhere; checked with a per-pixel 3-sigma bound and a
  bound on the fraction of pixels that differ at all;
* independent seeds: per-pixel 3-sigma test whose failure fraction must stay
  within a binomial bound around the 0.27 % expected under the null.
"""
import numpy as np
import pytest

from common import are, binomial_bound, sigma_test

pytestmark = pytest.mark.gpu


def small(cfg, w, h, spp, **kw):
    s, cam, par = are.build_config(cfg)
    par = dict(par, width=w, height=h, spp=spp, **kw)
    return s, cam, par


@pytest.mark.parametrize("cfg,w,h,spp", [(are.CONFIG_CORNELL, 96, 96, 64), (are.CONFIG_RANDOM_SPHERES, 160, 90, 32),
                                         (are.CONFIG_CORNELL_OCCLUDED, 64, 64, 32)])
def test_same_seed_matches_oracle(gpu_lib, oracle, nthreads, cfg, w, h, spp):
    s, cam, par = small(cfg, w, h, spp)
    m_gpu, v_gpu, st = are.Scene(s).render(cam, par)
    m_cpu, v_cpu, st_cpu = oracle.render(oracle.prepare(s), cam, par, nthreads=nthreads)
    assert st["samples"] == w * h * spp == st_cpu["samples"]
    assert np.isfinite(m_gpu).all() and np.isfinite(v_gpu).all()
    frac, flat = sigma_test(m_gpu, v_gpu, m_cpu, v_cpu)
    assert frac <= binomial_bound(m_gpu.size), frac
    close = np.abs(m_gpu - m_cpu) <= 1e-4 * np.maximum(1e-3, np.abs(m_cpu))
    assert close.mean() >= 0.98, close.mean()
    # path lengths agree (same random numbers)
    assert abs(st["segments"] - st_cpu["segments"]) <= 0.01 * st_cpu["segments"]


@pytest.mark.parametrize("cfg,w,h,spp", [(are.CONFIG_RANDOM_SPHERES, 100, 56, 256), (are.CONFIG_CORNELL, 48, 48, 1024)])
def test_independent_seeds_three_sigma(gpu_lib, oracle, nthreads, cfg, w, h, spp):
    s, cam, par = small(cfg, w, h, spp)
    m_gpu, v_gpu, _ = are.Scene(s).render(cam, dict(par, seed=11))
    m_cpu, v_cpu, _ = oracle.render(oracle.prepare(s), cam, dict(par, seed=12), nthreads=nthreads)
    frac, _ = sigma_test(m_gpu, v_gpu, m_cpu, v_cpu)
    assert frac <= binomial_bound(m_gpu.size, k=8.0), frac


def test_deterministic_across_pool_sizes(gpu_lib):
    """The image is a pure function of (scene, camera, params, seed): pool
    size and scheduling do not change a single bit."""
    s, cam, par = small(are.CONFIG_CORNELL, 80, 80, 32, chunk=8)
    sc = are.Scene(s)
    a, va, sa = sc.render(cam, dict(par, pool_size=4096))
    b, vb, sb = sc.render(cam, dict(par, pool_size=65536))
    c, vc, _ = sc.render(cam, dict(par, pool_size=65536))
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.array_equal(b.view(np.uint32), c.view(np.uint32))
    assert np.array_equal(va.view(np.uint32), vb.view(np.uint32))
    assert sa["samples"] == sb["samples"] == 80 * 80 * 32 and sa["error_word"] == 0


def test_full_size_cornell_properties(gpu_lib):
    """The full-size Cornell frame (600x600) at reduced spp: every sample completes,
    the image is finite and non-negative, and the mean radiance matches a
    second render with another seed within its standard error."""
    s, cam, par = are.build_config(are.CONFIG_CORNELL)
    par = dict(par, spp=16)
    sc = are.Scene(s)
    m1, v1, st1 = sc.render(cam, dict(par, seed=1))
    m2, v2, st2 = sc.render(cam, dict(par, seed=2))
    assert st1["samples"] == 600 * 600 * 16 and st1["error_word"] == 0
    assert np.isfinite(m1).all() and (m1 >= 0).all()
    se = np.sqrt(v1.sum() + v2.sum()) / m1.size
    assert abs(m1.mean() - m2.mean()) < 6 * se + 1e-6


def test_render_argument_errors(gpu_lib):
    s, cam, par = small(are.CONFIG_CORNELL, 8, 8, 1)
    sc = are.Scene(s)
    for bad in (dict(width=0), dict(spp=0), dict(max_depth=0), dict(max_depth=1000), dict(t_min=-1.0)):
        with pytest.raises(are.AreError) as e:
            sc.render(cam, dict(par, **bad))
        assert e.value.status == 1
    with pytest.raises(are.AreError):
        sc.render(dict(cam, vfov_deg=0.0), par)


def test_tail_kernel_leaves_the_image_unchanged(gpu_lib):
    """Random spheres (glass and metal: long paths): the tail kernel takes
    over at different points for different pool sizes, and the image is the
    same bit for bit."""
    s, cam, par = small(are.CONFIG_RANDOM_SPHERES, 96, 54, 16, schedule=are.SCHEDULE_WAVEFRONT)
    sc = are.Scene(s)
    n = 96 * 54 * 16
    a, va, sa = sc.render(cam, dict(par, pool_size=4096, chunk=1))
    b, vb, sb = sc.render(cam, dict(par, pool_size=n, chunk=1))
    assert sa["kernel_launches"]["intersect"] > 0  # the wavefront ran before the tail
    assert sa["aux"][0] > 0  # tail segments
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.array_equal(va.view(np.uint32), vb.view(np.uint32))
    assert sa["samples"] == sb["samples"] == n and sa["segments"] == sb["segments"]


@pytest.mark.parametrize("cfg,w,h,spp,chunk", [(are.CONFIG_CORNELL, 64, 64, 48, 4),           # linear scan
                                               (are.CONFIG_RANDOM_SPHERES, 96, 54, 24, 1),   # BVH in shared memory
                                               (are.CONFIG_CORNELL_OCCLUDED, 40, 40, 32, 16),
                                               (are.CONFIG_LEGACY_RT, 48, 48, 16, 3)])       # rt.cpp triangles
def test_megakernel_equals_wavefront(gpu_lib, cfg, w, h, spp, chunk):
    """The two schedules run every work item's samples in one slot in sample
    order with the same device functions: same chunk, same image bit for bit,
    whatever the pool size."""
    s, cam, par = small(cfg, w, h, spp, chunk=chunk, estimator=are.EST_PATH)
    sc = are.Scene(s)
    a, va, sa = sc.render(cam, dict(par, schedule=are.SCHEDULE_WAVEFRONT))
    b, vb, sb = sc.render(cam, dict(par, schedule=are.SCHEDULE_MEGAKERNEL))
    c, vc, sc_ = sc.render(cam, dict(par, schedule=are.SCHEDULE_MEGAKERNEL, pool_size=1024))
    assert sa["kernel_launches"]["intersect"] > 0 and sb["kernel_launches"]["intersect"] == 0
    for x, vx in ((b, vb), (c, vc)):
        assert np.array_equal(a.view(np.uint32), x.view(np.uint32))
        assert np.array_equal(va.view(np.uint32), vx.view(np.uint32))
    assert sa["samples"] == sb["samples"] == sc_["samples"] == w * h * spp
    assert sa["segments"] == sb["segments"] == sc_["segments"]
    assert sb["aux"][0] == sb["segments"]  # every segment traced by the megakernel


def test_megakernel_mesh_equals_wavefront(gpu_lib):
    """The 2M-triangle mesh (BVH far larger than shared memory, watertight
    triangles) at a small image: both schedules give the same bits."""
    s, cam, par = small(are.CONFIG_MESH, 64, 36, 8, chunk=2)
    sc = are.Scene(s)
    a, va, sa = sc.render(cam, dict(par, schedule=are.SCHEDULE_WAVEFRONT))
    b, vb, sb = sc.render(cam, dict(par, schedule=are.SCHEDULE_MEGAKERNEL))
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.array_equal(va.view(np.uint32), vb.view(np.uint32))
    assert sa["segments"] == sb["segments"] and sa["error_word"] == sb["error_word"] == 0


def test_mesh_tail_with_more_paths_than_threads(gpu_lib):
    """A wavefront render whose tail launch can get more queued paths than
    the 4-wide megakernel has resident threads (a 2M-path pool over 4M work
    items: the tail takes over once every item is taken and at most a
    quarter of the pool is queued), so threads may run several queue entries
    one after another through the interleaved walks: the image is still the
    megakernel schedule's bit for bit."""
    s, cam, par = small(are.CONFIG_MESH, 1024, 1024, 4, chunk=1)
    sc = are.Scene(s)
    a, va, sa = sc.render(cam, dict(par, schedule=are.SCHEDULE_WAVEFRONT, pool_size=1 << 21))
    b, vb, sb = sc.render(cam, dict(par, schedule=are.SCHEDULE_MEGAKERNEL))
    assert sa["aux"][0] > 0  # the tail launch traced the last paths
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.array_equal(va.view(np.uint32), vb.view(np.uint32))
    assert sa["segments"] == sb["segments"] and sa["error_word"] == sb["error_word"] == 0


def test_schedule_argument(gpu_lib):
    s, cam, par = small(are.CONFIG_CORNELL, 16, 16, 4)
    sc = are.Scene(s)
    _, _, st = sc.render(cam, par)  # automatic schedule: the megakernel
    assert st["kernel_launches"]["intersect"] == 0 and st["kernel_launches"]["other"] == 3
    for bad in (-1, 3):
        with pytest.raises(are.AreError) as e:
            sc.render(cam, dict(par, schedule=bad))
        assert e.value.status == 1
