"""Guided rendering (are_render_guided) on the occluded-light Cornell box:
unbiased against the plain estimator, and its error against the FP64 CPU
reference (tests/golden/guiding_reference_200.npz, 65,536 spp) at equal
samples and at equal time."""
import time

import numpy as np
import pytest

from common import GOLDEN, are

pytestmark = pytest.mark.gpu
REF = GOLDEN / "guiding_reference_200.npz"


def rel_mse(img, ref):
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))


def c4(res, spp, **kw):
    s, cam, par = are.build_config(are.CONFIG_CORNELL_OCCLUDED)
    return s, cam, dict(par, width=res, height=res, spp=spp, **kw)


SCHEDULES = [pytest.param(are.SCHEDULE_WAVEFRONT, id="wavefront"), pytest.param(are.SCHEDULE_MEGAKERNEL, id="megakernel")]


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_guided_is_unbiased(gpu_lib, schedule):
    s, cam, par = c4(48, 2048, seed=3, schedule=schedule)
    sc = are.Scene(s)
    g = are.Guide(seed=5)
    img, var, st = sc.render_guided(g, cam, par, are.GuideParams.make(batch=1 << 12))
    ref, rvar, _ = sc.render(cam, dict(par, spp=8192, seed=4))
    assert st["train_steps"] > 0 and st["error_word"] == 0
    assert np.isfinite(img).all()
    z = np.abs(img - ref) / np.sqrt(var + rvar + 1e-12)
    assert (z > 3).mean() < 0.02, (z > 3).mean()
    # image means agree within their standard errors
    se = np.sqrt(var.sum() + rvar.sum()) / img.size
    assert abs(img.mean() - ref.mean()) < 5 * se + 1e-5


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_mix_zero_is_the_plain_estimator(gpu_lib, schedule):
    """With mix = 0 every guided vertex samples the cosine lobe with the same
    random numbers, and the MIS weight is exactly 1: the image is the plain
    estimator's bit for bit, whatever the network (or the mixture cache of the
    megakernel schedule) holds."""
    s, cam, par = c4(64, 64, seed=21, schedule=schedule)
    sc = are.Scene(s)
    g = are.Guide(seed=4)
    gi, gv, st = sc.render_guided(g, cam, par, are.GuideParams.make(mix=0.0, guide_depth=4, train=0))
    pi, pv, _ = sc.render(cam, par)
    assert st["guided_vertices"] > 0
    assert np.array_equal(gi.view(np.uint32), pi.view(np.uint32))
    assert np.array_equal(gv.view(np.uint32), pv.view(np.uint32))


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_guided_beats_plain_at_equal_samples(gpu_lib, schedule):
    r = np.load(REF)
    ref = r["mean"].astype(np.float64)
    res = int(r["width"])
    s, cam, par = c4(res, 1024, seed=7, schedule=schedule)
    sc = are.Scene(s)
    g = are.Guide(seed=1)
    gp = are.GuideParams.make(guide_depth=3, batch=1 << 14, train=2)
    # train the network online over a few renders, then render with it frozen
    for k in range(6):
        sc.render_guided(g, cam, dict(par, seed=100 + k), gp, with_var=False)
    gi, _, st = sc.render_guided(g, cam, par, are.GuideParams.make(guide_depth=3, train=0), with_var=False)
    pi, _, _ = sc.render(cam, dict(par, schedule=are.SCHEDULE_AUTO), with_var=False)
    e_g, e_p = rel_mse(gi, ref), rel_mse(pi, ref)
    print(f"equal spp (1024, schedule {schedule}): relMSE guided {e_g:.4g} plain {e_p:.4g} ratio {e_p / e_g:.2f}; "
          f"{len(g.loss_history())} Adam steps")
    assert st["train_steps"] == 0
    assert e_g < 0.85 * e_p


@pytest.mark.skipif(not REF.exists(), reason="FP64 reference not generated")
def test_guided_vs_plain_at_equal_time(gpu_lib):
    """The guiding target: at equal wall-clock time (0.1 s per render, each
    method's samples per pixel fitted to it on a warmed call) the guided
    render of the occluded-light Cornell box has at least 2x lower relMSE
    against the FP64 65,536-spp reference than the plain one.  The network is
    the declared warm start of the benchmark: trained online while rendering
    ten earlier 1024-spp frames, then frozen.  Measured on GB300 at 200x200:
    2.7-4.1x (a fresh network trained inside the budget: 0.8-1.2x)."""
    r = np.load(REF)
    ref = r["mean"].astype(np.float64)
    res = int(r["width"])
    s, cam, par = c4(res, 64, seed=9)
    sc = are.Scene(s)
    budget = 0.1
    ge = dict(guide_depth=16, mix=0.5, batch=1 << 14, cache_res=32)
    g = are.Guide(seed=1)
    for k in range(10):
        sc.render_guided(g, cam, dict(par, spp=1024, seed=100 + k), are.GuideParams.make(train=8, **ge),
                         with_var=False)
    frozen = are.GuideParams.make(train=0, **ge)

    def fit(run):
        run(64)
        t = time.perf_counter()
        run(512)
        per = (time.perf_counter() - t) / 512
        spp = max(1, int(budget / per))
        t = time.perf_counter()
        img = run(spp)
        return img, spp, time.perf_counter() - t

    pi, spp_p, t_p = fit(lambda n: sc.render(cam, dict(par, spp=n, seed=12), with_var=False)[0])
    gi, spp_g, t_g = fit(lambda n: sc.render_guided(g, cam, dict(par, spp=n, seed=11), frozen, with_var=False)[0])
    e_g, e_p = rel_mse(gi, ref), rel_mse(pi, ref)
    print(f"equal time: guided {spp_g} spp {t_g:.3f}s relMSE {e_g:.4g}; plain {spp_p} spp {t_p:.3f}s relMSE {e_p:.4g}; "
          f"ratio {e_p / e_g:.2f}; {len(g.loss_history())} Adam steps")
    assert abs(t_g - t_p) < 0.35 * budget  # the two renders took about the same time
    assert e_p / e_g >= 2.0, e_p / e_g


@pytest.mark.parametrize("cfg,res", [(are.CONFIG_RANDOM_SPHERES, (96, 54)), (are.CONFIG_MESH, (64, 36))],
                         ids=["spheres_binary_bvh", "mesh_4wide_bvh"])
def test_guided_megakernel_on_bvh_scenes(gpu_lib, cfg, res):
    """The guided megakernel's BVH instantiations (binary tree; 4-wide tree):
    with mix 0 the image is the plain megakernel's bit for bit, and with a
    network training online it stays within the per-pixel 3-sigma bound of a
    plain render with another seed."""
    s, cam, par = are.build_config(cfg)
    par = dict(par, width=res[0], height=res[1], spp=32, seed=5, schedule=are.SCHEDULE_MEGAKERNEL)
    sc = are.Scene(s)
    g = are.Guide(seed=3)
    gi, gv, st = sc.render_guided(g, cam, par, are.GuideParams.make(mix=0.0, guide_depth=8, train=0))
    pi, pv, _ = sc.render(cam, par)
    assert st["guided_vertices"] > 0 and st["error_word"] == 0
    assert np.array_equal(gi.view(np.uint32), pi.view(np.uint32))
    assert np.array_equal(gv.view(np.uint32), pv.view(np.uint32))
    par = dict(par, spp=256)
    img, var, st = sc.render_guided(g, cam, par, are.GuideParams.make(guide_depth=8, batch=1 << 12, train=4))
    ref, rvar, _ = sc.render(cam, dict(par, seed=6))
    assert st["error_word"] == 0 and np.isfinite(img).all()
    z = np.abs(img - ref) / np.sqrt(var + rvar + 1e-12)
    assert (z > 3).mean() < 0.02, (z > 3).mean()
