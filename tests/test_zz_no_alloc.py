"""are_render_noalloc: the render entry point that allocates nothing.

It exists for callers that may not allocate device memory while they render
(plugin hosts that give a plugin a fixed memory budget, applications that
own all device memory through their own allocator).  Its scratch is one
static device array of the library, so these tests check, through the C ABI,
that (1) it produces the same image as the allocating entry point are_render
with the same work split, on calls in a row, (2) the device's free memory does
not change across calls once the first call on the device has done its
one-time set-up, and (3) frames beyond the stated maximum, and host output
pointers, are refused with a clear error.

This file is named so pytest collects it last; it also runs on its own in a
fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from common import are

pytestmark = pytest.mark.gpu


def _render_noalloc(lib, sc, cam, par, rgb_ptr, var_ptr):
    p = are.RenderParams.from_dict(dict(par, flags=int(par.get("flags", 0)) | are.FLAG_DEVICE_OUTPUT))
    c = are.Camera.from_dict(cam)
    st = are.RenderStats()
    status = lib.are_render_noalloc(sc.h, C.byref(c), C.byref(p), rgb_ptr, var_ptr, C.byref(st))
    return status, st.to_dict()


def test_noalloc_matches_are_render_twice(gpu_lib):
    torch = pytest.importorskip("torch")
    lib = gpu_lib
    cases = []
    for cfg, w, h, spp in ((are.CONFIG_CORNELL, 96, 80, 24), (are.CONFIG_RANDOM_SPHERES, 120, 68, 16)):
        s, cam, par = are.build_config(cfg)
        cases.append((are.Scene(s), cam, dict(par, width=w, height=h, spp=spp, seed=4)))
    torch.cuda.init()
    max_items = 524288
    for call, (sched, chunk) in enumerate(((are.SCHEDULE_AUTO, 0), (are.SCHEDULE_WAVEFRONT, 0),
                                           (are.SCHEDULE_MEGAKERNEL, 0), (are.SCHEDULE_MEGAKERNEL, 5))):
        # calls in a row per scene, alternating scenes, through both schedules; the automatic chunk
        # (the smallest whose work items fit the static array) and an explicit one
        for sc, cam, par in cases:
            par = dict(par, schedule=sched, chunk=chunk)
            npix = par["width"] * par["height"]
            used_chunk = chunk or -(-par["spp"] // (max_items // npix))
            n = par["width"] * par["height"] * 3
            rgb = torch.full((n,), -1.0, dtype=torch.float32, device="cuda")
            var = torch.full((n,), -1.0, dtype=torch.float32, device="cuda")
            torch.cuda.synchronize()
            status, st = _render_noalloc(lib, sc, cam, par, rgb.data_ptr(), var.data_ptr())
            assert status == 0, lib.are_last_error().decode()
            assert st["samples"] == par["width"] * par["height"] * par["spp"] and st["error_word"] == 0
            # the allocating entry point with the same work split
            ref, ref_var, _ = sc.render(cam, dict(par, chunk=used_chunk, schedule=are.SCHEDULE_AUTO))
            got = rgb.cpu().numpy().reshape(ref.shape)
            got_var = var.cpu().numpy().reshape(ref.shape)
            assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), f"call {call}: image differs"
            assert np.array_equal(got_var.view(np.uint32), ref_var.view(np.uint32)), f"call {call}: variance differs"


def test_noalloc_leaves_device_memory_untouched(gpu_lib):
    torch = pytest.importorskip("torch")
    lib = gpu_lib
    s, cam, par = are.build_config(are.CONFIG_CORNELL)
    par = dict(par, width=64, height=64, spp=8)
    sc = are.Scene(s)
    rgb = torch.empty(64 * 64 * 3, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    assert _render_noalloc(lib, sc, cam, par, rgb.data_ptr(), None)[0] == 0  # first call: one-time set-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for seed in (1, 2):
        assert _render_noalloc(lib, sc, cam, dict(par, seed=seed), rgb.data_ptr(), None)[0] == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_images_beyond_its_scratch(gpu_lib):
    torch = pytest.importorskip("torch")
    lib = gpu_lib
    s, cam, par = are.build_config(are.CONFIG_CORNELL)
    sc = are.Scene(s)
    rgb = torch.empty(3, dtype=torch.float32, device="cuda")
    status, _ = _render_noalloc(lib, sc, cam, dict(par, width=1024, height=1024, spp=1), rgb.data_ptr(), None)
    assert status == 1
    assert "at most 524288" in lib.are_last_error().decode()
    status, _ = _render_noalloc(lib, sc, cam, dict(par, width=8, height=8, spp=1, pool_size=1 << 20), rgb.data_ptr(),
                                None)
    assert status == 1
    # a chunk that makes more work items than the array holds
    status, _ = _render_noalloc(lib, sc, cam, dict(par, width=720, height=720, spp=4, chunk=1), rgb.data_ptr(), None)
    assert status == 1 and "work items" in lib.are_last_error().decode()


def test_noalloc_rejects_host_output(gpu_lib):
    """Host output buffers (no ARE_FLAG_DEVICE_OUTPUT) are refused with a
    status code before any device work."""
    lib = gpu_lib
    s, cam, par = are.build_config(are.CONFIG_CORNELL)
    sc = are.Scene(s)
    host = np.empty(8 * 8 * 3, np.float32)
    p = are.RenderParams.from_dict(dict(par, width=8, height=8, spp=1, flags=0))
    c = are.Camera.from_dict(cam)
    st = are.RenderStats()
    assert lib.are_render_noalloc(sc.h, C.byref(c), C.byref(p), host.ctypes.data, None, C.byref(st)) == 1
    assert "ARE_FLAG_DEVICE_OUTPUT" in lib.are_last_error().decode()
