"""Generate the committed golden fixtures from the reference itself.

Runs only where the reference tree exists: oracle/build.py compiles
experiments/rt.cpp and the library's src/*.cpp from their own sources into
oracle/_ref/, and this script records their outputs on seeded inputs:

* rt_scene.npy        rt.cpp Scene::Scene() triangles (rt.cpp:153-185), 28 floats each
* rt_intersect.npz    rays and rt.cpp intersect() hits on that scene (rt.cpp:209-218)
* rt_soup.npz         random triangle soups, rays and Tri::intersect linear-scan hits
* rt_kat.npz          CheckerTexture::at, rotateToHemisphere, writePPM bytes
* lib_kat.npz         are::reflect / are::refract, are::Plane::intersect_ray,
                      are::Triangle FP64 intersect_ray and constructor checks
* rt_render.npz       rt.cpp render() with std::random_device fixed to a seed
* rt_out_diffuse.npz  32x32-pixel block means of experiments/out_diffuse.ppm, the
                      reference's own committed rt.cpp render (512x512, unknown seed)

Usage: python tests/golden/make_golden.py   (from the repository root)
"""
from __future__ import annotations

import ctypes as C
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "tests"))

from oracle import build as obuild  # noqa: E402
from oracle.orc import RefLib, RefRT  # noqa: E402
from common import random_rays  # noqa: E402

_d = C.POINTER(C.c_double)


def dp(a):
    return a.ctypes.data_as(_d)


def out_diffuse_summary() -> None:
    """Block means of the reference's committed render (a P6 PPM, rt.cpp:377-392);
    its seed is unknown (rt.cpp:348-351), so only statistics can be compared."""
    raw = (obuild.REF_ROOT / "experiments" / "out_diffuse.ppm").read_bytes()
    magic, size, maxval, body = raw.split(b"\n", 3)
    w, h = map(int, size.split())
    assert magic == b"P6" and maxval == b"255" and len(body) == w * h * 3
    img = np.frombuffer(body, np.uint8).reshape(h, w, 3).astype(np.float64)
    blocks = img.reshape(h // 32, 32, w // 32, 32, 3).mean((1, 3))
    np.savez_compressed(HERE / "rt_out_diffuse.npz", width=w, height=h, block=32, means=blocks)


def main() -> None:
    obuild.build_ref()
    out_diffuse_summary()
    ref = RefRT()
    lib = RefLib()

    exp = ref.scene()
    np.save(HERE / "rt_scene.npy", exp)

    rays = random_rays(100_000, 2024)
    r6 = np.concatenate([rays[:, 0:3], rays[:, 4:7]], 1)
    # the reference's documented tie: the camera axis hits the back wall's diagonal
    r6[0] = [0, 0, 4, 0, 0, -1]
    hits = ref.intersect(r6)
    np.savez_compressed(HERE / "rt_intersect.npz", rays6=r6, hits=hits)

    rng = np.random.Generator(np.random.PCG64(77))
    soups, soup_rays, soup_hits = [], [], []
    for k in range(8):
        m = int(rng.integers(1, 40))
        tris = rng.uniform(-1, 1, size=(m, 9)).astype(np.float32)
        if k % 2:  # shared edges: fans around one vertex
            tris[1:, 0:3] = tris[0, 0:3]
        rr = random_rays(2000, 500 + k, lo=-1.5, hi=1.5, camera=(0.0, 0.0, 3.0))
        rr6 = np.concatenate([rr[:, 0:3], rr[:, 4:7]], 1)
        soups.append(tris)
        soup_rays.append(rr6)
        soup_hits.append(ref.intersect_soup(tris, rr6))
    np.savez_compressed(HERE / "rt_soup.npz", **{f"tris{k}": t for k, t in enumerate(soups)},
                        **{f"rays{k}": r for k, r in enumerate(soup_rays)},
                        **{f"hits{k}": h for k, h in enumerate(soup_hits)})

    # known answers from rt.cpp
    uv = rng.uniform(-3, 3, size=(2000, 2)).astype(np.float32)
    a = np.array([0.9, 0.9, 0.9], np.float32)
    b = np.array([0.1, 0.1, 0.1], np.float32)
    chk = np.zeros((len(uv), 3), np.float32)
    f = C.POINTER(C.c_float)
    out = np.zeros(3, np.float32)
    for i, (u, v) in enumerate(uv):
        ref.lib.ref_checker_at(a.ctypes.data_as(f), b.ctypes.data_as(f), 8.0, float(u), float(v),
                               out.ctypes.data_as(f))
        chk[i] = out
    nrm = rng.normal(size=(2000, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm[:10] = [[0, 0, 1], [0, 0, -1], [1, 0, 0], [0, 1, 0], [0, 0.9995, 0.0316], [0, 0, 0.9991],
                [0.0447, 0, 0.999], [0, -1, 0], [-1, 0, 0], [0.6, 0.8, 0]]
    nrm = nrm.astype(np.float32)
    luv = rng.uniform(-0.7, 0.7, size=(2000, 2)).astype(np.float32)
    hemi = np.zeros((len(nrm), 3), np.float32)
    for i in range(len(nrm)):
        ref.lib.ref_rotate_to_hemisphere(nrm[i].ctypes.data_as(f), float(luv[i, 0]), float(luv[i, 1]),
                                         out.ctypes.data_as(f))
        hemi[i] = out
    img = rng.uniform(-0.2, 1.2, size=(7, 5, 3)).astype(np.float32)
    img[0, 0] = [0.0, 1.0, 0.5]
    with tempfile.TemporaryDirectory() as td:
        pth = str(Path(td) / "o.ppm").encode()
        ref.lib.ref_write_ppm(img.reshape(-1).ctypes.data_as(f), 5, 7, pth)
        ppm = np.frombuffer(Path(pth.decode()).read_bytes(), np.uint8)
    np.savez_compressed(HERE / "rt_kat.npz", checker_uv=uv, checker_a=a, checker_b=b, checker_scale=8.0,
                        checker_out=chk, hemi_n=nrm, hemi_uv=luv, hemi_out=hemi, ppm_img=img, ppm_bytes=ppm)

    # known answers from the library (FP64)
    v = rng.normal(size=(500, 3))
    n = rng.normal(size=(500, 3))
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    eta = rng.uniform(0.4, 2.5, size=500)
    refl = np.zeros((500, 3))
    refr = np.zeros((500, 3))
    o3 = np.zeros(3)
    for i in range(500):
        lib.lib.ref_lib_reflect(dp(np.ascontiguousarray(v[i])), dp(np.ascontiguousarray(n[i])), dp(o3))
        refl[i] = o3
        lib.lib.ref_lib_refract(dp(np.ascontiguousarray(v[i])), dp(np.ascontiguousarray(n[i])), float(eta[i]), dp(o3))
        refr[i] = o3
    tris = rng.uniform(-1, 1, size=(12, 9))
    lrays = np.concatenate([rng.uniform(-2, 2, size=(3000, 3)), rng.normal(size=(3000, 3))], 1)
    lhits = np.zeros((3000, 4))
    lib.lib.ref_lib_triangles_intersect(dp(tris), 12, dp(lrays), 3000, dp(lhits))
    bad = [([0, 0, 0], [0, 0, 0], [1, 0, 0]), ([0, 0, 0], [1, 0, 0], [2, 0, 0]), ([0, 0, 0], [1, 0, 0], [0, 1, 0]),
           ([1, 1, 1], [1e-9, 0, 0], [0, 1, 0])]
    ctor = np.array([lib.lib.ref_lib_triangle_check(dp(np.array(q, float)), dp(np.array(u, float)),
                                                    dp(np.array(w, float))) for q, u, w in bad], np.int32)
    np.savez_compressed(HERE / "lib_kat.npz", v=v, n=n, eta=eta, reflect=refl, refract=refr, tris=tris,
                        rays=lrays, hits=lhits, ctor_cases=np.array(bad, float), ctor_throws=ctor)

    # the reference render with the per-row RNG seeded from a fixed value
    w = h = 64
    img = ref.render(7, w, h)
    np.savez_compressed(HERE / "rt_render.npz", seed=7, width=w, height=h, rgb=img)
    for p in sorted(HERE.glob("*.np*")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main()
