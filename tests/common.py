"""Shared helpers for the tests: import paths, scene builders and seeded rays."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[1]
PKG = REPO / "aurora-rendering-engine_gb300"
GOLDEN = REPO / "tests" / "golden"
for p in (str(REPO), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)

import are_gb300 as are  # noqa: E402

REF_T_MIN = 1e-5   # rt.cpp:15 EPS, the reference's t > EPS rule
REF_T_MAX = 1e30   # rt.cpp:16 INF, HitRec's initial t (rt.cpp:205)


def legacy_scene_from_export(exp: np.ndarray) -> are.SceneArrays:
    """SceneArrays equal to rt.cpp's Scene (rt.cpp:153-167), from the 28-float
    per-triangle export of oracle/_ref (or the committed fixture)."""
    s = are.SceneArrays()
    s.triangle_test = are.TRI_REFERENCE_MT
    s.background, s.bg_a = are.BG_CONSTANT, (0.06, 0.09, 0.14)
    tex_ids, mat_ids = {}, []
    for row in exp:
        key = tuple(np.round(row[20:28], 6))
        if key not in tex_ids:
            kind = int(row[20])
            tex_ids[key] = s.texture(are.TEX_CHECKER if kind == 1 else are.TEX_SOLID, a=row[21:24], b=row[24:27],
                                     scale=float(row[27]) if kind == 1 else 1.0)
        mt = are.MAT_METAL if int(row[15]) == 1 else are.MAT_LAMBERTIAN
        mat_ids.append(s.material(mt, texture=tex_ids[key], reflect_ratio=float(row[16]), tint=row[17:20]))
    s.add_triangles(exp[:, 0:9], np.array(mat_ids, np.int32), uv=exp[:, 9:15])
    return s


def random_rays(n: int, seed: int, lo=-1.2, hi=1.2, t_min=REF_T_MIN, t_max=REF_T_MAX,
                camera=(0.0, 0.0, 4.0), frac_camera=0.5) -> np.ndarray:
    """n x 8 rays (o, t_min, d, t_max): half from the reference camera
    position, half from random points of the box, directions uniform on the
    sphere.  numpy's PCG64 stream is the same on every platform."""
    rng = np.random.Generator(np.random.PCG64(seed))
    o = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    ncam = int(n * frac_camera)
    o[:ncam] = np.asarray(camera, np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.empty((n, 8), np.float32)
    rays[:, 0:3], rays[:, 3], rays[:, 4:7], rays[:, 7] = o, t_min, d.astype(np.float32), t_max
    return rays


def hit_ids(h: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(h[:, 1]).view(np.int32)


def sigma_test(m1, v1, m2, v2):
    """Fraction of pixel channels whose means differ by more than 3 standard
    errors of their difference; channels with zero variance on both sides must
    match to 1e-5 relative.  Returns (fraction, zero-variance mismatches)."""
    sd = np.sqrt(v1 + v2)
    z = np.abs(m1 - m2)
    flat = sd == 0
    bad_flat = flat & (z > 1e-5 * np.maximum(1.0, np.abs(m1)))
    out = ~flat & (z > 3 * sd)
    return (out.sum() + bad_flat.sum()) / m1.size, bad_flat.sum()


def binomial_bound(n, p=0.0027, k=5.0):
    """Upper bound on the failure fraction of n independent 3-sigma tests
    (expected 0.27 % under the null), k binomial standard deviations above."""
    return p + k * np.sqrt(p * (1 - p) / n)


def same_seed_agreement(m_gpu, m_cpu, rel=1e-4):
    """Fractions of pixel channels that are bit-identical and that agree to
    `rel` relative (floor 1e-3 absolute scale) between two same-seed renders."""
    same = (m_gpu.view(np.uint32) == m_cpu.view(np.uint32)).mean()
    close = (np.abs(m_gpu - m_cpu) <= rel * np.maximum(1e-3, np.abs(m_cpu))).mean()
    return float(same), float(close)


def adapted_scene() -> "are.SceneArrays":
    """The scene tests/harness/are_adapted_scene.cpp builds from the reference
    library's own types, as include/aurora_gb300_are.hpp converted it
    (tests/golden/are_adapted_scene.npz), lit by a sky-gradient background."""
    z = np.load(GOLDEN / "are_adapted_scene.npz")
    s = are.SceneArrays()
    s.triangles, s.triangle_uv, s.triangle_mat = z["triangles"], z["triangle_uv"], z["triangle_mat"]
    s.materials = np.frombuffer(z["materials"].tobytes(), are.MATERIAL_DTYPE).copy()
    s.textures = np.frombuffer(z["textures"].tobytes(), are.TEXTURE_DTYPE).copy()
    s.texels = z["texels"]
    s.background, s.bg_a, s.bg_b = are.BG_SKY_GRADIENT, (1.0, 1.0, 1.0), (0.5, 0.7, 1.0)
    s.triangle_test = are.TRI_WATERTIGHT
    return s


ADAPTED_CAMERA = {"lookfrom": [2.0, 2.2, -3.0], "lookat": [2.0, 1.0, 2.0], "vup": [0.0, 1.0, 0.0], "vfov_deg": 60.0,
                  "aperture": 0.0, "focus_dist": 1.0}
