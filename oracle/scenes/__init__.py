"""Workload scenes as plain arrays for the oracle (TEST INFRASTRUCTURE).

``load(name)`` returns (scene, camera dict, params dict) where the scene is
an object with the numpy attributes oracle.orc.Oracle.prepare reads.  Made
by make_scenes.py in this folder; nothing here loads the CUDA core.
"""
from __future__ import annotations

from pathlib import Path
from types import SimpleNamespace

import numpy as np

HERE = Path(__file__).resolve().parent
MATERIAL_BYTES, TEXTURE_BYTES = 48, 64


def load(name: str):
    z = np.load(HERE / f"{name}.npz")
    s = SimpleNamespace(**{k: z[k] for k in ("spheres", "sphere_mat", "quads", "quad_mat", "triangles",
                                             "triangle_mat")})
    s.triangle_uv = None
    s.texels = None
    # raw 48-byte material / 64-byte texture records, viewed as void records of that size
    s.materials = np.ascontiguousarray(z["materials"]).view(np.dtype((np.void, MATERIAL_BYTES)))
    s.textures = np.ascontiguousarray(z["textures"]).view(np.dtype((np.void, TEXTURE_BYTES)))
    s.background = int(z["background"])
    s.bg_a, s.bg_b = tuple(float(v) for v in z["bg_a"]), tuple(float(v) for v in z["bg_b"])
    s.triangle_test = int(z["triangle_test"])
    s.n_prims = len(s.sphere_mat) + len(s.quad_mat) + len(s.triangle_mat)
    cam = {k: [float(v) for v in z["cam_" + k]] for k in ("lookfrom", "lookat", "vup")}
    cam.update({k: float(z["cam_" + k]) for k in ("vfov_deg", "aperture", "focus_dist")})
    par = {k[4:]: z[k].item() for k in z.files if k.startswith("par_")}
    return s, cam, par
