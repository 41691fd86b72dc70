"""Writes the workload scenes the benchmark's reference arm renders, as
plain arrays (TEST INFRASTRUCTURE: read only by bench.py's reference arm and
its CPU-baseline leg, which must not load the CUDA core's library).

    python oracle/scenes/make_scenes.py

Each .npz holds the scene descriptor's arrays (the 48-byte material and
64-byte texture records as raw bytes), the camera and the render
parameters of one workload, exported from the scene builder of the core
(are_config_build) so both arms render the same scene.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO / "aurora-rendering-engine_gb300"))

import are_gb300 as are  # noqa: E402

SCENES = {"cornell_box": are.CONFIG_CORNELL, "random_spheres": are.CONFIG_RANDOM_SPHERES}


def main() -> None:
    for name, cfg in SCENES.items():
        s, cam, par = are.build_config(cfg)
        out = {k: np.asarray(getattr(s, k)) for k in ("spheres", "sphere_mat", "quads", "quad_mat", "triangles",
                                                        "triangle_mat")}
        out["materials"] = np.frombuffer(s.materials.tobytes(), np.uint8)
        out["textures"] = np.frombuffer(s.textures.tobytes(), np.uint8)
        out["background"] = np.int32(s.background)
        out["bg_a"], out["bg_b"] = np.float32(s.bg_a), np.float32(s.bg_b)
        out["triangle_test"] = np.int32(s.triangle_test)
        for k in ("lookfrom", "lookat", "vup"):
            out["cam_" + k] = np.float32(cam[k])
        for k in ("vfov_deg", "aperture", "focus_dist"):
            out["cam_" + k] = np.float32(cam[k])
        for k, v in par.items():
            out["par_" + k] = np.asarray(v)
        np.savez_compressed(HERE / f"{name}.npz", **out)
        print(name, s.n_prims, "primitives")


if __name__ == "__main__":
    main()
