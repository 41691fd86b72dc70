"""Builds tests/harness/are_adapted_scene.cpp against the reference library's
headers and compiled sources (oracle/_ref/libref_lib.so, made from the
reference tree by oracle/build.py), runs it, and saves the scene descriptor
the adapter produced as tests/golden/are_adapted_scene.npz, so the GPU test
(tests/test_gpu_render_edges.py) can render the adapted scene where the
reference tree is absent.

Usage: python tests/golden/make_adapted_scene.py
"""
from __future__ import annotations

import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "aurora-rendering-engine_gb300"))

import are_gb300 as are  # noqa: E402
from oracle.build import REF_OUT, REF_ROOT, build_ref  # noqa: E402


def build_and_run(out_bin: Path, workdir: Path) -> str:
    build_ref(REF_ROOT)
    exe = workdir / "are_adapted_scene"
    subprocess.run(["g++", "-std=c++20", "-O1", "-Wall", "-Werror", "-I", str(REF_ROOT / "include"), "-I",
                    str(REPO / "include"), str(REPO / "tests" / "harness" / "are_adapted_scene.cpp"), "-o", str(exe),
                    str(REF_OUT / "libref_lib.so"), f"-Wl,-rpath,{REF_OUT}"], check=True, capture_output=True,
                   text=True)
    return subprocess.run([str(exe), str(out_bin)], check=True, capture_output=True, text=True).stdout


def read(path: Path) -> dict:
    b = path.read_bytes()
    off = 0

    def take(dtype, count):
        nonlocal off
        a = np.frombuffer(b, dtype=dtype, count=count, offset=off)
        off += a.nbytes
        return a.copy()

    n = int(take(np.int32, 1)[0])
    d = {"triangles": take(np.float32, 9 * n).reshape(n, 9), "triangle_uv": take(np.float32, 6 * n).reshape(n, 6),
         "triangle_mat": take(np.int32, n)}
    d["materials"] = take(are.MATERIAL_DTYPE, int(take(np.int32, 1)[0]))
    d["textures"] = take(are.TEXTURE_DTYPE, int(take(np.int32, 1)[0]))
    d["texels"] = take(np.float32, 3 * int(take(np.int64, 1)[0])).reshape(-1, 3)
    assert off == len(b)
    return d


def main() -> None:
    with tempfile.TemporaryDirectory() as t:
        out = Path(t) / "scene.bin"
        print(build_and_run(out, Path(t)).strip())
        d = read(out)
    np.savez_compressed(HERE / "are_adapted_scene.npz", triangles=d["triangles"], triangle_uv=d["triangle_uv"],
                        triangle_mat=d["triangle_mat"], materials=np.frombuffer(d["materials"].tobytes(), np.uint8),
                        textures=np.frombuffer(d["textures"].tobytes(), np.uint8), texels=d["texels"])
    print("saved", len(d["triangles"]), "triangles")


if __name__ == "__main__":
    main()
