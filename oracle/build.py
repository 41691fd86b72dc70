"""Build recipe for the oracle (TEST INFRASTRUCTURE ONLY).

* ``build_oracle()`` compiles the C restatement (orc_*.c) into
  ``oracle/_build/liborc.so`` with ``-ffp-contract=off`` so FP32 results do
  not depend on the host's FMA contraction defaults (gcc contracts by default
  on aarch64).
* ``build_ref(ref_root)`` compiles the reference's own sources where they lie
  (experiments/rt.cpp through ``ref_rt_harness.cpp``; src/**/*.cpp through
  ``ref_lib_harness.cpp``) into ``oracle/_ref/``.  It only runs where the
  reference tree exists; nothing is copied out of it.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
# where the reference tree lies in the development container (absent on GPU hosts)
REF_ROOT = Path(os.environ.get("ARE_REFERENCE_ROOT", "/root/reference"))
ORACLE_SOURCES = ["orc_common.c", "orc_f32.c", "orc_f64.c", "orc_legacy.c", "orc_guide.c"]
REF_LIB_SOURCES = [
    "src/basic/vec3.cpp",
    "src/basic/ray.cpp",
    "src/basic/plane.cpp",
    "src/object/object.cpp",
    "src/object/triangle.cpp",
    "src/material/material.cpp",
    "src/material/diffuse.cpp",
    "src/material/reflective.cpp",
    "src/texture.cpp",
]


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + res.stdout + res.stderr)


def _stale(out: Path, inputs: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(p.stat().st_mtime > t for p in inputs)


def build_oracle(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    out = BUILD / "liborc.so"
    deps = [HERE / s for s in ORACLE_SOURCES] + [HERE / "orc.h", HERE / "orc_internal.h", HERE / "orc_core.inc"]
    if force or _stale(out, deps):
        tmp = out.with_suffix(".so.tmp%d" % os.getpid())
        _run(["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread",
              "-o", str(tmp)] + [str(HERE / s) for s in ORACLE_SOURCES] + ["-lm"])
        os.replace(tmp, out)
    return out


def build_ref(ref_root: str | os.PathLike = REF_ROOT, force: bool = False) -> list[Path]:
    """Compile the reference's sources into oracle/_ref (returns the .so paths)."""
    root = Path(ref_root)
    if not (root / "experiments" / "rt.cpp").exists():
        return []
    REF_OUT.mkdir(exist_ok=True)
    flags = ["-std=c++20", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w"]
    jobs = []
    rt_out = REF_OUT / "libref_rt.so"
    rt_deps = [HERE / "ref_rt_harness.cpp", root / "experiments" / "rt.cpp"]
    if force or _stale(rt_out, rt_deps):
        jobs.append(["g++", *flags, "-I", str(root), "-o", str(rt_out), str(HERE / "ref_rt_harness.cpp")])
    lib_out = REF_OUT / "libref_lib.so"
    lib_deps = [HERE / "ref_lib_harness.cpp"] + [root / s for s in REF_LIB_SOURCES]
    if force or _stale(lib_out, lib_deps):
        jobs.append(["g++", *flags, "-I", str(root / "include"), "-o", str(lib_out), str(HERE / "ref_lib_harness.cpp")]
                    + [str(root / s) for s in REF_LIB_SOURCES])
    with ThreadPoolExecutor(max_workers=2) as ex:
        list(ex.map(_run, jobs))
    return [rt_out, lib_out]


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
