"""Build recipe for libaurora_gb300.so (the product).

Compiles csrc/*.cu and csrc/*.cpp with nvcc for sm_103a only, in parallel,
into aurora-rendering-engine_gb300/_build/, and links one shared library with
the CUDA runtime linked statically (no torch, no other runtime dependency).
Host code is compiled with -ffp-contract=off so it does not depend on the
host compiler's contraction default (gcc contracts by default on aarch64).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
CSRC = HERE / "csrc"
OUT = HERE / "_build"
LIB = OUT / "libaurora_gb300.so"
CLI_SRC = HERE / "cli" / "are_render.cpp"
CLI = OUT / "are_render"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    raise FileNotFoundError("nvcc not found")


def _sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((REPO / "include").glob("*.h")))


def _run(cmd: list[str]) -> str:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def compile_one(src: Path, extra: list[str] | None = None) -> Path:
    obj = OUT / (src.name + ".o")
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
           "-I", str(REPO / "include"), "-I", str(CSRC), "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cu":
        cmd += ["-Xptxas", "-v"] if extra and "-v" in extra else []
    _run(cmd)
    return obj


def build(force: bool = False, jobs: int | None = None) -> Path:
    OUT.mkdir(exist_ok=True)
    srcs = _sources()
    newest_hdr = max((h.stat().st_mtime for h in _headers()), default=0)
    todo = []
    for s in srcs:
        obj = OUT / (s.name + ".o")
        if force or not obj.exists() or obj.stat().st_mtime < max(s.stat().st_mtime, newest_hdr):
            todo.append(s)
    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(compile_one, todo))
    objs = [OUT / (s.name + ".o") for s in srcs]
    if force or todo or not LIB.exists():
        tmp = LIB.with_name(LIB.name + ".tmp%d" % os.getpid())
        _run([nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs), "-lpthread", "-ldl",
              "-lrt"])
        os.replace(tmp, LIB)
    build_cli(force)
    return LIB


def build_cli(force: bool = False) -> Path:
    """The command-line renderer, a C++ program over include/aurora_gb300.hpp
    linked against the library (found next to it at run time)."""
    deps = [CLI_SRC, LIB, REPO / "include" / "aurora_gb300.hpp", REPO / "include" / "aurora_gb300.h"]
    if force or not CLI.exists() or CLI.stat().st_mtime < max(d.stat().st_mtime for d in deps):
        cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
        tmp = CLI.with_name(CLI.name + ".tmp%d" % os.getpid())
        _run([cxx, "-O2", "-std=c++17", "-Wall", "-I", str(REPO / "include"), str(CLI_SRC), "-o", str(tmp),
              "-L", str(OUT), "-laurora_gb300", "-Wl,-rpath,$ORIGIN"])
        os.replace(tmp, CLI)
    return CLI


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
