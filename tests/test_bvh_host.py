"""The host BVH builder (csrc/bvh.cpp) on its own, compiled with the host
compiler: deterministic across runs (its large subtrees are built by worker
threads), complete and well formed.  No GPU needed."""
import shutil
import subprocess

import pytest

from common import REPO


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    out = tmp_path_factory.mktemp("bvh") / "bvh_check"
    csrc = REPO / "aurora-rendering-engine_gb300" / "csrc"
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(csrc), "-I", str(REPO / "include"),
           "-I", "/usr/local/cuda/include", str(REPO / "tests" / "harness" / "bvh_check.cpp"), str(csrc / "bvh.cpp"),
           "-o", str(out), "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


@pytest.mark.parametrize("n,leaf", [(1, 4), (37, 4), (5000, 2), (300000, 4), (300000, 8)])
def test_build_is_deterministic_and_well_formed(harness, n, leaf):
    r = subprocess.run([str(harness), str(n), str(leaf)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr
