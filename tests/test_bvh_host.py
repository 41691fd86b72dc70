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


# Fingerprints (FNV-1a over the binary nodes, the leaf order and the 4-wide
# nodes) of the trees the builder made for these inputs with its append,
# layout, 4-wide collapse and node bounds done serially, one pass per node:
# the threaded phases and the bounds taken from the parent's bins must
# reproduce those trees byte for byte.
SERIAL_BUILD = {(1, 4): "c4fc79dec9708146", (37, 4): "36a1e945e89f77a2", (5000, 2): "f4e986d8a3b5046d",
                (300000, 4): "679c4fc7a64617ca", (300000, 8): "679c4fc7a64617ca"}


@pytest.mark.parametrize("n,leaf", sorted(SERIAL_BUILD))
def test_build_is_deterministic_and_well_formed(harness, n, leaf):
    r = subprocess.run([str(harness), str(n), str(leaf)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr
    assert r.stdout.split("fingerprint")[1].split()[0] == SERIAL_BUILD[(n, leaf)], r.stdout
