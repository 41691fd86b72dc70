"""FP64 CPU reference of the occluded-light Cornell box (guiding evaluation).

The oracle's FP64 path estimator (oracle/orc_f64.c) renders the occluded
Cornell workload (600x600, the workload's own frame, or 200x200 with the
same camera, which finishes in minutes rather than hours) at 65,536 samples
per pixel, depth 16, Russian roulette from depth 3, as 64 independent
1,024-spp passes with different seeds.  The mean image and its per-pixel
variance of the mean are saved as float32 to
tests/golden/guiding_reference_<res>.npz; partial progress is kept in
baseline/_ref/ so an interrupted run resumes (a 600x600 pass is 369 M FP64
samples: about three hours on six cores for the whole reference).

Usage: python tests/golden/make_guiding_reference.py [passes] [threads] [res]
"""
from __future__ import annotations

import os
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "tests"))

from common import are  # noqa: E402
from oracle.orc import Oracle  # noqa: E402

PASS_SPP = 1024


def main() -> None:
    passes = int(sys.argv[1]) if len(sys.argv) > 1 else 64
    threads = int(sys.argv[2]) if len(sys.argv) > 2 else (os.cpu_count() or 1)
    res = int(sys.argv[3]) if len(sys.argv) > 3 else 200
    part = REPO / "baseline" / "_ref" / ("guiding_reference_partial.npz" if res == 200 else
                                         f"guiding_reference_partial_{res}.npz")
    part.parent.mkdir(parents=True, exist_ok=True)
    s, cam, par = are.build_config(are.CONFIG_CORNELL_OCCLUDED)
    par = dict(par, width=res, height=res, spp=PASS_SPP)
    orc = Oracle()
    ctx = orc.prepare(s)
    done, s1, s2 = 0, np.zeros((res, res, 3)), np.zeros((res, res, 3))
    if part.exists():
        z = np.load(part)
        done, s1, s2 = int(z["done"]), z["s1"], z["s2"]
    while done < passes:
        t = time.time()
        m, v, st = orc.render(ctx, cam, dict(par, seed=100_000 + done), fp64=True, nthreads=threads)
        # per pass: mean m and variance of its mean v; combine passes exactly
        s1 += m
        s2 += v * PASS_SPP * (PASS_SPP - 1) + PASS_SPP * m * m  # sum of squares of the pass's samples
        done += 1
        np.savez(part, done=done, s1=s1, s2=s2)
        print(f"pass {done}/{passes} {time.time() - t:.1f}s", flush=True)
    n = done * PASS_SPP
    mean = s1 / done
    var = (s2 - n * mean * mean) / (n - 1) / n
    np.savez_compressed(HERE / f"guiding_reference_{res}.npz", mean=mean.astype(np.float32),
                        var=np.maximum(var, 0).astype(np.float32), spp=n, width=res, height=res,
                        config=are.CONFIG_CORNELL_OCCLUDED)
    print("saved", n, "spp")


if __name__ == "__main__":
    main()
