"""The N > 1 host path of bench.py on CPU with the gloo backend: ranks meet
at barriers, the slowest rank's time is what counts, and under torchrun only
rank 0 prints the reference arm's line.  The core itself runs replicas only
(one independent frame per GPU, no collective on the data path)."""
import json
import os
import socket
import subprocess
import sys

import pytest

from common import REPO

torch = pytest.importorskip("torch")


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _max_worker(rank: int, world: int, port: int, q) -> None:
    import torch.distributed as dist

    sys.path.insert(0, str(REPO))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(world)
    q.put((rank, bench.max_over_ranks(1.5 + rank, world)))
    bench.barrier(world)
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_max_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2.5), (1, 2.5)]


def test_reference_arm_under_torchrun_prints_one_line():
    env = dict(os.environ, ARE_REF_STEP_SECONDS="0.3")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(free_port()), "bench.py", "--impl", "reference", "--gpus", "2",
           "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"


def test_rank_gpu_pinning(monkeypatch):
    """Under torchrun each rank narrows CUDA_VISIBLE_DEVICES to its own GPU
    before CUDA starts (the library links its own CUDA runtime, so device 0
    must be the rank's GPU for both it and torch); nvidia-smi keeps the
    physical index.  One process (N = 1) changes nothing."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", REPO / "bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "3,5")
    bench.pin_rank_gpu(2, 1)
    assert os.environ["CUDA_VISIBLE_DEVICES"] == "5" and bench.DEVICE == 0 and bench.SMI_INDEX == 5
    monkeypatch.delenv("CUDA_VISIBLE_DEVICES")
    bench.pin_rank_gpu(4, 2)
    assert os.environ["CUDA_VISIBLE_DEVICES"] == "2" and bench.DEVICE == 0 and bench.SMI_INDEX == 2
    monkeypatch.delenv("CUDA_VISIBLE_DEVICES")
    bench.pin_rank_gpu(1, 0)
    assert "CUDA_VISIBLE_DEVICES" not in os.environ and bench.DEVICE == 0
