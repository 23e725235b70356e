"""The multi-GPU form is replicas only (every rank joins its own copy of the
workload; no data-path collective).  Its host logic -- max-over-ranks step
time, whole-job throughput, rank 0 alone printing the reference arm -- runs
here as two gloo ranks on the CPU."""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, world)  # rank 1 is the slow replica
    value = bench.job_points_per_s(1000, world, ms)
    dist.barrier()
    out[rank] = (ms, value)
    dist.destroy_process_group()


def _free_port():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_replicas_report_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    assert res[0] == res[1]
    ms, value = res[0]
    assert ms == 15.0
    assert value == pytest.approx(2 * 1000 / 15e-3)


def test_single_rank_is_unchanged():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(7.5, 1) == 7.5
    assert bench.job_points_per_s(100, 1, 10.0) == pytest.approx(1e4)


def test_reference_arm_under_two_ranks_prints_once(tmp_path):
    """`bench.py --impl reference` under torchrun: rank 0 runs and prints one
    line, the other rank exits 0 without work (no GPU is touched)."""
    env = dict(os.environ, MASTER_ADDR="127.0.0.1")
    port = str(_free_port())
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", port, os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--workload", "uniform18", "--points", "3000",
           "--steps", "1", "--warmup", "0", "--ref-seconds", "0.2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    j = json.loads(lines[0])
    assert j["impl"] == "reference" and j["n_gpus"] == 2 and j["value"] > 0
