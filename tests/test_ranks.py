"""The multi-GPU form of the bench is replicas only: every rank steps its own
copy of the workload, the time is the slowest rank's, throughputs of
independent replicas add up, and rank 0 alone prints.  Checked on the CPU
with two gloo ranks (no GPU needed): the reductions bench.py uses, and the
reference arm under torchrun."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch

    sys.path.insert(0, ROOT)
    import bench

    torch.distributed.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                                         world_size=world)
    try:
        ms = 10.0 + 5.0 * rank  # the slowest rank sets the time
        t = bench.ranks_reduce(ms, "max", "cpu")
        v = bench.ranks_reduce(1.0e8 * (rank + 1), "sum", "cpu")
        out[rank] = (t, v, bench.job_value(world, 1000, 20, t))
    finally:
        torch.distributed.destroy_process_group()


def test_rank_reductions_gloo():
    import torch.multiprocessing as mp

    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        t, v, val = res[rank]
        assert t == 15.0
        assert v == 3.0e8
        assert val == pytest.approx(2 * 1000 * 20 / 0.015)


def test_single_process_reduction_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.ranks_reduce(12.5, "max", "cpu") == 12.5
    assert bench.job_value(1, 4000, 10, 2.0) == pytest.approx(4000 * 10 / 0.002)


def test_reference_arm_under_torchrun(built):
    """Two ranks: rank 0 times the reference algorithm on the host and prints
    one line; rank 1 exits 0 without work (a small lattice keeps it quick)."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1", "--cells", "6", "--grid", "6"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
