"""Batched replicas and graph replay: a replica stepped inside a batch (one
CUDA-graph launch per step for all replicas) gives exactly the results of the
same replica stepped alone, and eph_step replayed from a captured graph
gives exactly the results of direct launches."""
import numpy as np
import pytest

import ephgb
from ephgb import workloads as W

pytestmark = pytest.mark.gpu
KEYS = ("x", "v", "f", "rho", "f_eph", "f_rng", "array")


def replica(beta_file, r):
    cells = (5, 7, 6)[r % 3]
    at = W.fcc_lattice(cells, seed=100 + r)
    if r == 1:
        W.add_pka(at, 500.0, seed=r)
    grid = (cells, cells, cells)
    return W.fix_args(beta_file, seed=1000 + r, grid=grid), at


@pytest.mark.parametrize("mode", [ephgb.MODE_FAST, ephgb.MODE_EXACT])
def test_batch_equals_replicas_alone(built, beta_file, mode):
    reps = [replica(beta_file, r) for r in range(3)]
    batch = ephgb.Batch(reps, dt=0.0005, mode=mode)
    batch.step(6)
    batch.synchronize()
    assert batch.launches_per_step() > 0
    for r, (words, at) in enumerate(reps):
        alone = ephgb.FixEPH(words, at, dt=0.0005, mode=mode)
        alone.step(6)
        got = batch.replicas[r]
        for k in KEYS:
            assert np.array_equal(got.get(k), alone.get(k)), (r, k)
        assert np.array_equal(got.get("T"), alone.get("T"))
        assert got.compute_vector(0) == alone.compute_vector(0)


def test_graph_replay_equals_direct(built, beta_file):
    words, at = replica(beta_file, 1)
    a = ephgb.FixEPH(words, at, dt=0.0005)
    b = ephgb.FixEPH(words, at, dt=0.0005)
    b.set_graph(True)
    a.step(8)
    b.step(5)
    b.step(3)  # replays the same captured step
    for k in KEYS:
        assert np.array_equal(a.get(k), b.get(k)), k
    assert np.array_equal(a.get("T"), b.get("T"))
    assert a.counter("wrap") == b.counter("wrap")
