"""The CPU restatement (oracle/eph_oracle.c) against the reference fix itself
(fix_eph.cpp and the eph_*.h headers compiled unchanged with the engine
stand-in): bit-identical on every per-atom array, the grid and the vector.
Needs the reference tree at build time (oracle/_ref); skipped elsewhere, where
tests/golden pins the oracle instead."""
import numpy as np
import pytest

from oracle.bindings import OracleFix, RefFix, ref_available
from helpers import SCENARIOS, n_in_group, scenario
from ephgb import workloads as W

pytestmark = pytest.mark.skipif(not ref_available(), reason="reference build (oracle/_ref) absent")


@pytest.mark.parametrize("name", SCENARIOS)
def test_oracle_is_the_reference(built, beta_file, beta_file_2el, name):
    words, at, dt = scenario(name, beta_file, beta_file_2el)
    o = OracleFix(words, at, dt)
    r = RefFix(words, at, dt)
    grid = (int(words[10]), int(words[11]), int(words[12]))
    ng = n_in_group(at)
    steps = 12 if name != "pka" else 40
    for s in range(steps):
        xi = W.gaussian_stream(ng, 5, s) if int(words[4], 0) & 2 else None
        o.step(xi)
        r.step(xi)
        for k in ("rho", "w", "f_eph", "f_rng", "f", "x", "v", "array", "vector"):
            assert np.array_equal(o.get(k), r.get(k)), (name, s, k)
        assert np.array_equal(o.get("T"), r.get_T(grid, at.boxlo, at.boxhi)), (name, s, "T")
    assert o.nbuild == r.nbuild
    if name == "pka":
        assert o.nbuild > 1


def test_neighbour_lists_match(built, beta_file):
    words, at, dt = scenario("c1_small", beta_file)
    o = OracleFix(words, at, dt)
    r = RefFix(words, at, dt)
    no, oo = o.neighbours()
    nr, orr = r.neighbours()
    assert np.array_equal(no, nr) and np.array_equal(oo, orr)
