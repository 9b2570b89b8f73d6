"""The LAMMPS fix eph/gb (user-eph_gb300/lammps/fix_eph_gb.cpp) running in
the same engine stand-in as the reference fix: same fix words, same hooks,
the same RanMars deviates drawn in the same order.  In exact mode its
forces, positions, velocities and per-atom array after the first step equal
the oracle's (and so the reference's) bit for bit; later steps agree to
1e-12 (the grid deposits are summed exactly rather than in atom order)."""
import numpy as np
import pytest

from ephgb import workloads as W
from helpers import n_in_group, rel_err, scenario
from oracle.bindings import GbFix, OracleFix

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["c1_small", "group", "pka", "two_elements", "noint"])
@pytest.mark.parametrize("mode", [0, 1])
def test_fix_eph_gb_in_engine(built, beta_file, beta_file_2el, name, mode):
    words, at, dt = scenario(name, beta_file, beta_file_2el)
    words = list(words)
    words[2] = "eph/gb"
    rc = 4.6
    gb = GbFix(words, at, dt, rc, mode=mode, xi_host=1)
    ref = OracleFix(words, at, dt)
    ng = n_in_group(at)
    rnd = int(words[4], 0) & 2
    steps = 25 if name == "pka" else 5
    for s in range(steps):
        xi = W.gaussian_stream(ng, 31, s) if rnd else None
        gb.step(xi)
        ref.step(xi)
        for k in ("x", "v", "f", "array"):
            a, b = gb.get(k), ref.get(k)
            if mode == 0 and s == 0:
                assert np.array_equal(a, b), (name, k, rel_err(a, b))
            else:
                assert rel_err(a, b) <= 1e-12, (name, s, k, rel_err(a, b))
        va, vb = gb.get("vector"), ref.get("vector")
        assert abs(va[1] - vb[1]) <= 1e-12 * abs(vb[1])
