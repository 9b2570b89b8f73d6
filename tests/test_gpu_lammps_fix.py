"""The LAMMPS fix eph/gb (user-eph_gb300/lammps/fix_eph_gb.cpp) running in
the same engine stand-in as the reference fix: same fix words, same hooks,
the same RanMars deviates drawn in the same order.  In exact mode its
forces, positions, velocities and per-atom array after the first step equal
the oracle's (and so the reference's) bit for bit; later steps agree to
1e-12 (the grid deposits are summed exactly rather than in atom order)."""
import numpy as np
import pytest

from ephgb import workloads as W
from helpers import key_err, n_in_group, scenario
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
                assert np.array_equal(a, b), (name, k, key_err(k, a, b))
            else:
                assert key_err(k, a, b) <= 1e-12, (name, s, k, key_err(k, a, b))
        va, vb = gb.get("vector"), ref.get("vector")
        assert abs(va[1] - vb[1]) <= 1e-12 * abs(vb[1])


def test_fix_eph_gb_peratom_every_n_steps(built, beta_file):
    """`fix_modify ID peratom 3`: the per-atom array is copied back on steps
    3, 6, ... only (and equals the reference's then), while x, v and f keep
    matching every step (here with kept candidate lists, `fix_modify ID
    list_skin 0.3`, and the knock-on atom forcing re-neighbouring)."""
    words, at, dt = scenario("pka", beta_file)
    words = list(words)
    words[2] = "eph/gb"
    gb = GbFix(words, at, dt, 4.6, mode=1, xi_host=1)
    gb.modify("peratom", 3)
    gb.modify("list_skin", 0.3)
    ref = OracleFix(words, at, dt)
    ng = n_in_group(at)
    held = gb.get("array")
    for s in range(1, 10):
        xi = W.gaussian_stream(ng, 31, s)
        gb.step(xi)
        ref.step(xi)
        for k in ("x", "v", "f"):
            assert key_err(k, gb.get(k), ref.get(k)) <= 1e-12, (s, k)
        arr = gb.get("array")
        if s % 3 == 0:
            assert key_err("array", arr, ref.get("array")) <= 1e-12, s
            held = arr
        else:
            assert np.array_equal(arr, held, equal_nan=True), s  # not copied back on this step
    with pytest.raises(RuntimeError):
        gb.modify("peratom", 0)


@pytest.mark.parametrize("pairs", ["fp64", "df64"])
def test_fix_eph_gb_pair_arithmetic(built, beta_file, pairs):
    """`fix_modify ID pairs fp64|df64` (kept when a later `fix_modify ID mode
    fast` makes a new context): both arithmetics match the reference fix to
    1e-12 per atom; other words are an error."""
    words, at, dt = scenario("pka", beta_file)
    words = list(words)
    words[2] = "eph/gb"
    gb = GbFix(words, at, dt, 4.6, mode=1, xi_host=1)
    gb.modify("pairs", pairs)
    gb.modify("mode", "fast")
    ref = OracleFix(words, at, dt)
    ng = n_in_group(at)
    for s in range(8):
        xi = W.gaussian_stream(ng, 31, s)
        gb.step(xi)
        ref.step(xi)
        for k in ("x", "v", "f", "array"):
            assert key_err(k, gb.get(k), ref.get(k)) <= 1e-12, (pairs, s, k)
    with pytest.raises(RuntimeError):
        gb.modify("pairs", "fp32")


def test_fix_eph_gb_list_skin_auto(built, beta_file):
    """`fix_modify ID list_skin auto`: after the first post_force the fix runs
    eph_autotune_list_skin (trial windows of steps on the device, the state
    restored); the run goes on matching the reference fix per atom (16,384
    atoms, one lane per atom, a knock-on atom)."""
    at = W.fcc_lattice(16, seed=93, temperature=300.0)
    W.add_pka(at, 1000.0, seed=94)
    words = W.fix_args(beta_file, grid=(8, 8, 8))
    words[2] = "eph/gb"
    gb = GbFix(words, at, 0.0005, 4.6, mode=1, xi_host=1)
    gb.modify("list_skin", "auto")
    ref = OracleFix(words, at, 0.0005)
    ng = n_in_group(at)
    for s in range(6):
        xi = W.gaussian_stream(ng, 37, s)
        gb.step(xi)
        ref.step(xi)
        for k in ("x", "v", "f", "array"):
            assert key_err(k, gb.get(k), ref.get(k)) <= 1e-12, (s, k, key_err(k, gb.get(k), ref.get(k)))
