"""The oracle against the golden fixtures written by the reference fix itself
(tests/golden, generated by make_golden.py): bit-identical.  Runs wherever
the oracle builds, including hosts without the reference tree."""
import numpy as np
import pytest

from golden_io import FIXTURES, GOLDEN, REF_FIXTURES, fixture_steps, fixture_xi, load_fix
from oracle.bindings import OracleFix

LAST_ONLY = ("f_eph", "f_rng", "w", "array")


@pytest.mark.parametrize("name", FIXTURES + REF_FIXTURES)
def test_oracle_matches_golden(built, tmp_path, name):
    """Every recorded step bit for bit.  The REF_FIXTURES run the reference's
    own input files: Tests/MD_Run (the deck's fix line `eph 1111 7 4 1.0 3.5e-6
    0.1248 0.0 7 8 9 NULL 0 T_out Ni.beta Ni Ni` with its Ni.beta: T_e = 0, a
    7x8x9 grid, two types on one element), Tests/EPH_Beta_zero (rho_cutoff 5,
    crossed by a knock-on atom: beta = alpha = 0 above it), the four-element
    NiCoCrFe beta file, and Examples/Example_4 (its atoms, grid file T.in and
    beta file)."""
    words, at, dt, rec = load_fix(name, str(tmp_path))
    o = OracleFix(words, at, dt)
    nsteps, recorded = fixture_steps(rec)
    for s in range(nsteps):
        xi = fixture_xi(rec, words, at, s)
        o.step(xi if xi is not None and xi.size else None)
        if s not in recorded:
            continue
        r = recorded.index(s)
        for k in ("x", "v", "f", "rho", "vector", "T"):
            assert np.array_equal(o.get(k), rec[k][r]), (name, s, k)
    for k in LAST_ONLY:
        assert np.array_equal(o.get(k), rec[k]), (name, k)


def test_beta_zero_fixture_crosses_rho_cutoff(tmp_path):
    """The Tests/EPH_Beta_zero fixture exercises the rho > rho_cutoff branch
    (eph_beta.h:174-197): some recorded step has an atom above rho_cutoff = 5,
    whose beta column in the per-atom array is 0."""
    words, at, dt, rec = load_fix("beta_zero", str(tmp_path))
    assert (rec["rho"] > 5.0).any()
    assert (rec["rho"] < 5.0).all(axis=1)[-1]  # and the pair has left the region again


def test_fdm_test1_golden(built):
    """The reference's FDM golden vectors (Tests/EPH_FDM/Test1/Out_Ref): a
    1000x1x1 grid over [-10, 10], C_e 2, kappa 2, rho_e 1, T 1, dt 1e-3, a
    source Q = 10 in the cell at x = 0 while t < 1.  The shipped files hold
    %.6e values and come from an older driver, so they pin the solver to the
    precision they carry: 1e-4 relative at t = 1, 2e-6 at t = 8."""
    from oracle.bindings import oracle_lib
    import ctypes as C
    import os

    lib = oracle_lib()
    g = lib.orc_fdm_create(1000, 1, 1, -10.0, 10.0, -1.0, 1.0, -1.0, 1.0, 1.0, 2.0, 1.0, 2.0)
    lib.orc_fdm_set_dt(g, 1e-3)
    gold = np.load(os.path.join(GOLDEN, "fdm_test1.npz"))
    T = np.zeros(1000)
    try:
        for i in range(0, 8001):
            if i * 1e-3 < 1.0:
                lib.orc_fdm_insert_energy(g, 1e-9, 0.0, 0.0, 10.0 * 1e-3)
            lib.orc_fdm_solve(g)
            if i in (1000, 8000):
                lib.orc_fdm_get(g, 0, T.ctypes.data_as(C.POINTER(C.c_double)))
                k = i // 1000
                rel = np.abs(T - gold[f"T{k}"]).max() / np.abs(gold[f"T{k}"]).max()
                assert rel < (1e-4 if k == 1 else 2e-6), (k, rel)
    finally:
        lib.orc_fdm_free(g)
