"""Temperature-dependent grid cells (the T_dynamic column of a grid file,
eph_fdm.h:73-104, :280-287, :378-382): C_e(T) and kappa_e(T) splines and the
E_e(T) inverse update.  The oracle's grid solve and the product's host-side
reader/writer against the reference's EPH_FDM, and the fix with such a grid
against the reference fix."""
import filecmp
import os

import numpy as np
import pytest

import ephgb
from ephgb import workloads as W
from helpers import n_in_group
from oracle.bindings import OracleFix, RefFix, RefGrid, oracle_lib, ref_available

needs_ref = pytest.mark.skipif(not ref_available(), reason="reference build (oracle/_ref) absent")


def tdyn_grid(tmp_path, T=2000.0):
    pf = W.write_grid_parameters(str(tmp_path / "params.data"))
    return W.write_grid_file(str(tmp_path / "Tdyn.in"), parameter_file=pf, tdyn=True, T=T)


@needs_ref
def test_oracle_solve_is_the_reference(built, tmp_path):
    import ctypes as C

    gf = tdyn_grid(tmp_path)
    r = RefGrid(path=gf)
    r.set_dt(1e-3)
    lib = oracle_lib()
    o = lib.orc_fdm_load(gf.encode())
    lib.orc_fdm_set_dt(o, 1e-3)
    try:
        n = lib.orc_fdm_ncells(o)
        T0 = np.zeros(n)
        lib.orc_fdm_get(o, 0, T0.ctypes.data_as(C.POINTER(C.c_double)))
        for _ in range(25):
            r.solve()
            lib.orc_fdm_solve(o)
        T = np.zeros(n)
        lib.orc_fdm_get(o, 0, T.ctypes.data_as(C.POINTER(C.c_double)))
        L, (nx, ny, nz) = 17.6, (8, 6, 5)
        Tr = np.array([r.get_T((i + 0.5) * L / nx, (j + 0.5) * L / ny, (k + 0.5) * L / nz)
                       for k in range(nz) for j in range(ny) for i in range(nx)])
        assert np.array_equal(T, Tr)
        assert np.abs(T - T0).max() > 1.0  # the T-dependent cells evolved
        r.save_state(str(tmp_path / "r.restart"))
        lib.orc_fdm_save_state(o, str(tmp_path / "o.restart").encode())
        assert filecmp.cmp(tmp_path / "r.restart", tmp_path / "o.restart", shallow=False)
    finally:
        lib.orc_fdm_free(o)


@needs_ref
def test_host_reader_writer_with_parameter_file(built, tmp_path):
    gf = tdyn_grid(tmp_path)
    ephgb.Grid(path=gf).save_state(str(tmp_path / "g.restart"))
    RefGrid(path=gf).save_state(str(tmp_path / "r.restart"))
    assert filecmp.cmp(tmp_path / "g.restart", tmp_path / "r.restart", shallow=False)


@needs_ref
def test_fix_with_tdyn_grid_oracle_is_reference(built, beta_file, tmp_path):
    gf = tdyn_grid(tmp_path)
    at = W.fcc_lattice(5, seed=61)
    words = W.fix_args(beta_file, T_infile=gf, grid=(1, 1, 1))
    o = OracleFix(words, at, 0.001)
    r = RefFix(words, at, 0.001)
    for s in range(8):
        xi = W.gaussian_stream(n_in_group(at), 3, s)
        o.step(xi)
        r.step(xi)
        for k in ("rho", "f_eph", "f_rng", "f", "x", "v", "array", "vector"):
            assert np.array_equal(o.get(k), r.get(k)), (s, k)
