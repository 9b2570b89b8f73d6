"""The product's host side (beta file reader, spline construction, grid
files, stability substeps) against the reference: the device tables must be
the reference's tables to the last bit."""
import filecmp
import os

import numpy as np
import pytest

import ephgb
from ephgb import workloads as W
from golden_io import GOLDEN, write_ref_input
from oracle.bindings import RefBeta, RefGrid, oracle_lib, ref_available

needs_ref = pytest.mark.skipif(not ref_available(), reason="reference build (oracle/_ref) absent")


def test_spline_tables_match_golden(built, beta_file):
    b = ephgb.BetaFile(beta_file)
    g = np.load(os.path.join(GOLDEN, "beta_tables.npz"))
    for w, name in enumerate(("rho_r", "rho_r_sq", "beta", "alpha")):
        assert np.array_equal(b.table(name, 0), g[f"t{w}"]), name
    assert np.array_equal(b.eval("rho_r_sq", 0, g["r2"]), g["rho_r_sq"])
    assert np.array_equal(b.eval("beta", 0, g["rho"]), g["beta"])
    assert np.array_equal(b.eval("alpha", 0, g["rho"]), g["alpha"])
    assert b.r_cutoff == g["rc"] and b.rho_cutoff == g["rho_cut"]


@needs_ref
@pytest.mark.parametrize("which", [0, 1, 2, 3])
def test_spline_tables_match_reference(built, beta_file_2el, which):
    b = ephgb.BetaFile(beta_file_2el)
    r = RefBeta(beta_file_2el)
    name = ("rho_r", "rho_r_sq", "beta", "alpha")[which]
    for e in range(2):
        assert np.array_equal(b.table(name, e), r.table(which, e))


@needs_ref
@pytest.mark.parametrize("name", ["MD_Run_Ni.beta", "Beta_zero_Ni.beta", "NiCoCrFe_PRB2019.beta"])
def test_real_reference_beta_file(built, tmp_path, name):
    """The reference's own beta files (Tests/MD_Run/Ni.beta: 1001 rho knots,
    50001 beta knots; Tests/EPH_Beta_zero/Ni.beta; the four-element
    NiCoCrFe file), kept under tests/golden/ref_inputs: host tables of every
    element bit-identical to the reference's EPH_Beta."""
    path = write_ref_input(name, str(tmp_path))
    b = ephgb.BetaFile(path)
    r = RefBeta(path)
    nel = 4 if name.startswith("NiCoCrFe") else 1
    for e in range(nel):
        for which, tab in enumerate(("rho_r", "rho_r_sq", "beta", "alpha")):
            assert np.array_equal(b.table(tab, e), r.table(which, e)), (tab, e)
        xs = np.linspace(0, 0.999 * r.r_cutoff ** 2, 101)
        assert np.array_equal(b.eval("rho_r_sq", e, xs), r.eval(1, e, xs))
    assert b.rho_cutoff == r.rho_cutoff and b.r_cutoff == r.r_cutoff


def test_spline_tables_match_oracle(built, beta_file):
    lib = oracle_lib()
    ob = lib.orc_beta_load(beta_file.encode())
    b = ephgb.BetaFile(beta_file)
    import ctypes as C

    try:
        for w, name in enumerate(("rho_r", "rho_r_sq", "beta", "alpha")):
            n = lib.orc_beta_table(ob, w, 0, None)
            out = np.zeros((n, 4))
            lib.orc_beta_table(ob, w, 0, out.ctypes.data_as(C.POINTER(C.c_double)))
            assert np.array_equal(out, b.table(name, 0)), name
    finally:
        lib.orc_beta_free(ob)


def grid_file(path, n=(6, 5, 4), box=(0.0, 12.0, -3.0, 7.0, 1.0, 9.0), seed=0):
    """A grid file in the reference format with every cell kind."""
    rng = np.random.default_rng(seed)
    with open(path, "w") as f:
        f.write("# grid\n#\n#\n")
        f.write(f"{n[0]} {n[1]} {n[2]} 2\n")
        f.write(f"{box[0]:.6e} {box[1]:.6e}\n{box[2]:.6e} {box[3]:.6e}\n{box[4]:.6e} {box[5]:.6e}\nNULL\n")
        for k in range(n[2]):
            for j in range(n[1]):
                for i in range(n[0]):
                    flag = 1
                    if i == 0:
                        flag = 2
                    elif j == 0 and k == 0:
                        flag = 0
                    T = rng.uniform(200, 2000)
                    S = rng.uniform(-1, 1) if flag == 1 and i == 3 else 0.0
                    f.write(f"{i} {j} {k} {T:.6e} {S:.6e} {rng.uniform(0.5, 1.5):.6e} {rng.uniform(1e-6, 5e-6):.6e} "
                            f"{rng.uniform(0.05, 0.2):.6e} {flag} 0\n")
    return path


@needs_ref
def test_grid_files_and_substeps(built, tmp_path):
    p = grid_file(str(tmp_path / "T.in"))
    g = ephgb.Grid(path=p)
    r = RefGrid(path=p)
    for dt in (1e-3, 5e-4, 1e-2):
        n, idt = g.substeps(dt)
        assert n >= 1 and idt > 0
    g.save_state(str(tmp_path / "a.restart"))
    r.save_state(str(tmp_path / "b.restart"))
    assert filecmp.cmp(tmp_path / "a.restart", tmp_path / "b.restart", shallow=False)
    g.save_temperature(str(tmp_path / "ta"), 3)
    r.save_temperature(str(tmp_path / "tb"), 3)
    assert filecmp.cmp(tmp_path / "ta_000003", tmp_path / "tb_000003", shallow=False)
    # uniform grid written by the fix constructor path
    lo, hi = np.array([0.0, 0.0, 0.0]), np.array([35.2, 35.2, 35.2])
    gu = ephgb.Grid(n=(10, 10, 10), lo=lo, hi=hi, T_e=300.0, C_e=3.5e-6, rho_e=1.0, kappa_e=0.1)
    ru = RefGrid(n=(10, 10, 10), lo=lo, hi=hi, T=300.0, Ce=3.5e-6, rho=1.0, kappa=0.1)
    gu.save_state(str(tmp_path / "u1"))
    ru.save_state(str(tmp_path / "u2"))
    assert filecmp.cmp(tmp_path / "u1", tmp_path / "u2", shallow=False)


def test_substep_count_matches_oracle_solver(built):
    """eph_grid_substeps is the count EPH_FDM::solve takes (eph_fdm.h:275-313)."""
    lib = oracle_lib()
    lo, hi = np.zeros(3), np.full(3, 281.6)
    for dt, ng in ((5e-4, 64), (1e-3, 10), (1e-3, 16)):
        h = np.full(3, 281.6 if ng == 64 else (35.2 if ng == 10 else 70.4))
        g = ephgb.Grid(n=(ng, ng, ng), lo=lo, hi=h, T_e=300.0, C_e=3.5e-6, rho_e=1.0, kappa_e=0.1)
        o = lib.orc_fdm_create(ng, ng, ng, 0.0, h[0], 0.0, h[1], 0.0, h[2], 300.0, 3.5e-6, 1.0, 0.1)
        lib.orc_fdm_set_dt(o, dt)
        try:
            assert g.substeps(dt)[0] == lib.orc_fdm_solve(o)
        finally:
            lib.orc_fdm_free(o)
