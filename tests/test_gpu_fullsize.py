"""The bench workload at full size — fcc Ni 80^3 cells (2,048,000 atoms), a
10 keV primary knock-on atom, 64^3 grid, dt 0.5 fs, flags 7, model 4 — checked
through properties that do not depend on the size:

* two steps against the oracle (the CPU restatement, run on all host cores)
  with the same injected deviates: FAST within 1e-12 per atom
  (helpers.atom_err), EXACT bit-identical on the first step;
* momentum: the friction pair terms are antisymmetric in (i, j), so
  sum_i f_EPH,i vanishes up to rounding; so does sum_i f_RNG,i while T_e is
  uniform (the first step: each atom's random force is scaled by the T_e of
  its own cell);
* energy: with uniform C_e, kappa_e and periodic boundaries the grid solve
  conserves sum_c rho_e C_e T_c dV, so the grid gains exactly the energy the
  ions gave up (E_e, the fix's first output);
* run to run: two contexts on the same atoms (one stepping directly, one
  replaying a captured graph) stay bit-identical."""
import os

import numpy as np
import pytest

import ephgb
from ephgb import workloads as W
from helpers import atom_err, key_err, n_in_group, xi_rows
from oracle.bindings import OracleFix

pytestmark = pytest.mark.gpu
TOL = 1e-12
CELLS, GRID, DT, PKA_EV, SEED = 80, (64, 64, 64), 0.0005, 10000.0, 4242
ATOM_KEYS = ("rho", "w", "f_eph", "f_rng", "f", "x", "v")


@pytest.fixture(scope="module")
def system(tmp_path_factory):
    wd = tmp_path_factory.mktemp("full")
    bf = W.write_beta_file(os.path.join(str(wd), "synth.beta"))
    atoms = W.fcc_lattice(CELLS, seed=SEED)
    W.add_pka(atoms, PKA_EV, seed=SEED + 1)
    words = W.fix_args(bf, seed=SEED, flags=7, model=4, grid=GRID, T_out=os.path.join(str(wd), "Te_out"))
    assert atoms.n == 2048000
    return words, atoms


@pytest.mark.parametrize("mode", [ephgb.MODE_FAST, ephgb.MODE_EXACT])
def test_full_size_against_oracle(built, system, mode):
    words, at = system
    gpu = ephgb.FixEPH(words, at, dt=DT, mode=mode)
    ref = OracleFix(words, at, DT, threads=os.cpu_count() or 1)
    ng = n_in_group(at)
    for s in range(2):
        stream = W.gaussian_stream(ng, 5, s)
        gpu.step(1, xi=xi_rows(at, stream))
        ref.step(stream)
        for k in ATOM_KEYS:
            a, b = gpu.get(k), ref.get(k)
            if mode == ephgb.MODE_EXACT and s == 0:
                assert np.array_equal(a, b), (k, key_err(k, a, b))
            else:
                assert key_err(k, a, b) <= TOL, (s, k, key_err(k, a, b))
        assert atom_err(gpu.get("T"), ref.get("T")) <= TOL, (s, atom_err(gpu.get("T"), ref.get("T")))


def test_full_size_momentum_and_energy(built, system):
    words, at = system
    gpu = ephgb.FixEPH(words, at, dt=DT, mode=ephgb.MODE_FAST)
    grid = gpu.get("T")
    ncell = grid.size
    rho_e, C_e = float(words[6]), float(words[7])  # fix ID group eph seed flags model rho_e C_e ...
    dV = float(np.prod((at.boxhi - at.boxlo) / np.array(GRID)))
    assert ncell == int(np.prod(GRID))
    Ee0, T0 = gpu.compute_vector(0), grid.astype(np.float64).sum()
    for s in range(4):
        gpu.step(1)
        for k in ("f_eph", "f_rng") if s == 0 else ("f_eph",):
            f = gpu.get(k)
            scale = np.abs(f).sum(axis=0)
            assert np.all(np.abs(f.sum(axis=0)) <= 1e-12 * scale), (s, k, f.sum(axis=0), scale)
        Ee1, T1 = gpu.compute_vector(0), gpu.get("T").sum()
        gained = rho_e * C_e * dV * (T1 - T0)
        given = Ee1 - Ee0
        assert abs(given) > 0.0
        assert abs(gained - given) <= 1e-9 * abs(given) + 1e-12 * rho_e * C_e * dV * T0, (s, gained, given)
        Ee0, T0 = Ee1, T1


def test_full_size_run_to_run_and_graph(built, system):
    import torch

    words, at = system
    a = ephgb.FixEPH(words, at, dt=DT, mode=ephgb.MODE_FAST)
    b = ephgb.FixEPH(words, at, dt=DT, mode=ephgb.MODE_FAST)
    stream = torch.cuda.Stream()  # graphs are not captured on the legacy default stream
    b.set_stream(stream.cuda_stream)
    b.set_graph(True)
    a.step(5)
    b.step(5)
    a.synchronize()
    b.synchronize()
    for k in ("x", "v", "f", "f_eph", "f_rng", "rho", "T"):
        assert np.array_equal(a.get(k), b.get(k)), k
    assert a.compute_vector(0) == b.compute_vector(0)
