"""The engine's eam/alloy pair force on the GPU (eph_set_pair_eam): against a
numpy restatement that reads the setfl file and builds its tables on its own
(oracle/eam_ref.py), against the gradient of its own energy, at rest in the
perfect lattice, and energy conservation of plain NVE.  Two potentials: a
generated Sutton-Chen Ni setfl (6 A cut-off) and the reference decks' own
Tests/MD_Run/Ni.eam (10001-point tables, 6.5 A cut-off; kept under
tests/golden/ref_inputs).  FAST mode sums the pair terms in double-float
(the default) or in FP64; both are checked.  LAMMPS itself is not available
here: what ties the pair force to LAMMPS's pair_style eam/alloy is the
reference's MD_Run deck against its LAMMPS output
(tests/test_gpu_md_run_deck.py); the tables follow the same cubic Hermite
scheme with five-point slopes."""
import numpy as np
import pytest

import ephgb
from ephgb import workloads as W
from golden_io import write_ref_input
from helpers import key_err
from oracle.eam_ref import energy_forces, read_setfl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=["sutton_chen_Ni", "MD_Run_Ni"])
def setfl(request, tmp_path_factory):
    d = str(tmp_path_factory.mktemp("eam"))
    if request.param == "MD_Run_Ni":
        return write_ref_input("MD_Run_Ni.eam", d)
    return W.write_eam_sutton_chen(d + "/SC_Ni.eam")


def forces_at(setfl, beta_file, at, mode=ephgb.MODE_FAST, pairs=ephgb.PAIRS_DF64):
    """EAM forces and energy at the atoms' positions: one step of a fix that
    applies nothing (flags 0) from zero velocities and forces (the box must
    be at least three cut-offs, 6 A, wide: 6^3 fcc cells); FAST mode sums the
    pairs in df64 by default, or in FP64"""
    a = W.Atoms(x=at.x.copy(), v=np.zeros_like(at.v), type=at.type, mask=at.mask, boxlo=at.boxlo, boxhi=at.boxhi,
                mass=at.mass)
    fix = ephgb.FixEPH(W.fix_args(beta_file, flags=0, grid=(4, 4, 4)), a, dt=0.001, mode=mode,
                       eam=(setfl, ["Ni"]))
    fix.set_pair_arithmetic(pairs)
    fix.step(1)
    np.testing.assert_array_equal(fix.get("x"), a.x)  # v = f = 0: the step did not move them
    return fix.get("f"), fix.pair_energy()


@pytest.mark.parametrize("mode,pairs", [(ephgb.MODE_FAST, ephgb.PAIRS_DF64), (ephgb.MODE_FAST, ephgb.PAIRS_FP64),
                                        (ephgb.MODE_EXACT, ephgb.PAIRS_DF64)])
def test_matches_the_numpy_restatement(built, setfl, beta_file, mode, pairs):
    """df64 pair sums (FAST, the default) and FP64 ones (FAST with
    EPH_PAIRS_FP64, EXACT) against the numpy restatement"""
    at = W.fcc_lattice(6, jitter=0.08, seed=61)
    f, E = forces_at(setfl, beta_file, at, mode, pairs)
    En, fn = energy_forces(read_setfl(setfl), at.x, at.type, {1: 0}, at.boxhi - at.boxlo)
    assert abs(E - En) <= 1e-12 * abs(En)
    assert np.abs(f - fn).max() <= 1e-11 * np.abs(fn).max()


def test_forces_are_minus_the_energy_gradient(built, setfl, beta_file):
    at = W.fcc_lattice(6, jitter=0.08, seed=62)
    f, _ = forces_at(setfl, beta_file, at)
    h = 1e-5
    for i, k in ((3, 0), (77, 1), (250, 2), (863, 0)):
        xp = at.x.copy()
        xp[i, k] += h
        _, Ep = forces_at(setfl, beta_file, W.Atoms(x=xp, v=at.v, type=at.type, mask=at.mask, boxlo=at.boxlo,
                                                    boxhi=at.boxhi, mass=at.mass))
        xm = at.x.copy()
        xm[i, k] -= h
        _, Em = forces_at(setfl, beta_file, W.Atoms(x=xm, v=at.v, type=at.type, mask=at.mask, boxlo=at.boxlo,
                                                    boxhi=at.boxhi, mass=at.mass))
        assert abs(f[i, k] + (Ep - Em) / (2 * h)) <= 1e-6 * np.abs(f).max(), (i, k)


@pytest.mark.parametrize("pairs", [ephgb.PAIRS_DF64, ephgb.PAIRS_FP64])
def test_perfect_lattice_is_at_rest(built, setfl, beta_file, pairs):
    at = W.fcc_lattice(6, jitter=0.0, seed=63)
    f, E = forces_at(setfl, beta_file, at, pairs=pairs)
    assert np.abs(f).max() <= 1e-10
    assert -4.5 < E / at.n < -4.0  # Ni cohesion: Sutton-Chen with the 6 A cut-off, and the reference's Ni.eam


def test_nve_conserves_energy(built, setfl, beta_file):
    at = W.fcc_lattice(6, temperature=600.0, seed=64)
    fix = ephgb.FixEPH(W.fix_args(beta_file, flags=0, grid=(4, 4, 4)), at, dt=0.001, eam=(setfl, ["Ni"]))
    m = at.mass[1]
    energies = []
    for _ in range(20):
        fix.step(10)
        v = fix.get("v")
        ke = 0.5 * m * W.MVV2E * (v * v).sum()
        energies.append(ke + fix.pair_energy())
    energies = np.array(energies)
    assert np.abs(energies - energies[0]).max() / at.n <= 2e-5  # eV per atom over 200 fs


def test_with_the_fix_and_graph_replay(built, setfl, beta_file):
    """fix eph (friction + random + grid) on top of the pair force: graph
    replays equal direct launches bit for bit"""
    at = W.fcc_lattice(6, seed=65)
    W.add_pka(at, 500.0, seed=3)
    out = []
    for graph in (False, True):
        fix = ephgb.FixEPH(W.fix_args(beta_file, flags=7, grid=(6, 6, 6)), at, dt=0.0005, eam=(setfl, ["Ni"]))
        fix.set_graph(graph)
        fix.step(40)
        out.append((fix.get("x"), fix.get("v"), fix.get("T"), fix.pair_energy()))
    for a, b in zip(out[0], out[1]):
        np.testing.assert_array_equal(a, b)


def test_setup_errors(built, setfl, beta_file, tmp_path):
    words = W.fix_args(beta_file, flags=0, grid=(4, 4, 4))
    at = W.fcc_lattice(6, seed=66)
    with pytest.raises(ephgb.EphError) as e:
        ephgb.FixEPH(words, at, dt=0.001, eam=(str(tmp_path / "missing.eam"), ["Ni"]))
    assert e.value.status == 2  # EPH_ERR_FILE
    with pytest.raises(ephgb.EphError) as e:
        ephgb.FixEPH(words, at, dt=0.001, eam=(setfl, ["Cu"]))
    assert e.value.status == 1  # EPH_ERR_ARG: element not in the file
    with pytest.raises(ephgb.EphError) as e:
        ephgb.FixEPH(words, W.fcc_lattice(5, seed=66), dt=0.001, eam=(setfl, ["Ni"]))
    assert e.value.status == 1  # box narrower than three cut-offs (6 and 6.5 A)
    fix = ephgb.FixEPH(words, at, dt=0.001)
    with pytest.raises(ephgb.EphError) as e:
        fix.set_pair_eam(setfl, ["Ni"])
    assert e.value.status == 7  # EPH_ERR_STATE: after the atoms


def test_fix_density_from_the_eam_pair_list(built, setfl, beta_file):
    """With the EAM force and one lane per atom, the fix's df64 density sweep
    takes its candidates from the step's EAM pair list instead of scanning
    the EAM-sized bins: five steps of the fix (friction, random force, grid)
    on top of the pair force agree per atom, to the FAST bar, with the FP64
    path (bin search, FP64 pair terms everywhere)."""
    at = W.fcc_lattice(6, seed=91, temperature=300.0)
    out = []
    for pairs in (ephgb.PAIRS_DF64, ephgb.PAIRS_FP64):
        fix = ephgb.FixEPH(W.fix_args(beta_file, flags=7, grid=(4, 4, 4)), at, dt=0.0005, eam=(setfl, ["Ni"]))
        fix.set_threads_per_atom(1)
        fix.set_pair_arithmetic(pairs)
        fix.step(5)
        out.append({k: fix.get(k) for k in ("x", "v", "f", "rho", "w", "f_eph", "f_rng")})
    for k in out[0]:
        assert key_err(k, out[0][k], out[1][k]) <= 1e-12, (k, key_err(k, out[0][k], out[1][k]))
