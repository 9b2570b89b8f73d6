"""Kept candidate lists (FAST mode, model 4, the one-lane density sweep): the
candidates within r_cutoff + s are searched on build steps only; atoms that
moved more than s/2 since the build, and the atoms near them, search afresh
every step, and more than 32 moved atoms make a build step.  The pairs, and
so the results, must be those of a search every step (up to the order of
the sums): checked against the oracle and against the same context with
reuse switched off, with a fast primary knock-on atom (moved atoms, wraps
across the box faces) and with hot atoms (builds forced by many moved
atoms); runs and graph replays stay bit-identical."""
import numpy as np
import pytest

import ephgb
from ephgb import workloads as W
from helpers import atom_err, key_err, n_in_group, scenario, xi_rows
from oracle.bindings import OracleFix

pytestmark = pytest.mark.gpu
TOL = 1e-12
ATOM_KEYS = ("rho", "w", "f_eph", "f_rng", "f", "x", "v", "array")


def _fix(words, at, dt, skin=0.3, tpa=1):
    """A FAST context with the list skin set (so it applies at any size)"""
    fix = ephgb.FixEPH(words, at, dt=dt, mode=ephgb.MODE_FAST)
    fix.set_threads_per_atom(tpa)
    fix.set_list_skin(skin)
    return fix


def _against_oracle(words, at, dt, steps, seed=5):
    gpu = _fix(words, at, dt)
    assert gpu.list_skin() == (0.3, True)
    ref = OracleFix(words, at, dt)
    ng = n_in_group(at)
    for s in range(steps):
        stream = W.gaussian_stream(ng, seed, s)
        gpu.step(1, xi=xi_rows(at, stream))
        ref.step(stream)
        for k in ATOM_KEYS:
            assert key_err(k, gpu.get(k), ref.get(k)) <= TOL, (s, k, key_err(k, gpu.get(k), ref.get(k)))
        assert atom_err(gpu.get("T"), ref.get("T")) <= TOL, s
    return gpu


def test_pka_against_oracle(built, beta_file):
    """A 2 keV knock-on atom (0.2 A per step) in 6^3 cells for 40 steps: it
    is a moved atom from the second step on and crosses box faces."""
    words, at, dt = scenario("pka", beta_file)
    gpu = _against_oracle(words, at, dt, 40)
    builds = gpu.counter("build")
    assert 1 <= builds < 40, builds


def test_hot_atoms_force_builds(built, beta_file):
    """Velocities of a few thousand kelvin: more than 32 atoms pass s/2
    within a few steps, so builds recur."""
    at = W.fcc_lattice(5, seed=31)
    at.v *= 4.0
    words = W.fix_args(beta_file, grid=(5, 5, 5))
    gpu = _against_oracle(words, at, 0.001, 30)
    builds = gpu.counter("build")
    assert 3 <= builds < 30, builds


def test_group_and_two_elements(built, beta_file, beta_file_2el):
    for name in ("group", "two_elements"):
        words, at, dt = scenario(name, beta_file, beta_file_2el)
        at.v *= 2.0
        _against_oracle(words, at, dt, 20)


@pytest.fixture(scope="module")
def cascade(tmp_path_factory):
    import os

    wd = str(tmp_path_factory.mktemp("list"))
    bf = W.write_beta_file(os.path.join(wd, "synth.beta"))
    at = W.fcc_lattice(16, seed=41)
    W.add_pka(at, 10000.0, seed=42)
    words = W.fix_args(bf, seed=43, grid=(8, 8, 8))
    return words, at


def test_same_as_search_every_step(built, cascade):
    """16,384 atoms, a 10 keV knock-on atom, 60 steps with the device RNG:
    kept lists against a bin search every step."""
    words, at = cascade
    a = _fix(words, at, 0.0005)
    b = _fix(words, at, 0.0005, skin=0.0)
    assert a.list_skin()[1] and not b.list_skin()[1]
    for _ in range(6):
        a.step(10)
        b.step(10)
        for k in ("rho", "w", "f_eph", "f_rng", "x", "v", "T"):
            assert key_err(k, a.get(k), b.get(k)) <= TOL, (k, key_err(k, a.get(k), b.get(k)))
    assert a.pair_count() == b.pair_count()
    assert 1 <= a.counter("build") < 60
    assert a.counter("wrap") == b.counter("wrap")


def test_with_lanes_in_the_force_sweep(built, cascade):
    """From 16,384 atoms on the one-lane density sweep feeds force sweeps
    with several lanes per atom: lists with 4 lanes against the bin search."""
    words, at = cascade
    a = _fix(words, at, 0.0005, tpa=4)
    b = _fix(words, at, 0.0005, skin=0.0, tpa=4)
    assert a.list_skin()[1] and a.threads_per_atom() == 4
    a.step(30)
    b.step(30)
    for k in ("rho", "w", "f_eph", "f_rng", "x", "v", "T"):
        assert key_err(k, a.get(k), b.get(k)) <= TOL, (k, key_err(k, a.get(k), b.get(k)))


def test_run_to_run_and_graph(built, cascade):
    """Direct steps and graph replays give the same bits (the build decisions
    live on the device)."""
    import torch

    words, at = cascade
    a = _fix(words, at, 0.0005)
    g = _fix(words, at, 0.0005)
    stream = torch.cuda.Stream()
    g.set_stream(stream.cuda_stream)
    g.set_graph(True)
    a.step(25)
    g.step(25)
    g.synchronize()
    for k in ("x", "v", "f", "f_eph", "f_rng", "rho", "T"):
        assert np.array_equal(a.get(k), g.get(k)), k
    assert a.counter("build") == g.counter("build") < 25


def test_hooks_with_host_positions(built, cascade):
    """The hooks driven as an engine does, positions, velocities and forces
    copied in and out every step (no wraps: the engine does those): kept
    lists against a bin search every step."""
    words, at = cascade
    out = []
    for skin in (0.3, 0.0):
        h = _fix(words, at, 0.0005, skin=skin)
        x, v = at.x.copy(), at.v.copy()
        f = np.zeros_like(x)
        for s in range(25):
            h.put("x", x)
            h.put("v", v)
            h.put("f", f)
            h.set_timestep(s + 1)
            h.initial_integrate()
            h.put("f", np.zeros_like(x))
            h.post_force()
            h.final_integrate()
            h.end_of_step()
            x, v, f = h.get("x"), h.get("v"), h.get("f")
        out.append(({k: h.get(k) for k in ("x", "v", "f", "f_eph", "f_rng", "rho", "T")}, h.counter("build")))
    (a, builds), (b, _) = out
    for k in a:
        assert key_err(k, a[k], b[k]) <= TOL, (k, key_err(k, a[k], b[k]))
    assert 1 <= builds < 25


def test_when_reuse_is_off(built, beta_file):
    words, at, dt = scenario("c1_small", beta_file)
    assert not ephgb.FixEPH(words, at, dt=dt, mode=ephgb.MODE_EXACT).list_skin()[1]
    fix = ephgb.FixEPH(words, at, dt=dt, mode=ephgb.MODE_FAST)
    fix.set_threads_per_atom(1)
    assert fix.list_skin() == (0.3, False)  # 500 atoms: below the default size range
    fix.set_list_skin(0.3)
    assert fix.list_skin() == (0.3, True)
    fix.set_threads_per_atom(4)  # below 16,384 atoms the density sweep has the lanes
    assert not fix.list_skin()[1]
    fix.set_threads_per_atom(1)
    assert fix.list_skin()[1]
    fix.set_list_skin(3.0)  # 17.6 A box: fewer than three bins of r_cutoff + 3 A
    assert fix.list_skin() == (3.0, False)
    fix.step(2)
    fix.set_list_skin(0.4)
    assert fix.list_skin() == (0.4, True)
    fix.step(2)
    with pytest.raises(ephgb.EphError):
        fix.set_list_skin(-1.0)


def test_autotune_list_skin_restores_the_state(built, beta_file, tmp_path):
    """eph_autotune_list_skin times windows of steps with each candidate skin
    from the current state and restores it: afterwards the context holds the
    state it had (x, v, f, T_e, the vector, the per-atom records), writes no
    temperature file of its trial steps, and steps on bit for bit as a twin
    context given eph_set_list_skin(chosen) at the same point."""
    at = W.fcc_lattice(16, seed=71)  # 16,384 atoms: one lane per atom
    W.add_pka(at, 2000.0, seed=72)
    tout = str(tmp_path / "Te_out")
    words = W.fix_args(beta_file, grid=(8, 8, 8), T_freq=5, T_out=tout)
    fixes = [ephgb.FixEPH(words, at, dt=0.0005, mode=ephgb.MODE_FAST) for _ in range(2)]
    for f in fixes:
        f.step(6)
    before = {k: fixes[0].get(k) for k in ("x", "v", "f", "T", "rho", "w", "f_eph", "f_rng")}
    E0 = fixes[0].compute_vector(0)
    written = sorted(p.name for p in tmp_path.iterdir())
    chosen = fixes[0].autotune_list_skin((0.0, 0.15, 0.3, 0.6), steps=8)
    assert chosen in (0.0, 0.15, 0.3, 0.6)
    assert fixes[0].list_skin()[0] == chosen
    for k, a in before.items():
        assert np.array_equal(fixes[0].get(k), a), k
    assert fixes[0].compute_vector(0) == E0
    assert sorted(p.name for p in tmp_path.iterdir()) == written  # no T_out of the trial steps
    fixes[1].set_list_skin(chosen)
    for f in fixes:
        f.step(12)
    for k in ("x", "v", "f", "T", "f_eph"):
        assert np.array_equal(fixes[0].get(k), fixes[1].get(k)), k
    assert fixes[0].compute_vector(0) == fixes[1].compute_vector(0)
    assert sorted(p.name for p in tmp_path.iterdir()) != written  # the real steps write theirs


def test_autotune_list_skin_where_lists_do_not_apply(built, beta_file):
    """EXACT mode keeps the bin search: nothing runs, the skin stays"""
    at = W.fcc_lattice(16, seed=73)
    fix = ephgb.FixEPH(W.fix_args(beta_file, grid=(8, 8, 8)), at, dt=0.0005, mode=ephgb.MODE_EXACT)
    fix.step(2)
    x = fix.get("x")
    assert fix.autotune_list_skin((0.2, 0.5), steps=4) == fix.list_skin()[0]
    assert np.array_equal(fix.get("x"), x)
    with pytest.raises(ephgb.EphError):
        fix.autotune_list_skin((-1.0,), steps=4)
