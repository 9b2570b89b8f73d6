"""CUDA path (libephgb.so through the C ABI) against the CPU oracle on the
same seeded inputs and the same injected deviates.

EXACT mode keeps the reference's expression order without FMA: on the first
step every per-atom array is bit-identical to the oracle; the grid sums its
deposits exactly (fixed point) instead of in atom order, so T_e (and from the
second step on everything that depends on T_e) agrees to rounding.  FAST mode
factors alpha/rho and rho(r^2)/r^2 and uses FMA.  Tolerance for both: the
parity bar, 1e-12 relative per atom (helpers.atom_err: max over atoms of
|a_i - b_i| / (|b_i| + s), s the larger of the median |b_j| and
1e-3 max_j |b_j|, so that no atom's error hides behind another atom's larger
value), per grid cell for T_e."""
import numpy as np
import pytest

import ephgb
from ephgb import workloads as W
from helpers import SCENARIOS, atom_err, key_err, n_in_group, scenario, xi_rows
from oracle.bindings import OracleFix

pytestmark = pytest.mark.gpu
TOL = 1e-12
ATOM_KEYS = ("rho", "w", "f_eph", "f_rng", "f", "x", "v", "array")


def run_pair(words, at, dt, mode, steps, check, seed=5, tpa=0):
    gpu = ephgb.FixEPH(words, at, dt=dt, mode=mode)
    if tpa:
        gpu.set_threads_per_atom(tpa)
    ref = OracleFix(words, at, dt)
    ng = n_in_group(at)
    rnd = int(words[4], 0) & 2
    for s in range(steps):
        stream = W.gaussian_stream(ng, seed, s) if rnd else None
        if rnd:
            gpu.step(1, xi=xi_rows(at, stream))
        else:
            gpu.step(1)
        ref.step(stream)
        check(s, gpu, ref)
    gpu.synchronize()
    return gpu, ref


@pytest.mark.parametrize("name", SCENARIOS)
def test_exact_mode_bitwise_first_step(built, beta_file, beta_file_2el, name):
    words, at, dt = scenario(name, beta_file, beta_file_2el)

    def check(s, gpu, ref):
        for k in ATOM_KEYS:
            a, b = gpu.get(k), ref.get(k)
            if s == 0:
                assert np.array_equal(a, b), (k, key_err(k, a, b))
            else:
                assert key_err(k, a, b) <= TOL, (s, k, key_err(k, a, b))
        assert atom_err(gpu.get("T"), ref.get("T")) <= TOL
        Ee_g, Ee_r = gpu.compute_vector(0), ref.get("vector")[0]
        scale = max(abs(Ee_r), np.abs(ref.get("f_eph")).max() * 1e-3 + 1e-300)
        assert abs(Ee_g - Ee_r) <= TOL * scale * at.n
        assert abs(gpu.compute_vector(1) - ref.get("vector")[1]) <= TOL * abs(ref.get("vector")[1])

    run_pair(words, at, dt, ephgb.MODE_EXACT, 6 if name != "pka" else 30, check)


@pytest.mark.parametrize("tpa", [0, 1])
@pytest.mark.parametrize("name", SCENARIOS)
def test_fast_mode_within_tolerance(built, beta_file, beta_file_2el, name, tpa):
    """tpa 0: lanes per atom from the atom count (4 for these small systems);
    tpa 1: one lane per atom, stage 1 folded into the density sweep (as at the
    bench size)"""
    words, at, dt = scenario(name, beta_file, beta_file_2el)

    def check(s, gpu, ref):
        for k in ATOM_KEYS:
            assert key_err(k, gpu.get(k), ref.get(k)) <= TOL, (s, k, key_err(k, gpu.get(k), ref.get(k)))
        assert atom_err(gpu.get("T"), ref.get("T")) <= TOL

    run_pair(words, at, dt, ephgb.MODE_FAST, 6 if name != "pka" else 30, check, tpa=tpa)


def test_c1_config_fast_and_exact(built, beta_file):
    """The 4,000-atom CPU-runnable case (10^3 grid) for 20 steps."""
    words, at, dt = scenario("c1", beta_file)
    for mode in (ephgb.MODE_EXACT, ephgb.MODE_FAST):
        def check(s, gpu, ref):
            if s in (0, 9, 19):
                for k in ATOM_KEYS:
                    assert key_err(k, gpu.get(k), ref.get(k)) <= TOL, (mode, s, k)
                assert atom_err(gpu.get("T"), ref.get("T")) <= TOL

        run_pair(words, at, dt, mode, 20, check)


def test_hook_sequence_matches_step(built, beta_file):
    """Driving the four hooks one by one equals eph_step (no wrap needed at
    300 K over a few steps)."""
    words, at, dt = scenario("c1_small", beta_file)
    a = ephgb.FixEPH(words, at, dt=dt, mode=ephgb.MODE_EXACT)
    b = ephgb.FixEPH(words, at, dt=dt, mode=ephgb.MODE_EXACT)
    for s in range(3):
        xi = xi_rows(at, W.gaussian_stream(at.n, 9, s))
        a.step(1, xi=xi)
        b.set_timestep(s + 1)
        b.initial_integrate()
        b.put("f", np.zeros((at.n, 3)))
        b.post_force(xi=xi)
        b.final_integrate()
        b.end_of_step()
        for k in ATOM_KEYS:
            assert np.array_equal(a.get(k), b.get(k)), (s, k)
        assert np.array_equal(a.get("T"), b.get("T"))


@pytest.mark.parametrize("mode", [ephgb.MODE_EXACT, ephgb.MODE_FAST])
def test_tdyn_grid(built, beta_file, tmp_path, mode):
    """A grid file with temperature-dependent cells (C_e(T), kappa_e(T),
    E_e(T) inverse update): the device grid solve against the oracle."""
    pf = W.write_grid_parameters(str(tmp_path / "params.data"))
    gf = W.write_grid_file(str(tmp_path / "Tdyn.in"), parameter_file=pf, tdyn=True, T=2000.0)
    at = W.fcc_lattice(5, seed=61)
    words = W.fix_args(beta_file, T_infile=gf, grid=(1, 1, 1))

    def check(s, gpu, ref):
        for k in ATOM_KEYS:
            if mode == ephgb.MODE_EXACT and s == 0:
                assert np.array_equal(gpu.get(k), ref.get(k)), k
            else:
                assert key_err(k, gpu.get(k), ref.get(k)) <= TOL, (s, k)
        assert atom_err(gpu.get("T"), ref.get("T")) <= TOL, s

    run_pair(words, at, 0.001, mode, 10, check)
    gpu = ephgb.FixEPH(words, at, dt=0.001, mode=mode)
    gpu.step(3)
    gpu.save_state(str(tmp_path / "after.restart"))  # C_e, kappa_e follow T in the written state
    text = open(tmp_path / "after.restart").read().splitlines()
    assert text[7].endswith("params.data") and len(text) == 8 + 8 * 6 * 5


def test_threads_per_atom_variants(built, beta_file):
    """FAST-mode sweeps with 1, 2, 4 and 8 lanes per atom give the same
    forces within rounding (the order of the sums differs), and the autotuner
    picks one of them and restores the forces it touched."""
    words, at, dt = scenario("c1_small", beta_file)
    ng = n_in_group(at)
    out = {}
    for tpa in (1, 2, 4, 8):
        gpu = ephgb.FixEPH(words, at, dt=dt, mode=ephgb.MODE_FAST)
        gpu.set_threads_per_atom(tpa)
        assert gpu.threads_per_atom() == tpa
        for s in range(4):
            gpu.step(1, xi=xi_rows(at, W.gaussian_stream(ng, 5, s)))
        out[tpa] = {k: gpu.get(k) for k in ("w", "f_eph", "f_rng", "x", "v")}
        out[tpa]["T"] = gpu.get("T")
    for tpa in (2, 4, 8):
        for k, a in out[tpa].items():
            assert key_err(k, a, out[1][k]) <= 1e-13, (tpa, k, key_err(k, a, out[1][k]))
    gpu = ephgb.FixEPH(words, at, dt=dt, mode=ephgb.MODE_FAST)
    gpu.step(1)
    f_before = gpu.get("f")
    assert gpu.autotune() in (1, 2, 4, 8)
    np.testing.assert_array_equal(gpu.get("f"), f_before)


@pytest.mark.parametrize("tpa", [2, 4, 8])
def test_folded_sweeps_with_lanes(built, beta_file, tpa):
    """From 16,384 atoms on, FAST mode folds stage 1 and M_i into the density
    sweep at any number of lanes per atom (k_forces_m with TPA lanes): 16^3
    fcc cells against the oracle for 3 steps."""
    at = W.fcc_lattice(16, seed=21)
    assert at.n == 16384
    words = W.fix_args(beta_file, grid=(8, 8, 8))

    def check(s, gpu, ref):
        for k in ATOM_KEYS:
            assert key_err(k, gpu.get(k), ref.get(k)) <= TOL, (s, k, key_err(k, gpu.get(k), ref.get(k)))
        assert atom_err(gpu.get("T"), ref.get("T")) <= TOL

    gpu, _ = run_pair(words, at, 0.001, ephgb.MODE_FAST, 3, check, tpa=tpa)
    assert gpu.threads_per_atom() == tpa


def test_async_host_copies(built, beta_file):
    """Hooks driven with queued host copies (EPH_HOST_ASYNC, one
    synchronisation per step) give what the synchronous copies give."""
    import torch

    words, at, dt = scenario("c1_small", beta_file)
    n = at.n
    out = []
    for asynchronous in (False, True):
        fix = ephgb.FixEPH(words, at, dt=dt)
        x = torch.from_numpy(at.x.copy()).pin_memory().numpy()
        v = torch.from_numpy(at.v.copy()).pin_memory().numpy()
        f = torch.zeros((n, 3), dtype=torch.float64).pin_memory().numpy()
        for _ in range(4):
            fix.put("x", x, asynchronous)
            fix.put("v", v, asynchronous)
            fix.put("f", f, asynchronous)
            fix.initial_integrate()
            fix.post_force()
            fix.final_integrate()
            fix.end_of_step()
            if asynchronous:
                fix.get_async("x", x)
                fix.get_async("v", v)
                fix.get_async("f", f)
                fix.synchronize()
            else:
                fix.get("x", out=x)
                fix.get("v", out=v)
                fix.get("f", out=f)
        out.append((x.copy(), v.copy(), f.copy(), fix.get("T")))
    for a, b in zip(out[0], out[1]):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("cells,pinned", [(5, False), (16, True), (40, True)])
def test_host_array_hooks(built, beta_file, cells, pinned):
    """eph_initial_integrate_host / eph_post_force_host / eph_final_integrate_host
    (chunked copies overlapped on two copy streams, fused kernels, the per-atom
    array sent out on a third stream) equal the put / hook / get sequence bit
    for bit over several steps: 500 and 16,384 atoms (one chunk), 256,000
    atoms (3 chunks), pageable and pinned host arrays, with and without the
    positions uploaded in post_force and the per-atom array."""
    import torch

    at = W.fcc_lattice(cells, seed=81, temperature=300.0)
    W.add_pka(at, 500.0, seed=82)
    words = W.fix_args(beta_file, grid=(6, 6, 6))
    n = at.n

    def rows(a, k=3):
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(n, k)
        return torch.from_numpy(a.copy()).pin_memory().numpy() if pinned else a.copy()

    ref = ephgb.FixEPH(words, at, dt=0.0005)
    fix = ephgb.FixEPH(words, at, dt=0.0005)
    xr, vr, fr = rows(at.x), rows(at.v), rows(np.zeros((n, 3)))
    x, v, f, arr = rows(at.x), rows(at.v), rows(np.zeros((n, 3))), rows(np.zeros((n, 8)), 8)
    for s in range(6):
        fpair = np.full((n, 3), 1e-3 * (s + 1))  # an engine force
        # the reference sequence
        ref.set_timestep(s + 1)
        ref.put("x", xr)
        ref.put("v", vr)
        ref.initial_integrate()
        ref.get("x", out=xr)
        ref.get("v", out=vr)
        if s % 2 == 0:
            ref.put("x", xr)
        fr[:] = fpair
        ref.put("f", fr)
        ref.post_force()
        ref.get("f", out=fr)
        ref.put("f", fr)
        ref.final_integrate()
        ref.get("v", out=vr)
        ref.end_of_step()
        arr_ref = ref.get("array")
        # the host-array hooks
        fix.set_timestep(s + 1)
        fix.initial_integrate_host(x, v)
        f[:] = fpair
        fix.post_force_host(x if s % 2 == 0 else None, f, arr if s % 3 != 1 else None)
        fix.final_integrate_host(f, v)
        fix.end_of_step()
        for a, b, k in ((x, xr, "x"), (v, vr, "v"), (f, fr, "f")):
            assert np.array_equal(a, b), (s, k)
        if s % 3 != 1:
            assert np.array_equal(arr, arr_ref), s
        assert np.array_equal(fix.get("T"), ref.get("T")), s
        assert fix.compute_vector(0) == ref.compute_vector(0)


@pytest.mark.parametrize("two_el", [False, True])
def test_df64_pair_sums_against_oracle_and_fp64(built, beta_file, beta_file_2el, two_el):
    """The FAST one-lane sweeps with df64 pair arithmetic (the default from
    16,384 atoms on) against the oracle, and against the same sweeps in FP64
    (eph_set_pair_arithmetic): 16^3 fcc cells with a 3 keV knock-on atom, one
    and two elements (the second: H_ij != H_ji, two rho(r^2) tables), 4 steps,
    1e-12 per atom."""
    at = W.fcc_lattice(16, seed=31)
    W.add_pka(at, 3000.0, seed=32)
    if two_el:
        at.type = np.where(np.arange(at.n) % 3 == 1, 2, 1).astype(np.int32)
        at.mass = np.array([0.0, W.NI_MASS, 55.845])
        words = W.fix_args(beta_file_2el, grid=(8, 8, 8), elements=("Ni", "Fe"))
    else:
        words = W.fix_args(beta_file, grid=(8, 8, 8))
    dt = 0.0005
    fixes = {}
    for arith in (ephgb.PAIRS_DF64, ephgb.PAIRS_FP64):
        fx = ephgb.FixEPH(words, at, dt=dt, mode=ephgb.MODE_FAST)
        fx.set_list_skin(0.0)  # the bin search every step (the df64 sweeps' path)
        fx.set_pair_arithmetic(arith)
        fixes[arith] = fx
    ref = OracleFix(words, at, dt)
    ng = n_in_group(at)
    for s in range(4):
        stream = W.gaussian_stream(ng, 5, s)
        for fx in fixes.values():
            fx.step(1, xi=xi_rows(at, stream))
        ref.step(stream)
        for k in ATOM_KEYS:
            a, b, o = fixes[ephgb.PAIRS_DF64].get(k), fixes[ephgb.PAIRS_FP64].get(k), ref.get(k)
            assert key_err(k, a, o) <= TOL, (s, k, key_err(k, a, o))
            assert key_err(k, a, b) <= TOL, (s, k, key_err(k, a, b))
        assert atom_err(fixes[ephgb.PAIRS_DF64].get("T"), ref.get("T")) <= TOL
    # the two arithmetics really ran different kernels: their last bits differ
    assert not np.array_equal(fixes[ephgb.PAIRS_DF64].get("f_eph"), fixes[ephgb.PAIRS_FP64].get("f_eph"))
