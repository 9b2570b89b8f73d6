"""The hand-written adjoint against central finite differences (h = 1e-6
relative) of the plain forward: the GPU path's own trajectories, and the
oracle's (the CPU restatement pinned to the reference) driven with the GPU's
deviates.  Loss: L = sum_t wE[t] E[t] + wT[t] T_mean[t] with seeded weights,
E[t] the step's ion-to-electron energy, T_mean[t] the mean electronic
temperature after the step."""
import numpy as np
import pytest

import ephgb
from ephgb import workloads as W
from ephgb.adjoint import Adjoint, read_beta_columns, write_beta_columns

pytestmark = pytest.mark.gpu

STEPS = 12
TOL = 1e-6  # gradient vs finite differences, norm-wise per parameter group, above the differences' own noise


def curved_beta(rho):
    """beta(rho) with curvature over the whole table: the table construction's
    slope weights are |differences of knot slopes|, ill-conditioned where the
    knots lie nearly on a line (the synthetic tanh beta over rho < 0.3), and a
    finite difference of 1e-6 relative would then measure that, not the
    gradient"""
    return 0.02 + 2.0 * rho * rho


def make(tmp_path, mode=ephgb.MODE_FAST, flags=7, K=5, grid=(4, 4, 4), T_e=2000.0, seed=31, mask_every=0):
    beta = W.write_beta_file(str(tmp_path / "adj.beta"), n_rho=16, n_beta=24, drho=0.3 / 23, beta_fn=curved_beta)
    at = W.fcc_lattice(5, seed=seed)
    if mask_every:
        at.mask = np.where(np.arange(at.n) % mask_every == 0, 2, 1).astype(np.int32)
    words = W.fix_args(beta, flags=flags, T_e=T_e, grid=grid)
    fix = ephgb.FixEPH(words, atoms=at, dt=0.001, mode=mode)
    return fix, Adjoint(fix, checkpoint_every=K), at, words


def weights(E, T, seed=3):
    rng = np.random.default_rng(seed)
    sE = np.abs(E).max() or 1.0
    sT = np.abs(T).max() or 1.0
    return rng.standard_normal(len(E)) / sE, rng.standard_normal(len(T)) / sT


def adjoint_grads(adj, wE, wT):
    adj.backward(wE, wT)
    return adj.gradients(0)


def fd_grads(loss, cols, C_e, kappa_e, h=1e-6, scale=None):
    """Central differences of loss(rho_knots, beta_knots, C_e, kappa_e), and
    (scale given: sum of |terms| of the loss) each difference's rounding
    noise, 2 eps scale / (2 step): the knots near the cutoff are ~1e-5, so a
    1e-6 relative step is ~1e-11 and the loss's own rounding shows there."""
    r0, b0 = cols
    out = {"rho_knots": np.zeros(len(r0)), "beta_knots": np.zeros(len(b0))}
    noise = {"rho_knots": np.zeros(len(r0)), "beta_knots": np.zeros(len(b0))}
    eps = 2.0 ** -52 * (scale or 0.0)
    floor = np.abs(r0[r0 != 0]).min()  # a zero knot moves by 1e-6 of the smallest non-zero one
    for k in range(len(r0)):
        d = h * max(abs(r0[k]), floor)
        p, m = r0.copy(), r0.copy()
        p[k] += d
        m[k] -= d
        out["rho_knots"][k] = (loss(p, b0, C_e, kappa_e) - loss(m, b0, C_e, kappa_e)) / (2 * d)
        noise["rho_knots"][k] = eps / d
    for k in range(len(b0)):
        d = h * abs(b0[k])
        p, m = b0.copy(), b0.copy()
        p[k] += d
        m[k] -= d
        out["beta_knots"][k] = (loss(r0, p, C_e, kappa_e) - loss(r0, m, C_e, kappa_e)) / (2 * d)
        noise["beta_knots"][k] = eps / d
    d = h * C_e
    out["C_e"] = (loss(r0, b0, C_e + d, kappa_e) - loss(r0, b0, C_e - d, kappa_e)) / (2 * d)
    noise["C_e"] = eps / d
    d = h * kappa_e
    out["kappa_e"] = (loss(r0, b0, C_e, kappa_e + d) - loss(r0, b0, C_e, kappa_e - d)) / (2 * d)
    noise["kappa_e"] = eps / d
    return (out, noise) if scale is not None else out


def gpu_loss_fn(adj, wE, wT):
    def loss(r, b, C_e, kappa_e):
        adj.set_knots(0, r, b)
        adj.set_grid_constants(C_e, kappa_e)
        E, T = adj.forward(STEPS)
        return float(wE @ E + wT @ T)
    return loss


def compare(g, fd, noise=None):
    """norm-wise relative error per group; with the differences' noise, the
    part of each error above 10x that noise"""
    errs = {}
    for k in g:
        d = np.abs(np.asarray(g[k]) - fd[k])
        if noise is not None:
            d = np.maximum(d - 10.0 * np.asarray(noise[k]), 0.0)
        errs[k] = float(np.max(d) / np.abs(fd[k]).max())
    return errs


def loss_scale(E, T, wE, wT):
    return float(np.abs(wE * E).sum() + np.abs(wT * T).sum())


@pytest.mark.parametrize("mode", [ephgb.MODE_FAST, ephgb.MODE_EXACT])
def test_gradient_matches_finite_differences(built, tmp_path, mode):
    fix, adj, at, words = make(tmp_path, mode=mode)
    E, T = adj.forward(STEPS)
    wE, wT = weights(E, T)
    g = adjoint_grads(adj, wE, wT)
    cols = tuple(c.copy() for c in adj.columns[0])
    fd, noise = fd_grads(gpu_loss_fn(adj, wE, wT), cols, adj.C_e, adj.kappa_e, scale=loss_scale(E, T, wE, wT))
    errs = compare(g, fd, noise)
    assert max(errs.values()) <= TOL, errs


@pytest.mark.parametrize("flags,mask_every", [(1, 0), (6, 0), (7 | 0x10, 0), (7, 3)])
def test_gradient_flag_matrix(built, tmp_path, flags, mask_every):
    """friction only, random + grid only, friction computed but not applied,
    and a fix group that leaves every third atom out"""
    fix, adj, at, words = make(tmp_path, flags=flags, mask_every=mask_every)
    E, T = adj.forward(STEPS)
    wE, wT = weights(E, T)
    g = adjoint_grads(adj, wE, wT)
    cols = tuple(c.copy() for c in adj.columns[0])
    fd, noise = fd_grads(gpu_loss_fn(adj, wE, wT), cols, adj.C_e, adj.kappa_e, scale=loss_scale(E, T, wE, wT))
    if not flags & 4:  # no grid solve: C_e and kappa_e do not enter
        assert g["C_e"] == 0.0 and g["kappa_e"] == 0.0 and fd["C_e"] == 0.0 and fd["kappa_e"] == 0.0
        g = {k: g[k] for k in ("rho_knots", "beta_knots")}
    errs = compare(g, fd, noise)
    assert max(errs.values()) <= TOL, errs


def test_checkpoint_interval_does_not_change_the_gradient(built, tmp_path):
    grads = []
    for K in (1, 5, STEPS):
        fix, adj, at, words = make(tmp_path, K=K)
        E, T = adj.forward(STEPS)
        wE, wT = weights(E, T)
        grads.append(adjoint_grads(adj, wE, wT))
    # every sum of the backward pass has a fixed order: bit for bit
    for g in grads[1:]:
        for k in g:
            np.testing.assert_array_equal(np.asarray(g[k]), np.asarray(grads[0][k]), err_msg=k)


def test_forward_is_the_plain_trajectory(built, tmp_path):
    fix, adj, at, words = make(tmp_path)
    E, T = adj.forward(STEPS)
    plain = ephgb.FixEPH(words, atoms=at, dt=0.001)
    Ee_prev = plain.compute_vector(0)
    for t in range(STEPS):
        plain.step(1)
        Ee = plain.compute_vector(0)
        assert abs((Ee - Ee_prev) - E[t]) <= 1e-12 * abs(Ee) + 1e-300, t
        assert abs(plain.compute_vector(1) - T[t]) <= 1e-12 * T[t], t
        Ee_prev = Ee
    np.testing.assert_array_equal(plain.get("x"), fix.get("x"))
    np.testing.assert_array_equal(plain.get("v"), fix.get("v"))


def test_reference_gradient_from_the_oracle(built, tmp_path):
    """Finite differences of the oracle (pinned bit for bit to the reference
    fix) driven with the GPU generator's deviates, against the adjoint of the
    EXACT-mode GPU path."""
    from oracle.bindings import OracleFix

    fix, adj, at, words = make(tmp_path, mode=ephgb.MODE_EXACT)
    E, T = adj.forward(STEPS)
    wE, wT = weights(E, T)
    g = adjoint_grads(adj, wE, wT)
    # the deviates of each step, from a plain run of the same context
    plain = ephgb.FixEPH(words, atoms=at, dt=0.001, mode=ephgb.MODE_EXACT)
    xis = []
    for t in range(STEPS):
        plain.step(1)
        xis.append(plain.get("xi").ravel().copy())
    _, elems, n_rho, dr, n_beta, drho, rc, cols = read_beta_columns(words[16])
    counter = [0]

    def loss(r, b, C_e, kappa_e):
        counter[0] += 1
        path = write_beta_columns(str(tmp_path / f"fd{counter[0] % 2}.beta"), [(r, b)], n_rho, dr, n_beta, drho, rc,
                                  elements=elems)
        w = list(words)
        w[7], w[8], w[16] = repr(float(C_e)), repr(float(kappa_e)), path
        ref = OracleFix(w, at, 0.001)
        L, Ee_prev = 0.0, 0.0
        for t in range(STEPS):
            ref.step(xis[t])
            vec = ref.get("vector")
            L += wE[t] * (vec[0] - Ee_prev) + wT[t] * vec[1]
            Ee_prev = vec[0]
        return L

    # the oracle's loss is the GPU path's
    assert abs(loss(*cols[0], adj.C_e, adj.kappa_e) - float(wE @ E + wT @ T)) <= 1e-10 * np.abs(wT @ T)
    fd, noise = fd_grads(loss, cols[0], adj.C_e, adj.kappa_e, scale=loss_scale(E, T, wE, wT))
    errs = compare(g, fd, noise)
    assert max(errs.values()) <= TOL, errs


def test_matches_the_numpy_restatement(built, tmp_path):
    """The CUDA adjoint against oracle/adjoint_ref.py on the same start, the
    same deviates (the device generator's, read back from a plain run) and the
    same loss: trajectory and knot gradients."""
    from ephgb import BetaFile
    from oracle.adjoint_ref import Grid as NGrid
    from oracle.adjoint_ref import Tables, reverse, trajectory

    steps = 6
    fix, adj, at, words = make(tmp_path)
    plain = ephgb.FixEPH(words, atoms=at, dt=0.001)
    xis = []
    for _ in range(steps):
        plain.step(1)
        xis.append(plain.get("xi").copy())
    E, T = adj.forward(steps)
    wE, wT = weights(E, T)
    g = adjoint_grads(adj, wE, wT)
    B = BetaFile(words[16])
    _, _, n_rho, dr, n_beta, drho, rc, _ = read_beta_columns(words[16])
    tab = Tables(B.table("rho_r_sq", 0), (n_rho - 1) / (rc * rc), B.table("alpha", 0), 1.0 / drho,
                 drho * (n_beta - 1), rc)
    dt = 0.001
    nsub, idt = ephgb.Grid(n=(4, 4, 4), lo=at.boxlo, hi=at.boxhi, T_e=2000.0, C_e=3.5e-6, rho_e=1.0,
                           kappa_e=0.1).substeps(dt)
    grid = NGrid((4, 4, 4), at.boxlo, at.boxhi, 3.5e-6, 1.0, 0.1, dt, nsub, idt)
    P = dict(dtfm=0.5 * dt * W.FTM2V / W.NI_MASS, dt=dt, eta=np.sqrt(2 * W.BOLTZ / dt), box=at.boxhi - at.boxlo)
    s0 = (at.x.copy(), at.v.copy(), np.zeros((at.n, 3)), np.full(64, 2000.0))
    En, Tn = trajectory(s0, xis, P, tab, grid)
    assert np.abs(E - En).max() <= 1e-10 * np.abs(En).max()
    assert np.abs(T - Tn).max() <= 1e-12 * np.abs(Tn).max()
    R = reverse(s0, xis, P, tab, grid, wE, wT)
    gr, gb = B.knot_gradient(0, R["g_rho_r_sq"], R["g_alpha"])
    assert np.abs(g["rho_knots"] - gr).max() <= 1e-9 * np.abs(gr).max()
    assert np.abs(g["beta_knots"] - gb).max() <= 1e-9 * np.abs(gb).max()
    assert abs(g["C_e"] - R["C_e"]) <= 1e-9 * abs(R["C_e"])
    assert abs(g["kappa_e"] - R["kappa_e"]) <= 1e-9 * abs(R["kappa_e"])


def test_graph_replay_matches_direct_launches(built, tmp_path):
    fix, adj, at, words = make(tmp_path)
    out = []
    for graph in (False, True, True):  # direct, capture + replay, replay
        adj.set_graph(graph)
        E, T = adj.forward(STEPS)
        wE, wT = weights(E, T, seed=9)
        out.append((E, T, adjoint_grads(adj, wE, wT)))
    for E, T, g in out[1:]:
        np.testing.assert_array_equal(E, out[0][0])
        np.testing.assert_array_equal(T, out[0][1])
        for k in g:
            np.testing.assert_array_equal(np.asarray(g[k]), np.asarray(out[0][2][k]), err_msg=k)


def test_autograd_function_and_fitting_harness(built, tmp_path):
    """Trajectory (torch.autograd.Function) gives the adjoint's gradients, and
    Adam on log(beta) lowers an energy-exchange loss against a curve made with
    a hidden beta(rho)."""
    import torch

    from ephgb.adjoint import fit_beta, trajectory_function

    fix, adj, at, words = make(tmp_path)
    r0, b0 = (c.copy() for c in adj.columns[0])
    hidden = b0 * (1.0 + 0.4 * np.sin(np.arange(b0.size) / 3.0))
    adj.set_knots(0, r0, hidden)
    target, _ = adj.forward(STEPS)
    adj.set_knots(0, r0, b0)
    fn = trajectory_function()
    beta = torch.tensor(b0, requires_grad=True)
    rho = torch.tensor(r0, requires_grad=True)
    ce = torch.tensor(adj.C_e, dtype=torch.float64, requires_grad=True)
    ka = torch.tensor(adj.kappa_e, dtype=torch.float64, requires_grad=True)
    E, T = fn.apply(adj, STEPS, beta, rho, ce, ka)
    loss = ((E - torch.from_numpy(target)) ** 2).sum()
    loss.backward()
    adj.backward(2.0 * (E.detach().numpy() - target), None)
    g = adj.gradients(0)
    np.testing.assert_allclose(beta.grad.numpy(), g["beta_knots"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(rho.grad.numpy(), g["rho_knots"], rtol=1e-12, atol=0)
    assert float(ce.grad) == pytest.approx(g["C_e"], rel=1e-12)
    _, hist = fit_beta(adj, STEPS, target, b0, iters=15, lr=0.05)
    assert hist[-1] < 0.5 * hist[0]


def test_batch_equals_the_adjoints_run_alone(built, tmp_path):
    """Three replicas of different sizes and electron temperatures: the
    batched passes (one graph each) give every replica's trajectory and
    gradient bit for bit as its adjoint run alone."""
    from ephgb.adjoint import AdjointBatch

    beta = W.write_beta_file(str(tmp_path / "b.beta"), n_rho=16, n_beta=24, drho=0.3 / 23, beta_fn=curved_beta)
    reps = []
    for k, (cells, T_e) in enumerate(((4, 1500.0), (5, 2500.0), (6, 3500.0))):
        at = W.fcc_lattice(cells, seed=40 + k)
        words = W.fix_args(beta, seed=100 + k, flags=7, T_e=T_e, grid=(4, 4, 4))
        fix = ephgb.FixEPH(words, atoms=at, dt=0.001)
        reps.append((fix, Adjoint(fix, checkpoint_every=4)))
    alone = []
    for fix, adj in reps:
        E, T = adj.forward(STEPS)
        wE, wT = weights(E, T, seed=len(alone))
        alone.append((E, T, wE, wT, adjoint_grads(adj, wE, wT)))
    batch = AdjointBatch([adj for _, adj in reps])
    for _ in range(2):  # capture, then replay
        E, T = batch.forward(STEPS)
        batch.backward(np.stack([a[2] for a in alone]), np.stack([a[3] for a in alone]))
        for r, (fix, adj) in enumerate(reps):
            np.testing.assert_array_equal(E[r], alone[r][0])
            np.testing.assert_array_equal(T[r], alone[r][1])
            g = adj.gradients(0)
            for k in g:
                np.testing.assert_array_equal(np.asarray(g[k]), np.asarray(alone[r][4][k]), err_msg=k)


def test_two_element_gradient(built, tmp_path):
    """A Ni/Fe beta file (the tables of both elements in the pair terms):
    the knot gradients of each element against central differences."""
    beta = W.write_beta_file(str(tmp_path / "NiFe.beta"), elements=("Ni", "Fe"), numbers=(28, 26), n_rho=16,
                             n_beta=24, drho=0.3 / 23, beta_fn=curved_beta)
    at = W.fcc_lattice(5, seed=71)
    at.type = np.where(np.arange(at.n) % 4 == 1, 2, 1).astype(np.int32)
    at.mass = np.array([0.0, W.NI_MASS, 55.845])
    words = W.fix_args(beta, flags=7, T_e=2000.0, grid=(4, 4, 4), elements=("Ni", "Fe"))
    fix = ephgb.FixEPH(words, atoms=at, dt=0.001)
    adj = Adjoint(fix, checkpoint_every=5)
    E, T = adj.forward(STEPS)
    wE, wT = weights(E, T)
    adj.backward(wE, wT)
    scale = loss_scale(E, T, wE, wT)
    eps = 2.0 ** -52 * scale
    grads = [adj.gradients(elem) for elem in (0, 1)]  # before the forward passes of the differences
    for elem in (0, 1):
        g = grads[elem]
        r0, b0 = (c.copy() for c in adj.columns[elem])

        def loss(r, b):
            adj.set_knots(elem, r, b)
            E2, T2 = adj.forward(STEPS)
            return float(wE @ E2 + wT @ T2)

        fd_b, noise_b = np.zeros(b0.size), np.zeros(b0.size)
        for k in range(b0.size):
            d = 1e-6 * b0[k]
            p, m = b0.copy(), b0.copy()
            p[k] += d
            m[k] -= d
            fd_b[k] = (loss(r0, p) - loss(r0, m)) / (2 * d)
            noise_b[k] = eps / d
        floor = np.abs(r0[r0 != 0]).min()
        fd_r, noise_r = np.zeros(r0.size), np.zeros(r0.size)
        for k in range(r0.size):
            d = 1e-6 * max(abs(r0[k]), floor)
            p, m = r0.copy(), r0.copy()
            p[k] += d
            m[k] -= d
            fd_r[k] = (loss(p, b0) - loss(m, b0)) / (2 * d)
            noise_r[k] = eps / d
        adj.set_knots(elem, r0, b0)
        errs = compare({"beta_knots": g["beta_knots"], "rho_knots": g["rho_knots"]},
                       {"beta_knots": fd_b, "rho_knots": fd_r}, {"beta_knots": noise_b, "rho_knots": noise_r})
        assert max(errs.values()) <= TOL, (elem, errs)


@pytest.mark.parametrize("case", ["model1", "coloured", "eam"])
def test_unsupported_contexts_are_refused(built, tmp_path, case):
    beta = W.write_beta_file(str(tmp_path / "b.beta"), n_rho=16, n_beta=24, drho=0.3 / 23)
    at = W.fcc_lattice(6, seed=81)
    words = W.fix_args(beta, flags=7, grid=(4, 4, 4), model=1 if case == "model1" else 4)
    eam = None
    if case == "coloured":
        words[2], words[5] = "eph/coloured/exp", "0.005"
    if case == "eam":
        eam = (W.write_eam_sutton_chen(str(tmp_path / "sc.eam")), ["Ni"])
    fix = ephgb.FixEPH(words, atoms=at, dt=0.001, eam=eam)
    with pytest.raises(ephgb.EphError) as e:
        Adjoint(fix)
    assert e.value.status == 3  # EPH_ERR_UNSUPPORTED_MODEL


def test_specified_step_on_the_adjoint_workload(built, tmp_path):
    """The adjoint workload at its stated size (fcc Ni 20^3 cells = 32,000
    atoms, ions 300 K, T_e 2,000 K on a 16^3 grid, 200 steps of 1 fs, flags
    7, 64 beta knots, loss sum_t (E[t] - E*[t])^2 against a hidden beta's
    curve) with central differences at exactly the stated step, h = 1e-6
    relative, for the beta knots and C_e: within 1e-6 (norm-wise per group).
    The loss is only piecewise smooth (an atom crossing into another grid
    cell sees another T_e), so a knot whose difference at h disagrees with
    the one at h/2 by more than 1e-6 of the largest has a jump inside its
    stencil and is left out; at most 4 of the 64 may be (this trajectory has
    one: knot 5, 1 % off at h, where the two stencils differ by as much).  The
    rho(r) knots and kappa_e are left to the bench's balanced-step check:
    their gradients are small against the loss, and at h = 1e-6 the loss's
    rounding dominates their differences (~1e-6 and ~1e-4)."""
    bf = W.write_beta_file(str(tmp_path / "adj.beta"), n_rho=16, n_beta=64, drho=0.02,
                           beta_fn=lambda r: 0.02 + 2.0 * r * r)
    at = W.fcc_lattice(20, seed=4249)
    words = W.fix_args(bf, seed=4242, flags=7, T_e=2000.0, grid=(16, 16, 16))
    fix = ephgb.FixEPH(words, at, dt=0.001, mode=ephgb.MODE_FAST)
    adj = Adjoint(fix, checkpoint_every=20)
    r0, b0 = (c.copy() for c in adj.columns[0])
    adj.set_knots(0, r0, b0 * (1.0 + 0.3 * np.sin(np.arange(b0.size) / 6.0)))
    target, _ = adj.forward(200)
    adj.set_knots(0, r0, b0)
    C_e0 = adj.C_e

    def loss(b, C_e):
        adj.set_knots(0, r0, b)
        adj.set_grid_constants(C_e, adj.kappa_e)
        E, _ = adj.forward(200)
        return float(((E - target) ** 2).sum())

    E, _ = adj.forward(200)
    adj.backward(2.0 * (E - target), None)
    g = adj.gradients(0)

    def fd_beta(h):
        out = np.zeros(b0.size)
        for k in range(b0.size):
            d = h * abs(b0[k])
            p, m = b0.copy(), b0.copy()
            p[k] += d
            m[k] -= d
            out[k] = (loss(p, C_e0) - loss(m, C_e0)) / (2 * d)
        return out

    fd_b, fd_b2 = fd_beta(1e-6), fd_beta(5e-7)
    scale = np.abs(fd_b).max()
    smooth = np.abs(fd_b - fd_b2) <= 1e-6 * scale
    assert smooth.sum() >= b0.size - 4, np.flatnonzero(~smooth)
    err_b = np.abs(g["beta_knots"] - fd_b)[smooth].max() / scale
    d = 1e-6 * C_e0
    fd_c = (loss(b0, C_e0 + d) - loss(b0, C_e0 - d)) / (2 * d)
    err_c = abs(g["C_e"] - fd_c) / abs(fd_c)
    assert err_b <= 1e-6 and err_c <= 1e-6, (err_b, err_c)


@pytest.mark.parametrize("mode", [ephgb.MODE_FAST, ephgb.MODE_EXACT])
def test_df64_reverse_sweeps_match_fp64(built, tmp_path, mode):
    """The reverse pair sweeps in df64 (the default, with the df64 forward)
    against the FP64 sweeps (eph_set_pair_arithmetic(EPH_PAIRS_FP64), FP64
    forward and reverse): the same gradients within 1e-9 per group (the two
    forwards differ in their last bits; the rest is the df64 arithmetic)."""
    out = []
    for arith in (ephgb.PAIRS_DF64, ephgb.PAIRS_FP64):
        fix, _, at, words = make(tmp_path, mode=mode)
        fix.set_pair_arithmetic(arith)
        adj = Adjoint(fix, checkpoint_every=5)
        E, T = adj.forward(STEPS)
        wE, wT = weights(E, T)
        out.append(adjoint_grads(adj, wE, wT))
    for k in out[0]:
        a, b = np.asarray(out[0][k], dtype=float), np.asarray(out[1][k], dtype=float)
        assert np.abs(a - b).max() <= 1e-9 * max(np.abs(b).max(), 1e-300), (k, np.abs(a - b).max())
