"""Host side of the adjoint (no GPU): the chain rule from table-coefficient
gradients to the beta file's knot columns (eph_beta_knot_gradient) against
central finite differences through the table construction itself."""
import numpy as np
import pytest

from ephgb import BetaFile
from ephgb import workloads as W
from ephgb.adjoint import read_beta_columns


@pytest.mark.parametrize("n_rho,n_beta", [(16, 24), (40, 64)])
def test_knot_gradient_matches_finite_differences(tmp_path, n_rho, n_beta):
    # a beta(rho) with curvature over the table (the slope weights of the
    # table construction are ill-conditioned where the knots lie on a line)
    path = W.write_beta_file(str(tmp_path / "s.beta"), n_rho=n_rho, n_beta=n_beta, drho=0.3 / (n_beta - 1),
                             beta_fn=lambda r: 0.05 + 0.02 * np.tanh(8.0 * (r - 0.15)) + 0.01 * r * r)
    b = BetaFile(path)
    rng = np.random.default_rng(5)
    g_rs = rng.standard_normal((n_rho, 4))
    g_a = rng.standard_normal((n_beta, 4))
    gr, gb = b.knot_gradient(0, g_rs, g_a)
    r0, b0 = read_beta_columns(path)[7][0]

    def S(r, bb):
        b.set_knots(0, r, bb)
        return float((b.table("rho_r_sq", 0) * g_rs).sum() + (b.table("alpha", 0) * g_a).sum())

    # small absolute steps: the knots near the cutoff are ~1e-5 and the table
    # construction's slope weights vary on that scale
    fd_r = np.zeros(n_rho)
    hr = 1e-8
    for k in range(n_rho):
        p, m = r0.copy(), r0.copy()
        p[k] += hr
        m[k] -= hr
        fd_r[k] = (S(p, b0) - S(m, b0)) / (2 * hr)
    fd_b = np.zeros(n_beta)
    for k in range(n_beta):
        h = 1e-8
        p, m = b0.copy(), b0.copy()
        p[k] += h
        m[k] -= h
        fd_b[k] = (S(r0, p) - S(r0, m)) / (2 * h)
    # the slope weights are |differences of slopes|: where the second
    # difference of the knots changes sign the construction has a kink, and a
    # central difference straddling it is off by O(h); 1e-5 covers that at h = 1e-8
    assert np.abs(gr - fd_r).max() <= 1e-5 * np.abs(fd_r).max()
    assert np.abs(gb - fd_b).max() <= 1e-5 * np.abs(fd_b).max()


def test_set_knots_reproduces_the_file(tmp_path):
    path = W.write_beta_file(str(tmp_path / "s.beta"), n_rho=30, n_beta=50)
    b = BetaFile(path)
    before = {w: b.table(w, 0).copy() for w in ("rho_r", "rho_r_sq", "beta", "alpha")}
    r0, b0 = read_beta_columns(path)[7][0]
    b.set_knots(0, r0 * 1.5, b0)
    assert not np.array_equal(b.table("rho_r", 0), before["rho_r"])
    b.set_knots(0, r0, b0)
    for w, t in before.items():
        assert np.array_equal(b.table(w, 0), t), w


def _small_case(steps, seed=1):
    from ephgb import Grid
    from oracle.adjoint_ref import Grid as NGrid
    from oracle.adjoint_ref import Tables

    import tempfile, os
    d = tempfile.mkdtemp()
    path = W.write_beta_file(os.path.join(d, "a.beta"), n_rho=16, n_beta=24, drho=0.3 / 23)
    B = BetaFile(path)
    at = W.fcc_lattice(4, seed=31)
    dt = 0.001
    hg = Grid(n=(4, 4, 4), lo=at.boxlo, hi=at.boxhi, T_e=2000.0, C_e=3.5e-6, rho_e=1.0, kappa_e=0.1)
    nsub, idt = hg.substeps(dt)
    P = dict(dtfm=0.5 * dt * W.FTM2V / W.NI_MASS, dt=dt, eta=np.sqrt(2 * W.BOLTZ / dt), box=at.boxhi - at.boxlo)
    rng = np.random.default_rng(seed)
    xis = [rng.standard_normal((at.n, 3)) for _ in range(steps)]
    T0 = 2000.0 + 50.0 * np.random.default_rng(5).standard_normal(64)

    def build(rs, al, C, K):
        tab = Tables(rs, 15 / B.r_cutoff ** 2, al, 23 / 0.3, 0.3, B.r_cutoff)
        g = NGrid((4, 4, 4), at.boxlo, at.boxhi, C, 1.0, K, dt, nsub, idt)
        return tab, g, (at.x.copy(), at.v.copy(), np.zeros((at.n, 3)), T0.copy())

    return B, P, xis, build


def test_numpy_adjoint_matches_its_finite_differences():
    """The adjoint's mathematics (oracle/adjoint_ref.py, the same formulas as
    the CUDA kernels) against central differences of the numpy forward: table
    coefficients, C_e and kappa_e, integrator on, three steps."""
    from oracle.adjoint_ref import reverse, trajectory

    B, P, xis, build = _small_case(3)
    rs, al = B.table("rho_r_sq", 0), B.table("alpha", 0)
    tab, g, s0 = build(rs, al, 3.5e-6, 0.1)
    E, T = trajectory(s0, xis, P, tab, g)
    rng = np.random.default_rng(2)
    wE, wT = rng.standard_normal(3) / np.abs(E).max(), rng.standard_normal(3) / np.abs(T).max()
    R = reverse(s0, xis, P, tab, g, wE, wT)

    def L(rs_, al_, C, K):
        tab, g, s0 = build(rs_, al_, C, K)
        E, T = trajectory(s0, xis, P, tab, g)
        return wE @ E + wT @ T

    h = 1e-6
    for name, base, gr in (("rho_r_sq", rs, R["g_rho_r_sq"]), ("alpha", al, R["g_alpha"])):
        fd = np.zeros_like(base)
        for idx in zip(*np.nonzero(gr)):
            d = h * abs(base[idx])
            p, m = base.copy(), base.copy()
            p[idx] += d
            m[idx] -= d
            args_p = (p, al) if name == "rho_r_sq" else (rs, p)
            args_m = (m, al) if name == "rho_r_sq" else (rs, m)
            fd[idx] = (L(*args_p, 3.5e-6, 0.1) - L(*args_m, 3.5e-6, 0.1)) / (2 * d)
        assert np.abs(fd - gr).max() <= 1e-6 * np.abs(fd).max(), name
    fdC = (L(rs, al, 3.5e-6 * (1 + h), 0.1) - L(rs, al, 3.5e-6 * (1 - h), 0.1)) / (2 * h * 3.5e-6)
    assert abs(R["C_e"] - fdC) <= 1e-6 * abs(fdC)
