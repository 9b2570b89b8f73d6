"""Test infrastructure only: a numpy restatement of the fix-eph step and of
its reverse-mode derivative, for small systems (all pairs found by brute
force).  It checks the adjoint's mathematics on the CPU (against its own
finite differences) and the CUDA adjoint's implementation (against this) on
the same inputs.  Nothing of the product imports it.

The step follows the reference's order (fix_eph.cpp:305-348 integrator,
:431-466 density, :699-836 force_prl, :364-404 deposition, eph_fdm.h:267-400
grid solve) with the spline tables of the beta file; the deviates of each step
are given.  The reverse uses the pair structure of the forward:
W[v]_i = a_i sum_j H_ij e e.(v_i - v_j) and F[y]_i = sum_j e e.(a_i H_ij y_i -
a_j H_ji y_j) are transposes of each other.
"""
from __future__ import annotations

import numpy as np


class Tables:
    """Spline tables {a,b,c,d} per knot as the library builds them."""

    def __init__(self, rho_r_sq, inv_dr_sq, alpha, inv_drho, rho_cutoff, r_cutoff):
        self.g, self.ig = np.asarray(rho_r_sq), inv_dr_sq
        self.al, self.ia = np.asarray(alpha), inv_drho
        self.rho_cutoff, self.rc2 = rho_cutoff, r_cutoff * r_cutoff

    @staticmethod
    def eval(tab, inv, x):
        idx = np.minimum(np.floor(x * inv).astype(np.int64), len(tab) - 1)
        c = tab[idx]
        val = c[..., 0] + x * (c[..., 1] + x * (c[..., 2] + x * c[..., 3]))
        der = c[..., 1] + x * (2.0 * c[..., 2] + 3.0 * x * c[..., 3])
        return val, der, idx


class Grid:
    def __init__(self, n, lo, hi, C, rho_e, kappa, dt, nsub, inner_dt):
        self.n = tuple(int(v) for v in n)
        self.lo, self.hi = np.asarray(lo, float), np.asarray(hi, float)
        self.h = (self.hi - self.lo) / np.array(self.n)
        self.C, self.rho_e, self.kappa = C, rho_e, kappa
        self.nsub, self.inner_dt = nsub, inner_dt
        self.dV = float(np.prod(self.h))
        self.dt = dt

    def cell(self, x):
        ijk = np.floor((x - self.lo) / self.h).astype(np.int64)
        ijk %= np.array(self.n)
        return ijk[:, 0] + self.n[0] * (ijk[:, 1] + self.n[1] * ijk[:, 2])

    def lap(self, T):
        T3 = T.reshape(self.n[2], self.n[1], self.n[0])  # z, y, x
        out = np.zeros_like(T3)
        for ax, hh in zip((2, 1, 0), self.h):
            out += (np.roll(T3, 1, ax) + np.roll(T3, -1, ax) - 2.0 * T3) / (hh * hh)
        return out.ravel()

    def substep(self, T, src):
        # uniform kappa: the (kappa_q - kappa_p) term vanishes
        return T + (self.kappa * self.lap(T) + src) / (self.rho_e * self.C) * self.inner_dt


def pairs(x, box, rc2):
    """Directed in-cutoff pairs (i, j, e = x_j - x_i minimum image)."""
    n = len(x)
    d = x[None, :, :] - x[:, None, :]
    d -= box * np.round(d / box)
    r2 = (d * d).sum(-1)
    np.fill_diagonal(r2, np.inf)
    i, j = np.nonzero(r2 < rc2)
    return i, j, d[i, j], r2[i, j], n


def step(state, xi, P, tab, grid, keep=False):
    """One engine step; returns the new state, the step's energy E and mean T,
    and (keep=True) the intermediates the reverse needs."""
    x, v, f, T = state
    dtfm, dt, eta, box = P["dtfm"], P["dt"], P["eta"], P["box"]
    v1 = v + dtfm * f
    x1 = x + P.get("dtv", dt) * v1
    i, j, e, r2, n = pairs(x1, box, tab.rc2)
    g, gd, gidx = Tables.eval(tab.g, tab.ig, r2)
    rho = np.bincount(i, weights=g, minlength=n)
    live = rho > 0
    al = np.zeros(n)
    ald = np.zeros(n)
    aidx = np.zeros(n, dtype=np.int64)
    ok = live & (rho <= tab.rho_cutoff)
    al[ok], ald[ok], aidx[ok] = Tables.eval(tab.al, tab.ia, rho[ok])
    a = np.zeros(n)
    a[live] = al[live] / rho[live]
    H = g / r2
    ev = lambda y: (e * y).sum(-1)  # noqa: E731
    dv = v1[i] - v1[j]
    w = np.zeros((n, 3))
    for k in range(3):
        w[:, k] = a * np.bincount(i, weights=H * ev(dv) * e[:, k], minlength=n)
    L = live[i] & live[j]

    def F(y):
        s = (a[i] * H * ev(y[i]) - a[j] * H * ev(y[j])) * L
        return np.stack([np.bincount(i, weights=s * e[:, k], minlength=n) for k in range(3)], 1) * live[:, None]

    c = grid.cell(x1)
    Te = T[c]
    s_i = eta * np.sqrt(Te)
    fE = -F(w)
    Fx = F(xi)
    fR = s_i[:, None] * Fx
    fn = fE + fR
    v2 = v1 + dtfm * fn
    dE = -dt * ((fE * v2).sum(1) + (fR * v2).sum(1))
    E = dE.sum()
    src = np.bincount(c, weights=dE / (grid.dV * grid.dt), minlength=len(T))
    Ts = [T]
    for _ in range(grid.nsub):
        Ts.append(grid.substep(Ts[-1], src))
    new = (x1, v2, fn, Ts[-1])
    out = (new, E, Ts[-1].mean())
    if keep:
        return out + (dict(x1=x1, v1=v1, v2=v2, i=i, j=j, e=e, r2=r2, g=g, gd=gd, gidx=gidx, rho=rho, live=live,
                           al=al, ald=ald, aidx=aidx, ok=ok, a=a, H=H, w=w, xi=xi, c=c, Te=Te, s=s_i, fE=fE, fR=fR,
                           Fx=Fx, src=src, Ts=Ts, L=L, n=n),)
    return out


def trajectory(state0, xis, P, tab, grid):
    s = state0
    E, Tm = [], []
    for xi in xis:
        s, e, t = step(s, xi, P, tab, grid)
        E.append(e)
        Tm.append(t)
    return np.array(E), np.array(Tm)


def reverse(state0, xis, P, tab, grid, wE, wT):
    """Gradient of sum_t wE[t] E[t] + wT[t] Tmean[t] with respect to the
    rho(r^2)-table and alpha-table coefficients, C_e and kappa_e."""
    recs = []
    s = state0
    for xi in xis:
        s, _, _, r = step(s, xi, P, tab, grid, keep=True)
        recs.append(r)
    n = recs[0]["n"]
    xb = np.zeros((n, 3))
    vb = np.zeros((n, 3))
    fb = np.zeros((n, 3))
    Tb = np.zeros(len(state0[3]))
    g_tab = np.zeros_like(tab.g)
    a_tab = np.zeros_like(tab.al)
    gC = 0.0
    gK = 0.0
    dtfm, dt, eta = P["dtfm"], P["dt"], P["eta"]
    nc = len(Tb)
    for t in range(len(xis) - 1, -1, -1):
        R = recs[t]
        # grid solve in reverse (all cells dynamic, no clamp)
        lam = Tb + wT[t] / nc
        srcbar = np.zeros(nc)
        rc = grid.rho_e * grid.C
        for k in range(grid.nsub - 1, -1, -1):
            Tk = R["Ts"][k]
            u = lam
            wgt = u * grid.inner_dt / rc
            srcbar += wgt
            gC -= (wgt * (grid.kappa * grid.lap(Tk) + R["src"]) * grid.rho_e / rc).sum()
            gK += (wgt * grid.lap(Tk)).sum()
            lam = u + grid.kappa * grid.lap(wgt)  # the Laplacian is symmetric
        Tb = lam
        # energy and final integrate
        G = wE[t] + srcbar[R["c"]] / (grid.dV * grid.dt)
        v1b = vb - dt * G[:, None] * (R["fE"] + R["fR"])  # dL/dv' in total (v' = v + dtf/m f)
        ftot = fb + dtfm * v1b
        fbE = ftot - dt * G[:, None] * R["v2"]
        fbR = ftot - dt * G[:, None] * R["v2"]
        live = R["live"]
        cE = -fbE * live[:, None]
        cR = R["s"][:, None] * fbR * live[:, None]
        np.add.at(Tb, R["c"], (fbR * R["fR"]).sum(1) / (2.0 * R["Te"]))
        i, j, e, H, a = R["i"], R["j"], R["e"], R["H"], R["a"]
        Lp = R["L"].astype(np.float64)
        ev = lambda y: (e * y).sum(-1)  # noqa: E731
        dcE = cE[i] - cE[j]
        dcR = cR[i] - cR[j]
        U = np.stack([np.bincount(i, weights=Lp * H * ev(dcE) * e[:, k], minlength=n) for k in range(3)], 1)
        V = np.stack([np.bincount(i, weights=Lp * H * ev(dcR) * e[:, k], minlength=n) for k in range(3)], 1)
        om = a[:, None] * U
        ab = 2.0 * (R["w"] * U).sum(1) + (R["xi"] * V).sum(1)
        rb = np.zeros(n)
        ok = R["ok"]
        rho = R["rho"]
        rb[ok] = ab[ok] * (R["ald"][ok] - a[ok]) / rho[ok]
        q = np.where(ok, ab / np.where(rho > 0, rho, 1.0), 0.0)
        for p in range(4):
            np.add.at(a_tab[:, p], R["aidx"][ok], (q * rho ** p)[ok])
        # pair sweep 2
        r2, g, gd = R["r2"], R["g"], R["gd"]
        Hp = (gd - H) / r2
        Pi, Pj = a[i] * H, a[j] * H
        dv = R["v1"][i] - R["v1"][j]
        e_dv = ev(dv)
        eoi, eoj = ev(om[i]), ev(om[j])
        w, xi = R["w"], R["xi"]
        ewi, ewj, exi, exj = ev(w[i]), ev(w[j]), ev(xi[i]), ev(xi[j])
        e_dE, e_dR = ev(dcE), ev(dcR)
        Bi = Lp * (ewi * e_dE + exi * e_dR) + e_dv * eoi
        Bj = -Lp * (ewj * e_dE + exj * e_dR) - e_dv * eoj
        Od = Pi[:, None] * om[i] - Pj[:, None] * om[j]
        eOd = Pi * eoi - Pj * eoj
        gx = e_dv[:, None] * Od + dv * eOd[:, None]
        Wd = Pi[:, None] * w[i] - Pj[:, None] * w[j]
        Xd = Pi[:, None] * xi[i] - Pj[:, None] * xi[j]
        gx += Lp[:, None] * (e_dE[:, None] * Wd + dcE * ev(Wd)[:, None] + e_dR[:, None] * Xd + dcR * ev(Xd)[:, None])
        s2 = a[i] * Bi * Hp + a[j] * Bj * Hp + rb[i] * gd + rb[j] * gd
        gx += 2.0 * s2[:, None] * e
        xbar = xb - np.stack([np.bincount(i, weights=gx[:, k], minlength=n) for k in range(3)], 1)
        vbar = v1b + np.stack([np.bincount(i, weights=e[:, k] * eOd, minlength=n) for k in range(3)], 1)
        cS = a[i] * Bi / r2 + rb[i]
        for p in range(4):
            np.add.at(g_tab[:, p], R["gidx"], cS * r2 ** p)
        vbar = vbar + P.get("dtv", P["dt"]) * xbar
        xb, vb, fb = xbar, vbar, dtfm * vbar
    return {"g_rho_r_sq": g_tab, "g_alpha": a_tab, "C_e": gC, "kappa_e": gK}
