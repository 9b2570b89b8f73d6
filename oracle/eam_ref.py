"""Test infrastructure only: a numpy restatement of the eam/alloy pair force
for small systems (all pairs by brute force), reading the setfl file and
building its cubic Hermite tables independently of the library.  Not part of
the product."""
from __future__ import annotations

import numpy as np


def read_setfl(path):
    with open(path) as fd:
        lines = fd.read().split("\n")
    el = lines[3].split()
    nel = int(el[0])
    tok = " ".join(lines[4:]).split()
    nrho, drho, nr, dr, rc = int(tok[0]), float(tok[1]), int(tok[2]), float(tok[3]), float(tok[4])
    pos = 5
    F, f = [], []
    for _ in range(nel):
        pos += 4
        F.append(np.array(tok[pos:pos + nrho], dtype=float))
        pos += nrho
        f.append(np.array(tok[pos:pos + nr], dtype=float))
        pos += nr
    z2r = {}
    for a in range(nel):
        for b in range(a + 1):
            z2r[(a, b)] = np.array(tok[pos:pos + nr], dtype=float)
            pos += nr
    return dict(nrho=nrho, drho=drho, nr=nr, dr=dr, rc=rc, F=F, f=f, z2r=z2r, names=el[1:1 + nel])


def hermite(y):
    """slopes (per knot spacing) and the cubic per interval in p in [0, 1]"""
    n = len(y)
    s = np.zeros(n)
    s[0] = y[1] - y[0]
    s[-1] = y[-1] - y[-2]
    s[1] = 0.5 * (y[2] - y[0])
    s[-2] = 0.5 * (y[-1] - y[-3])
    s[2:-2] = ((y[:-4] - y[4:]) + 8.0 * (y[3:-1] - y[1:-3])) / 12.0
    d = np.diff(y)
    c = np.zeros((n, 4))
    c[:-1, 0] = y[:-1]
    c[:-1, 1] = s[:-1]
    c[:-1, 2] = 3.0 * d - 2.0 * s[:-1] - s[1:]
    c[:-1, 3] = s[:-1] + s[1:] - 2.0 * d
    c[-1, 0] = y[-1]
    c[-1, 1] = s[-1]
    return c


def evaluate(c, x):
    n = len(c)
    m = np.minimum(np.floor(x).astype(int), n - 2)
    p = np.minimum(x - m, 1.0)
    k = c[m]
    v = k[..., 0] + p * (k[..., 1] + p * (k[..., 2] + p * k[..., 3]))
    dv = k[..., 1] + p * (2.0 * k[..., 2] + 3.0 * p * k[..., 3])
    return v, dv


def energy_forces(setfl, x, types, type_map, box):
    """Total energy and forces (n x 3) of positions x in a periodic box."""
    t = setfl
    cF = [hermite(F) for F in t["F"]]
    cf = [hermite(f) for f in t["f"]]
    cz = {k: hermite(v) for k, v in t["z2r"].items()}
    el = np.array([type_map[tt] for tt in types])
    n = len(x)
    d = x[None, :, :] - x[:, None, :]
    d -= box * np.round(d / box)
    r2 = (d * d).sum(-1)
    np.fill_diagonal(r2, np.inf)
    i, j = np.nonzero(r2 < t["rc"] ** 2)
    e = d[i, j]
    r = np.sqrt(r2[i, j])
    q = r / t["dr"]
    fj = np.zeros(len(i))
    dfj = np.zeros(len(i))
    dfi = np.zeros(len(i))
    phi = np.zeros(len(i))
    dphi = np.zeros(len(i))
    for a in range(len(cf)):
        sel = el[j] == a
        fj[sel], dfj[sel] = evaluate(cf[a], q[sel])
        sel = el[i] == a
        _, dfi[sel] = evaluate(cf[a], q[sel])
    for (a, b), c in cz.items():
        sel = ((el[i] == a) & (el[j] == b)) | ((el[i] == b) & (el[j] == a))
        z, dz = evaluate(c, q[sel])
        phi[sel] = z / r[sel]
        dphi[sel] = (dz / t["dr"] - phi[sel]) / r[sel]
    rho = np.bincount(i, weights=fj, minlength=n)
    rho_max = t["drho"] * (t["nrho"] - 1)
    Fv = np.zeros(n)
    dF = np.zeros(n)
    for a in range(len(cF)):
        sel = el == a
        v, dv = evaluate(cF[a], rho[sel] / t["drho"])
        dv = dv / t["drho"]
        Fv[sel] = v + np.where(rho[sel] > rho_max, dv * (rho[sel] - rho_max), 0.0)
        dF[sel] = dv
    E = Fv.sum() + 0.5 * phi.sum()
    dEdr = dF[i] * dfj / t["dr"] + dF[j] * dfi / t["dr"] + dphi
    s = dEdr / r
    f = np.stack([np.bincount(i, weights=s * e[:, k], minlength=n) for k in range(3)], 1)
    return E, f
