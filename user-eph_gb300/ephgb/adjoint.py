"""Reverse-mode gradients through the fix-eph step (eph_adjoint_* of
include/eph_gb.h) and a small fitting harness on top of them.

`Adjoint` runs trajectories of a `FixEPH` context from a recorded start and
returns, per step, the energy the ions gave the electrons (E[t], the
reference's E_local) and the mean electronic temperature (T[t]); its backward
pass gives the gradient of a loss of those with respect to the beta file's
rho(r) and beta(rho) knot columns, C_e and kappa_e.  `Trajectory` wraps one
forward/backward pair as a torch.autograd.Function so that losses and
optimisers can be written in PyTorch; the parameters are small host tensors
and every step runs in the CUDA library.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import EphError, FixEPH, _dp, lib

GRAD_RHO_KNOTS, GRAD_BETA_KNOTS, GRAD_C_E, GRAD_KAPPA = 0, 1, 2, 3


def beta_file_of(words):
    """Path of the beta file in `fix ID group eph ...` words (fix_eph.cpp:36-58)."""
    return words[16]


def read_beta_columns(path):
    """Header and knot columns of a beta file (eph_beta.h:39-128): returns
    (header lines, elements [(name, number)], n_rho, dr, n_beta, drho, r_cutoff,
    [(rho_knots, beta_knots)] per element)."""
    with open(path) as fd:
        lines = fd.read().split("\n")
    head = lines[:3]
    el = lines[3].split()
    names = el[1:1 + int(el[0])]
    tok = " ".join(lines[4:]).split()
    n_rho, dr, n_beta, drho, rc = int(tok[0]), float(tok[1]), int(tok[2]), float(tok[3]), float(tok[4])
    pos = 5
    cols = []
    numbers = []
    for _ in names:
        numbers.append(int(tok[pos]))
        pos += 1
        r = np.array(tok[pos:pos + n_rho], dtype=np.float64)
        pos += n_rho
        b = np.array(tok[pos:pos + n_beta], dtype=np.float64)
        pos += n_beta
        cols.append((r, b))
    return head, list(zip(names, numbers)), n_rho, dr, n_beta, drho, rc, cols


def write_beta_columns(path, columns, n_rho, dr, n_beta, drho, r_cutoff, elements=(("Ni", 28),),
                       head=("# beta file", "#", "#")):
    """Write a beta file (the reference format) from knot columns
    [(rho_knots, beta_knots)] per element; values round-trip exactly."""
    with open(path, "w") as f:
        for h in head[:3]:
            f.write(h + "\n")
        f.write(f"{len(elements)} {' '.join(n for n, _ in elements)}\n")
        f.write(f"{n_rho} {float(dr)!r} {n_beta} {float(drho)!r} {float(r_cutoff)!r}\n")
        for (_, z), (r, b) in zip(elements, columns):
            f.write(f"{z}\n")
            f.write("\n".join(repr(float(v)) for v in r) + "\n")
            f.write("\n".join(repr(float(v)) for v in b) + "\n")
    return path


class Adjoint:
    """Trajectories of a context from its present state, and their gradients."""

    def __init__(self, fix: FixEPH, checkpoint_every: int = 20):
        self.fix = fix
        self.L = lib()
        h = C.c_void_p()
        rc = self.L.eph_adjoint_create(fix.h, int(checkpoint_every), C.byref(h))
        if rc:
            msg = self.L.eph_adjoint_last_error(h).decode() if h.value else self.L.eph_last_error(fix.h).decode()
            if h.value:
                self.L.eph_adjoint_destroy(h)
            raise EphError(rc, msg)
        self.h = h
        _, elems, self.n_rho, _, self.n_beta, _, _, cols = read_beta_columns(beta_file_of(fix.words))
        self.n_elements = len(elems)
        self.columns = [(r.copy(), b.copy()) for r, b in cols]
        self.C_e, self.kappa_e = float(fix.words[7]), float(fix.words[8])
        self.nsteps = 0

    def __del__(self):
        if getattr(self, "h", None):
            self.L.eph_adjoint_destroy(self.h)
            self.h = None

    def _check(self, rc):
        if rc:
            raise EphError(rc, self.L.eph_adjoint_last_error(self.h).decode())

    # ---- parameters
    def set_knots(self, elem, rho_knots=None, beta_knots=None):
        r, b = self.columns[elem]
        if rho_knots is not None:
            r = np.array(rho_knots, dtype=np.float64).reshape(self.n_rho)
        if beta_knots is not None:
            b = np.array(beta_knots, dtype=np.float64).reshape(self.n_beta)
        self.fix.set_beta_knots(elem, r, b)
        self.columns[elem] = (r.copy(), b.copy())

    def set_grid_constants(self, C_e, kappa_e):
        self.fix.set_grid_constants(C_e, kappa_e)
        self.C_e, self.kappa_e = float(C_e), float(kappa_e)

    def set_graph(self, on=True):
        self._check(self.L.eph_adjoint_set_graph(self.h, 1 if on else 0))

    # ---- passes
    def forward(self, nsteps):
        E = np.zeros(nsteps)
        T = np.zeros(nsteps)
        self._check(self.L.eph_adjoint_forward(self.h, int(nsteps), E.ctypes.data_as(_dp), T.ctypes.data_as(_dp)))
        self.nsteps = nsteps
        return E, T

    def backward(self, dL_dE=None, dL_dT=None):
        a = None if dL_dE is None else np.ascontiguousarray(dL_dE, dtype=np.float64)
        b = None if dL_dT is None else np.ascontiguousarray(dL_dT, dtype=np.float64)
        for v in (a, b):
            if v is not None and v.size != self.nsteps:
                raise ValueError("one cotangent per step of the last forward pass")
        self._check(self.L.eph_adjoint_backward(self.h, None if a is None else a.ctypes.data_as(_dp),
                                                None if b is None else b.ctypes.data_as(_dp)))

    def gradient(self, which, elem=0):
        n = {GRAD_RHO_KNOTS: self.n_rho, GRAD_BETA_KNOTS: self.n_beta}.get(which, 1)
        out = np.zeros(n)
        self._check(self.L.eph_adjoint_gradient(self.h, which, elem, out.ctypes.data_as(_dp), n))
        return out if n > 1 else float(out[0])

    def gradients(self, elem=0):
        return {"rho_knots": self.gradient(GRAD_RHO_KNOTS, elem), "beta_knots": self.gradient(GRAD_BETA_KNOTS, elem),
                "C_e": self.gradient(GRAD_C_E), "kappa_e": self.gradient(GRAD_KAPPA)}

    def timing(self):
        f, b = C.c_double(), C.c_double()
        lf, lb = C.c_long(), C.c_long()
        self._check(self.L.eph_adjoint_timing(self.h, C.byref(f), C.byref(b), C.byref(lf), C.byref(lb)))
        return {"forward_ms": f.value, "backward_ms": b.value, "forward_launches": lf.value,
                "backward_launches": lb.value}


def trajectory_function():
    """torch.autograd.Function over one element's knot columns, C_e and kappa_e:
    apply(adjoint, nsteps, beta_knots, rho_knots, C_e, kappa_e) -> (E, T_mean)."""
    import torch

    class Trajectory(torch.autograd.Function):
        @staticmethod
        def forward(ctx, adj, nsteps, beta_knots, rho_knots, C_e, kappa_e):
            adj.set_knots(0, rho_knots.detach().cpu().numpy(), beta_knots.detach().cpu().numpy())
            adj.set_grid_constants(float(C_e), float(kappa_e))
            E, T = adj.forward(int(nsteps))
            ctx.adj = adj
            return torch.from_numpy(E), torch.from_numpy(T)

        @staticmethod
        def backward(ctx, gE, gT):
            adj = ctx.adj
            adj.backward(None if gE is None else gE.detach().cpu().numpy(),
                         None if gT is None else gT.detach().cpu().numpy())
            g = adj.gradients(0)
            return (None, None, torch.from_numpy(g["beta_knots"]), torch.from_numpy(g["rho_knots"]),
                    torch.tensor(g["C_e"], dtype=torch.float64), torch.tensor(g["kappa_e"], dtype=torch.float64))

    return Trajectory


def fit_beta(adj, nsteps, target_E, beta0, iters=50, lr=0.05, rho_knots=None, C_e=None, kappa_e=None,
             target_T=None, weight_T=0.0, log=None):
    """Fit element 0's beta(rho) knots to a target energy-exchange curve (and
    optionally a mean-T_e curve) with Adam on log(beta) (keeps beta > 0).
    Returns (beta knots, loss history)."""
    import torch

    fn = trajectory_function()
    theta = torch.tensor(np.log(np.asarray(beta0, dtype=np.float64)), requires_grad=True)
    rho = torch.tensor(adj.columns[0][0] if rho_knots is None else rho_knots, dtype=torch.float64)
    ce = torch.tensor(float(C_e if C_e is not None else adj.C_e), dtype=torch.float64)
    ka = torch.tensor(float(kappa_e if kappa_e is not None else adj.kappa_e), dtype=torch.float64)
    tE = torch.as_tensor(np.asarray(target_E, dtype=np.float64))
    tT = None if target_T is None else torch.as_tensor(np.asarray(target_T, dtype=np.float64))
    opt = torch.optim.Adam([theta], lr=lr)
    hist = []
    for it in range(iters):
        opt.zero_grad()
        E, T = fn.apply(adj, nsteps, torch.exp(theta), rho, ce, ka)
        loss = ((E - tE) ** 2).sum()
        if tT is not None and weight_T:
            loss = loss + weight_T * ((T - tT) ** 2).sum()
        loss.backward()
        opt.step()
        hist.append(float(loss.detach()))
        if log:
            log(it, float(loss))
    return torch.exp(theta).detach().numpy(), hist


class AdjointBatch:
    """Several adjoints run together: every pass of every adjoint is a
    parallel branch of one CUDA graph (eph_adjoint_batch_*)."""

    def __init__(self, adjoints):
        self.adjs = list(adjoints)
        self.L = lib()
        arr = (C.c_void_p * len(self.adjs))(*[a.h.value for a in self.adjs])
        h = C.c_void_p()
        rc = self.L.eph_adjoint_batch_create(len(self.adjs), arr, C.byref(h))
        self.h = h
        if rc:
            raise EphError(rc, self.L.eph_adjoint_batch_last_error(h).decode() if h.value else "")
        self.nsteps = 0

    def __del__(self):
        if getattr(self, "h", None):
            self.L.eph_adjoint_batch_destroy(self.h)
            self.h = None

    def _check(self, rc):
        if rc:
            raise EphError(rc, self.L.eph_adjoint_batch_last_error(self.h).decode())

    def forward(self, nsteps):
        n = len(self.adjs)
        E = np.zeros((n, nsteps))
        T = np.zeros((n, nsteps))
        self._check(self.L.eph_adjoint_batch_forward(self.h, int(nsteps), E.ctypes.data_as(_dp),
                                                     T.ctypes.data_as(_dp)))
        self.nsteps = nsteps
        for a in self.adjs:
            a.nsteps = nsteps
        return E, T

    def backward(self, dL_dE=None, dL_dT=None):
        shape = (len(self.adjs), self.nsteps)
        a = None if dL_dE is None else np.ascontiguousarray(np.broadcast_to(dL_dE, shape), dtype=np.float64)
        b = None if dL_dT is None else np.ascontiguousarray(np.broadcast_to(dL_dT, shape), dtype=np.float64)
        self._check(self.L.eph_adjoint_batch_backward(self.h, None if a is None else a.ctypes.data_as(_dp),
                                                      None if b is None else b.ctypes.data_as(_dp)))

    def timing(self):
        f, b = C.c_double(), C.c_double()
        lf, lb = C.c_long(), C.c_long()
        self._check(self.L.eph_adjoint_batch_timing(self.h, C.byref(f), C.byref(b), C.byref(lf), C.byref(lb)))
        return {"forward_ms": f.value, "backward_ms": b.value, "forward_launches": lf.value,
                "backward_launches": lb.value}


def fit_beta_batch(batch, nsteps, target_T, beta0, iters=30, lr=0.05, smooth=10.0, log=None):
    """Fit the beta(rho) knots shared by every replica of `batch` to target
    mean-T_e curves (one row per replica) with Adam on log(beta).  Loss =
    sum over replicas and steps of ((T - T*) / T*_0)^2 + smooth * sum of the
    squared second differences of log(beta): the curves constrain beta only
    where the atoms' densities lie, and the penalty keeps the other knots
    from wandering.  Returns (beta knots, history of the data term)."""
    import torch

    tT = np.asarray(target_T, dtype=np.float64)
    scale = 1.0 / (tT[:, :1] ** 2)
    theta = torch.tensor(np.log(np.asarray(beta0, dtype=np.float64)), requires_grad=True)
    opt = torch.optim.Adam([theta], lr=lr)
    hist = []
    for it in range(iters):
        beta = np.exp(theta.detach().numpy())
        for a in batch.adjs:
            a.set_knots(0, None, beta)
        _, T = batch.forward(nsteps)
        d = T - tT
        hist.append(float((scale * d * d).sum()))
        batch.backward(None, 2.0 * scale * d)
        g = sum(a.gradient(GRAD_BETA_KNOTS) for a in batch.adjs)
        opt.zero_grad()
        d2 = theta[2:] - 2.0 * theta[1:-1] + theta[:-2]
        (smooth * (d2 * d2).sum()).backward()
        theta.grad += torch.from_numpy(g * beta)  # the data term, d/dlog(beta)
        opt.step()
        if log:
            log(it, hist[-1])
    return np.exp(theta.detach().numpy()), hist
