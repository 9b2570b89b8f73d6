"""Shared test scenarios: seeded synthetic systems and the deviates the fix
draws, in both layouts (the reference's draw order and per-atom rows)."""
from __future__ import annotations

import numpy as np

from ephgb import workloads as W


def xi_rows(atoms, stream, groupbit=1):
    """Per-atom rows (n x 3) of a draw-order stream (3 per in-group atom)."""
    rows = np.zeros((atoms.n, 3))
    sel = (atoms.mask & groupbit) != 0
    rows[sel] = np.asarray(stream).reshape(-1, 3)
    return rows


def n_in_group(atoms, groupbit=1):
    return int(((atoms.mask & groupbit) != 0).sum())


def rel_err(a, b):
    """max |a - b| over max |b| (norm-wise relative error of an array)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.abs(b).max()
    if scale == 0:
        return float(np.abs(a - b).max())
    return float(np.abs(a - b).max() / scale)


def atom_err(a, b, floor=None):
    """Per-atom relative error: max over atoms i of |a_i - b_i| / (|b_i| + s),
    with |.| the largest component of atom i's row (a 3-vector, or a scalar
    for 1-D arrays).  Every atom is measured against its own magnitude —
    unlike a norm-wise error, which a single fast atom's large value
    dominates — plus a floor s for values that nearly vanish by cancellation
    (their own digits are rounding noise in any arithmetic, the reference's
    included).  s defaults to the larger of the median of |b_i| (a typical
    atom) and 1e-3 max_i |b_i|; the second only matters where most atoms
    carry nothing, as in a lattice at rest hit by one knock-on atom, whose
    other nonzero values are sums cancelling by the lattice's symmetry.
    Rows equal in both count as 0 (also where b_i = 0)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.ndim == 1:
        a, b = a[:, None], b[:, None]
    d = np.abs(a - b).max(axis=1)
    m = np.abs(b).max(axis=1)
    s = max(float(np.median(m)), 1e-3 * float(m.max(initial=0.0))) if floor is None else float(floor)
    den = m + s
    e = np.zeros_like(d)
    nz = d != 0
    e[nz] = d[nz] / np.where(den[nz] > 0, den[nz], np.inf)
    e[nz & (den == 0)] = np.inf
    return float(e.max()) if e.size else 0.0


# column groups of the fix's per-atom array (fix_eph.cpp:406-415): rho_i,
# beta(rho_i), f_EPH, f_RNG
ARRAY_GROUPS = ((0, 1), (1, 2), (2, 5), (5, 8))


def key_err(key, a, b):
    """The per-atom error of a named per-atom output (atom_err per row; the
    per-atom array per column group); the grid T per cell."""
    if key == "array":
        return max(atom_err(np.asarray(a)[:, lo:hi], np.asarray(b)[:, lo:hi]) for lo, hi in ARRAY_GROUPS)
    return atom_err(a, b)


def scenario(name, beta_file, beta_file_2el=None):
    """(words, atoms, dt, flags) of a named test scenario."""
    if name == "c1_small":  # the C1 setting on 5^3 cells
        at = W.fcc_lattice(5, seed=11)
        return W.fix_args(beta_file, grid=(5, 5, 5)), at, 0.001
    if name == "c1":  # the CPU-runnable case: 10^3 cells, 4000 atoms, 10^3 grid
        at = W.fcc_lattice(10, seed=12)
        return W.fix_args(beta_file, grid=(10, 10, 10)), at, 0.001
    if name == "friction_only":
        at = W.fcc_lattice(5, seed=13)
        return W.fix_args(beta_file, flags=1, grid=(4, 4, 4)), at, 0.001
    if name == "fric_rand_nofdm":
        at = W.fcc_lattice(5, seed=14)
        return W.fix_args(beta_file, flags=3, grid=(1, 1, 1)), at, 0.001
    if name == "random_only_fdm":
        at = W.fcc_lattice(5, seed=15)
        return W.fix_args(beta_file, flags=6, grid=(3, 5, 7)), at, 0.001
    if name == "noapply":  # friction+random+fdm computed but not applied (NOFRICTION|NORANDOM)
        at = W.fcc_lattice(5, seed=16)
        return W.fix_args(beta_file, flags=7 | 0x10 | 0x20, grid=(5, 5, 5)), at, 0.001
    if name == "noint":
        at = W.fcc_lattice(5, seed=17)
        return W.fix_args(beta_file, flags=7 | 0x08, grid=(5, 5, 5)), at, 0.001
    if name == "group":  # every third atom outside the fix group
        at = W.fcc_lattice(5, seed=18)
        at.mask = np.where(np.arange(at.n) % 3 == 0, 2, 1).astype(np.int32)
        return W.fix_args(beta_file, grid=(5, 5, 5)), at, 0.001
    if name == "pka":  # fast atom: rebuilds and position wraps
        at = W.fcc_lattice(6, seed=19)
        W.add_pka(at, 2000.0, seed=3)
        return W.fix_args(beta_file, grid=(6, 6, 6)), at, 0.0005
    if name == "hot_electrons":
        at = W.fcc_lattice(5, seed=20)
        return W.fix_args(beta_file, T_e=2000.0, grid=(5, 5, 5)), at, 0.001
    if name == "two_elements":
        at = W.fcc_lattice(5, seed=21)
        at.type = np.where(np.arange(at.n) % 4 == 1, 2, 1).astype(np.int32)
        at.mass = np.array([0.0, W.NI_MASS, 55.845])
        return W.fix_args(beta_file_2el, grid=(5, 5, 5), elements=("Ni", "Fe")), at, 0.001
    if name == "ttm":  # model 1: local Langevin with beta(rho_i)
        at = W.fcc_lattice(5, seed=23)
        at.mask = np.where(np.arange(at.n) % 5 == 0, 2, 1).astype(np.int32)
        return W.fix_args(beta_file, model=1, grid=(5, 5, 5)), at, 0.001
    if name == "coloured":  # fix eph/coloured/exp, tau0 = 5 fs
        at = W.fcc_lattice(5, seed=24)
        words = W.fix_args(beta_file, grid=(5, 5, 5))
        words[2], words[5] = "eph/coloured/exp", "0.005"
        return words, at, 0.001
    if name == "uneven_box":
        at = W.fcc_lattice((5, 4, 6), seed=22)
        return W.fix_args(beta_file, grid=(7, 3, 4)), at, 0.001
    raise KeyError(name)


SCENARIOS = ["c1_small", "friction_only", "fric_rand_nofdm", "random_only_fdm", "noapply", "noint", "group", "pka",
             "hot_electrons", "two_elements", "uneven_box", "ttm", "coloured"]
