"""Synthetic inputs for the fix-eph hot path: fcc lattices, Maxwell-Boltzmann
velocities, the synthetic beta(rho) file and the `fix eph` argument vector.

The reference ships no dataset for this path; its benchmarks are LAMMPS decks
on fcc Ni (TB_Bench/01_Profile/*/run.lmp).  These generators produce seeded
inputs with the shapes and value distributions of those decks: fcc Ni with
a = 3.52 A, Gaussian position jitter, velocities at a set temperature, and a
beta file in the reference format (Doc/Beta/input.beta, read by
eph_beta.h:39-128).  Units are LAMMPS metal units throughout.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

# LAMMPS metal units: Boltzmann constant in eV/K, and the conversion of
# eV/A/amu into A/ps^2 (ftm2v) whose inverse converts amu*A^2/ps^2 into eV.
BOLTZ = 8.617343e-5
MVV2E = 1.0364269e-4
FTM2V = 1.0 / MVV2E

NI_MASS = 58.69
NI_LATTICE = 3.52


@dataclass
class Atoms:
    """Atoms of one periodic orthogonal box, arrays in LAMMPS layout."""

    x: np.ndarray  # (n, 3) float64
    v: np.ndarray  # (n, 3) float64
    type: np.ndarray  # (n,) int32, LAMMPS types 1..ntypes
    mask: np.ndarray  # (n,) int32, group bits
    boxlo: np.ndarray  # (3,)
    boxhi: np.ndarray  # (3,)
    mass: np.ndarray = field(default_factory=lambda: np.array([0.0, NI_MASS]))  # index 1..ntypes

    @property
    def n(self) -> int:
        return int(self.x.shape[0])


def fcc_lattice(cells: int | tuple, a: float = NI_LATTICE, jitter: float = 0.05, temperature: float = 300.0,
                mass: float = NI_MASS, seed: int = 12345) -> Atoms:
    """fcc crystal of cells^3 unit cells (4 atoms each), positions jittered by
    a Gaussian of standard deviation `jitter` (A), velocities drawn from the
    Maxwell-Boltzmann distribution at `temperature` with the centre-of-mass
    velocity removed."""
    if isinstance(cells, int):
        cells = (cells, cells, cells)
    nx, ny, nz = cells
    rng = np.random.default_rng(seed)
    basis = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.0], [0.5, 0.0, 0.5], [0.0, 0.5, 0.5]])
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    # atom order: x fastest over unit cells, like a LAMMPS create_atoms box
    origins = np.stack([ix.ravel(order="F"), iy.ravel(order="F"), iz.ravel(order="F")], axis=1).astype(np.float64)
    x = ((origins[:, None, :] + basis[None, :, :]) * a).reshape(-1, 3)
    x = x + rng.normal(0.0, jitter, size=x.shape)
    boxlo = np.zeros(3)
    boxhi = np.array([nx * a, ny * a, nz * a], dtype=np.float64)
    x = boxlo + np.mod(x - boxlo, boxhi - boxlo)
    sigma = math.sqrt(BOLTZ * temperature / (mass * MVV2E)) if temperature > 0 else 0.0
    v = rng.normal(0.0, sigma, size=x.shape)
    v -= v.mean(axis=0)
    n = x.shape[0]
    return Atoms(x=np.ascontiguousarray(x), v=np.ascontiguousarray(v), type=np.ones(n, dtype=np.int32),
                 mask=np.ones(n, dtype=np.int32), boxlo=boxlo, boxhi=boxhi, mass=np.array([0.0, mass]))


def add_pka(atoms: Atoms, energy_ev: float, seed: int = 7) -> int:
    """Give the atom nearest the box centre `energy_ev` of kinetic energy in a
    seeded random direction; returns its index."""
    rng = np.random.default_rng(seed)
    centre = 0.5 * (atoms.boxlo + atoms.boxhi)
    i = int(np.argmin(((atoms.x - centre) ** 2).sum(axis=1)))
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    m = atoms.mass[atoms.type[i]]
    speed = math.sqrt(2.0 * energy_ev / (m * MVV2E))
    atoms.v[i] = speed * d
    return i


def kinetic_temperature(atoms: Atoms) -> float:
    m = atoms.mass[atoms.type][:, None]
    ke = 0.5 * MVV2E * float((m * atoms.v ** 2).sum())
    dof = 3 * atoms.n - 3
    return 2.0 * ke / (dof * BOLTZ)


def synthetic_rho(r: np.ndarray, rc: float = 4.6, length: float = 0.6) -> np.ndarray:
    """rho(r) = exp(-r/length) * (1 - (r/rc)^2)^2 for r < rc, 0 beyond: smooth
    (C1) at the cutoff."""
    r = np.asarray(r, dtype=np.float64)
    s = np.clip(1.0 - (r / rc) ** 2, 0.0, None)
    return np.exp(-r / length) * s * s


def synthetic_beta(rho: np.ndarray) -> np.ndarray:
    """beta(rho) = 0.05 + 0.02 tanh(rho - 2) in eV ps / A^2 (>= 0.03)."""
    return 0.05 + 0.02 * np.tanh(np.asarray(rho, dtype=np.float64) - 2.0)


def write_beta_file(path: str, elements=("Ni",), numbers=(28,), n_rho: int = 2000, rc: float = 4.6,
                    n_beta: int = 2000, drho: float = 0.005, rho_fn=synthetic_rho, beta_fn=synthetic_beta) -> str:
    """Write a beta file in the reference format (three comment lines,
    "N name...", "Nrho dr Nbeta drho rcut", then per element Z, the Nrho
    rho(r) knots and the Nbeta beta(rho) knots), values round-trip exact."""
    dr = rc / (n_rho - 1)
    r = np.arange(n_rho) * dr
    rho_knots = rho_fn(r)
    beta_knots = beta_fn(np.arange(n_beta) * drho)
    with open(path, "w") as f:
        f.write("# synthetic beta(rho) file\n")
        f.write("# rho(r) = exp(-r/0.6)*(1-(r/rc)^2)^2, beta(rho) = 0.05 + 0.02 tanh(rho - 2)\n")
        f.write("# r in A, beta in eV ps / A^2\n")
        f.write(f"{len(elements)} {' '.join(elements)}\n")
        f.write(f"{n_rho} {dr!r} {n_beta} {drho!r} {rc!r}\n")
        for k, z in enumerate(numbers):
            f.write(f"{z}\n")
            scale = 1.0 + 0.1 * k  # distinct densities per element for multi-element files
            f.write("\n".join(repr(float(val)) for val in rho_knots * scale))
            f.write("\n")
            f.write("\n".join(repr(float(val)) for val in beta_knots * (1.0 + 0.05 * k)))
            f.write("\n")
    return path


def fix_args(beta_file: str, seed: int = 4242, flags: int | str = 7, model: int = 4, rho_e: float = 1.0,
             C_e: float = 3.5e-6, kappa_e: float = 0.1, T_e: float = 300.0, grid=(10, 10, 10),
             T_infile: str = "NULL", T_freq: int = 0, T_out: str = "Te_out", elements=("Ni",),
             fix_id: str = "eph", group: str = "all") -> list[str]:
    """The words of `fix ID group eph seed flags model rho_e C_e kappa_e T_e
    NX NY NZ T_infile freq Te_out beta_file A B ...` (README.md:186-214)."""
    return [fix_id, group, "eph", str(seed), str(flags), str(model), repr(rho_e), repr(C_e), repr(kappa_e),
            repr(T_e), str(grid[0]), str(grid[1]), str(grid[2]), T_infile, str(T_freq), T_out, beta_file,
            *elements]


def gaussian_stream(n_in_group: int, seed: int, step: int) -> np.ndarray:
    """Deviates a RanMars-like source would hand the fix in one step: three
    per in-group atom, atom order.  Seeded per (seed, step)."""
    return np.random.default_rng([seed, step]).standard_normal(3 * n_in_group)


def batched_cascades(nrep: int = 64, beta_file: str = "synth.beta", seed: int = 2024, min_atoms: int = 32000,
                     max_atoms: int = 500000):
    """Independent fcc Ni cascades for the batched form: atom counts drawn
    log-uniformly in [min_atoms, max_atoms] and rounded to whole fcc cells
    (4 n^3 atoms, cubic boxes), a PKA of 1-20 keV in a random direction per
    replica, an FDM grid from 16^3 to 48^3 growing with the box, one seed per
    replica.  Returns a list of (words, atoms)."""
    rng = np.random.default_rng(seed)
    out = []
    for r in range(nrep):
        target = math.exp(rng.uniform(math.log(min_atoms), math.log(max_atoms)))
        n = int(round((target / 4.0) ** (1.0 / 3.0)))
        n = max(20, min(50, n))
        at = fcc_lattice(n, seed=seed + 17 * r)
        add_pka(at, float(rng.uniform(1000.0, 20000.0)), seed=seed + 31 * r)
        g = int(round(16 + (n - 20) * 32.0 / 30.0))
        words = fix_args(beta_file, seed=seed + r + 1, flags=7, model=4, grid=(g, g, g))
        out.append((words, at))
    return out


def write_grid_file(path, n=(8, 6, 5), box=((0.0, 17.6), (0.0, 17.6), (0.0, 17.6)), T=300.0, C_e=3.5e-6,
                    rho_e=1.0, kappa_e=0.1, parameter_file=None, seed=0, walls=True, tdyn=False):
    """A grid file in the reference format (Doc/FDM/T_input.fdm, read by
    eph_fdm.h:48-119): three comment lines, "nx ny nz steps", three box lines,
    the parameter-file name (or NULL), then one line per cell
    "i j k T S rho_e C_e kappa_e flag T_dynamic".  With walls, the x = 0
    plane is ZERO_DERIVATIVE and one y-z line is CONSTANT; tdyn marks the
    DYNAMIC cells temperature dependent.  Values carry the file's %.6e
    precision; returns the path."""
    rng = np.random.default_rng(seed)
    with open(path, "w") as f:
        f.write("# grid\n#\n#\n")
        f.write(f"{n[0]} {n[1]} {n[2]} 1\n")
        for lo, hi in box:
            f.write(f"{lo:.6e} {hi:.6e}\n")
        f.write((parameter_file or "NULL") + "\n")
        for k in range(n[2]):
            for j in range(n[1]):
                for i in range(n[0]):
                    fl = 1
                    if walls and i == 0:
                        fl = 2
                    elif walls and j == 0 and k == 0:
                        fl = 0
                    t = T * rng.uniform(0.8, 1.6)
                    s = rng.uniform(-1e-3, 1e-3) if fl == 1 and i == 2 else 0.0
                    td = 1 if (tdyn and fl == 1) else 0
                    f.write(f"{i} {j} {k} {t:.6e} {s:.6e} {rho_e:.6e} {C_e * rng.uniform(0.8, 1.2):.6e} "
                            f"{kappa_e * rng.uniform(0.8, 1.2):.6e} {fl} {td}\n")
    return path


def write_grid_parameters(path, n=1001, dT=10.0, C0=3.5e-6, T0=3000.0, kappa0=0.1):
    """A grid parameter file (eph_fdm.h:73-104): three comment lines, "n dT",
    then C_e(T) and kappa_e(T) on T = 0, dT, ...: C_e = C0 (1 + T/T0),
    kappa_e = kappa0 (1 + T/T0) / (1 + (T/T0)^2)."""
    T = np.arange(n) * dT
    C = C0 * (1.0 + T / T0)
    K = kappa0 * (1.0 + T / T0) / (1.0 + (T / T0) ** 2)
    with open(path, "w") as f:
        f.write("#\n#\n#\n")
        f.write(f"{n} {dT!r}\n")
        for c, k in zip(C, K):
            f.write(f"{c:.6e} {k:.6e}\n")
    return path


# Sutton-Chen parameters for Ni (A. P. Sutton and J. Chen, Phil. Mag. Lett. 61,
# 139 (1990)): E = eps [1/2 sum_ij (a/r)^n - c sum_i sqrt(rho_i)], rho_i =
# sum_j (a/r)^m — an EAM form with phi(r) = eps (a/r)^n, f(r) = (a/r)^m,
# F(rho) = -c eps sqrt(rho).
SC_NI = dict(eps=1.5707e-2, a=3.52, c=39.432, n=9, m=6)


def _taper(r, r_on, rc):
    """1 below r_on, 0 from rc on, C2 smoothstep between."""
    x = np.clip((r - r_on) / (rc - r_on), 0.0, 1.0)
    return 1.0 - x ** 3 * (10.0 - 15.0 * x + 6.0 * x * x)


def write_eam_sutton_chen(path: str, rc: float = 6.0, r_on: float = 5.0, nr: int = 3001, nrho: int = 2001,
                          rho_max: float = 500.0, r_core: float = 1.5, p=SC_NI, element="Ni", z=28,
                          mass=NI_MASS) -> str:
    """Write a setfl (eam/alloy) file of the Sutton-Chen Ni potential, cut
    smoothly between r_on and rc.  Below r_core the tabulated r*phi(r) and
    f(r) continue linearly (finite, repulsive)."""
    dr = rc / (nr - 1)
    drho = rho_max / (nrho - 1)
    r = np.arange(nr) * dr
    rr = np.maximum(r, r_core)
    s = _taper(rr, r_on, rc)
    f = (p["a"] / rr) ** p["m"] * s
    zphi = rr * p["eps"] * (p["a"] / rr) ** p["n"] * s
    # linear continuation below r_core (slopes at r_core)
    k = r < r_core
    h = 1e-6
    fs = ((p["a"] / (r_core + h)) ** p["m"] - (p["a"] / (r_core - h)) ** p["m"]) / (2 * h)
    zs = ((r_core + h) * p["eps"] * (p["a"] / (r_core + h)) ** p["n"] -
          (r_core - h) * p["eps"] * (p["a"] / (r_core - h)) ** p["n"]) / (2 * h)
    f[k] = f[k] + fs * (r[k] - r_core)
    zphi[k] = zphi[k] + zs * (r[k] - r_core)
    F = -p["c"] * p["eps"] * np.sqrt(np.arange(nrho) * drho)
    with open(path, "w") as fd:
        fd.write("# Sutton-Chen Ni (Sutton & Chen 1990), eam/alloy tables\n")
        fd.write(f"# eps {p['eps']} eV, a {p['a']} A, c {p['c']}, n {p['n']}, m {p['m']}; "
                 f"C2 cut-off between {r_on} and {rc} A\n#\n")
        fd.write(f"1 {element}\n")
        fd.write(f"{nrho} {drho!r} {nr} {dr!r} {rc!r}\n")
        fd.write(f"{z} {mass!r} {p['a']!r} fcc\n")
        for arr in (F, f, zphi):
            fd.write("\n".join(repr(float(v)) for v in arr) + "\n")
    return path
