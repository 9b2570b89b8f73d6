"""Why the pair loop keeps the exact spline index floor(r^2 / dx) in FP64.

An index from FP32 copies (r^2 truncated by its bits, an FP32 product) can
land one interval off when r^2 lies within ~2.4e-7 (relative) of a knot;
the neighbouring cubic is then evaluated next to its knot.  The tables are
C2 splines, so the two cubics meet there, and for the synthetic beta file
(and the reference's Ni.beta from 1.5 A on) they agree to ~1e-15.  But
Ni.beta's rho(r^2) spline has a sharp kink near r = 0.16 A, where the two
cubics differ by ~1e-8: beyond the 1e-12 parity bar for any atom such a
pair touches (atoms do come that close in cascades).  So the FP32 index,
measured 3 % faster in the density sweep, is not used.  Host tables only,
no GPU."""

import numpy as np
import pytest

import ephgb
from ephgb import workloads as W
from golden_io import write_ref_input

SLIP = 2.5e-7  # relative distance from a knot within which an FP32 index can slip


def horner(c, x):
    return c[:, 0] + x * (c[:, 1] + x * (c[:, 2] + x * c[:, 3]))


def neighbour_gaps(path):
    """(r at each interior knot, largest |difference| of the two cubics
    meeting there, evaluated within SLIP of the knot)"""
    bf = ephgb.BetaFile(path)
    tab = bf.table("rho_r_sq", 0)
    n = tab.shape[0]
    dx = bf.r_cutoff ** 2 / (n - 1)
    k = np.arange(1, n - 1)
    gap = np.zeros(k.size)
    for rel in (-SLIP, 0.0, SLIP):
        x = k * dx * (1.0 + rel)
        gap = np.maximum(gap, np.abs(horner(tab[k - 1], x) - horner(tab[k], x)))
    return np.sqrt(k * dx), gap


def test_synthetic_beta_file(tmp_path):
    r, gap = neighbour_gaps(W.write_beta_file(str(tmp_path / "synth.beta")))
    assert gap.max() < 1e-14


def test_reference_ni_beta_needs_the_exact_index(tmp_path):
    """Tests/MD_Run/Ni.beta, kept under tests/golden/ref_inputs."""
    r, gap = neighbour_gaps(write_ref_input("MD_Run_Ni.beta", str(tmp_path)))
    assert gap[r >= 1.5].max() < 1e-14  # lattice distances: harmless
    # a lattice atom's density is ~0.05 (12 neighbours at 2.49 A, ~0.004 each):
    # near r = 0.16 A a slipped index would move it by far more than 1e-12
    assert gap[r < 0.3].max() > 1e-12 * 0.05
