"""The rule behind the kept candidate lists (k_list_check, k_list_mark,
k_density_list), restated in numpy and checked against a brute-force pair
search: after a build with list radius r_cutoff + s, any displacements, at
most 32 atoms past s/2 ("moved"), atoms whose build position lies within
r_cutoff + s/2 of a moved atom's current position flagged; an unflagged atom
takes its list, a flagged or moved one searches the build positions within
r_cutoff + s (moved atoms left out) and adds every moved atom.  Every pair
within r_cutoff must then be a candidate exactly once.  No GPU."""
import numpy as np
import pytest

RC, SKIN, L = 4.6, 0.3, 24.0
FMAX = 32


def min_image(d):
    return d - L * np.round(d / L)


def dist2(a, b):
    d = min_image(b[None, :, :] - a[:, None, :])
    return (d * d).sum(axis=2)


def candidates(x_build, x_now, mark=True):
    n = len(x_build)
    lists = dist2(x_build, x_build) < (RC + SKIN) ** 2
    np.fill_diagonal(lists, False)
    disp2 = (min_image(x_now - x_build) ** 2).sum(axis=1)
    moved = disp2 >= (0.5 * SKIN) ** 2
    if moved.sum() > FMAX:
        return None  # a build step
    flagged = moved.copy()
    if moved.any() and mark:
        near = dist2(x_build, x_now[moved]) < (RC + 0.5 * SKIN) ** 2  # [atom, moved atom]
        flagged |= near.any(axis=1)
    ref = np.where(moved[:, None], x_now, x_build)  # a moved atom searches around where it is now
    fresh = dist2(ref, x_build) < (RC + SKIN) ** 2
    fresh[:, moved] = False
    fresh[:, np.flatnonzero(moved)] |= True
    np.fill_diagonal(fresh, False)
    return np.where(flagged[:, None], fresh, lists)


def displaced(seed):
    """Build positions and current ones: every atom displaced by up to just
    below s/2, then 1 to 32 of them by a few angstrom"""
    rng = np.random.default_rng(seed)
    n = 400
    x_build = rng.uniform(0.0, L, size=(n, 3))
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    step = u * rng.uniform(0.0, 0.4999 * SKIN, size=(n, 1))  # unmoved atoms: up to just below s/2
    fast = rng.choice(n, size=rng.integers(1, FMAX + 1), replace=False)
    step[fast] = rng.normal(scale=3.0, size=(len(fast), 3))  # moved atoms, some far
    return x_build, (x_build + step) % L


def missing_pairs(x_build, x_now, mark=True):
    cand = candidates(x_build, x_now, mark)
    assert cand is not None
    within = dist2(x_now, x_now) < RC * RC
    np.fill_diagonal(within, False)
    return int((within & ~cand).sum())


@pytest.mark.parametrize("seed", range(6))
def test_kept_lists_hold_every_pair(seed):
    assert missing_pairs(*displaced(seed)) == 0


def test_without_the_flags_pairs_go_missing():
    """The model can fail: without flagging the atoms near moved ones, the
    pairs a moved atom formed with atoms outside its list are lost."""
    assert sum(missing_pairs(*displaced(seed), mark=False) for seed in range(6)) > 0


def test_many_moved_atoms_build():
    rng = np.random.default_rng(7)
    x_build = rng.uniform(0.0, L, size=(200, 3))
    x_now = (x_build + rng.normal(scale=1.0, size=(200, 3))) % L
    assert candidates(x_build, x_now) is None
