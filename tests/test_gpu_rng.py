"""The device generator of the random force (Philox4x32-10 + Box-Muller) and
the physics it has to reproduce, checked statistically.

* the deviates: mean 0, variance 1, no correlation between components,
  atoms or steps, Gaussian tails;
* fluctuation-dissipation: with the electrons held at T_e (flags 3, no grid),
  the ions' kinetic temperature relaxes to T_e, and at T_ion = T_e the mean
  energy exchange per step vanishes while friction alone keeps removing
  energy."""
import math

import numpy as np
import pytest

import ephgb
from ephgb import workloads as W

pytestmark = pytest.mark.gpu


def test_deviates_are_standard_normal(built, beta_file):
    at = W.fcc_lattice(20, seed=41)  # 32,000 atoms -> 96,000 deviates per step
    fix = ephgb.FixEPH(W.fix_args(beta_file, flags=3, grid=(1, 1, 1)), at, dt=0.001)
    prev = None
    for s in range(4):
        fix.step(1)
        xi = fix.get("xi")
        z = xi.ravel()
        n = z.size
        assert abs(z.mean()) < 5.0 / math.sqrt(n)
        assert abs(z.var() - 1.0) < 5.0 * math.sqrt(2.0 / n)
        c = np.corrcoef(xi.T)
        assert np.abs(c - np.eye(3)).max() < 5.0 / math.sqrt(at.n)
        # neighbouring atoms and consecutive steps are independent
        assert abs(np.corrcoef(z[:-3], z[3:])[0, 1]) < 5.0 / math.sqrt(n)
        if prev is not None:
            assert abs(np.corrcoef(prev, z)[0, 1]) < 5.0 / math.sqrt(n)
        prev = z
        # tails: P(|z| > 3) = 0.0027
        tail = (np.abs(z) > 3.0).mean()
        assert abs(tail - 0.0026998) < 6.0 * math.sqrt(0.0027 / n)
        fourth = (z ** 4).mean()
        assert abs(fourth - 3.0) < 0.1
        # FP64 deviates (53-bit uniforms, FP64 Box-Muller, as the reference's
        # RanMars Gaussian): almost none is an FP32 number
        assert (z == z.astype(np.float32)).mean() < 1e-4


def kinetic_T(v, mass):
    v = v - v.mean(axis=0)
    ke = 0.5 * W.MVV2E * mass * (v ** 2).sum()
    return 2.0 * ke / ((3 * v.shape[0] - 3) * W.BOLTZ)


def test_ions_relax_to_the_electron_temperature(built, beta_file):
    """T_e fixed at 2,000 K (no grid solve): the ions, started at 300 K, heat
    up to T_e (the electron-ion coupling relaxes them in ~0.1 ps)."""
    at = W.fcc_lattice(16, seed=42, temperature=300.0)
    fix = ephgb.FixEPH(W.fix_args(beta_file, flags=3, T_e=2000.0, grid=(1, 1, 1)), at, dt=0.001)
    T0 = kinetic_T(fix.get("v"), W.NI_MASS)
    temps = []
    for _ in range(30):
        fix.step(100)
        temps.append(kinetic_T(fix.get("v"), W.NI_MASS))
    late = np.mean(temps[-15:])
    assert T0 < 400.0
    assert abs(late - 2000.0) < 0.05 * 2000.0, (T0, temps)


def exchange_series(beta_file, xi_source, steps=1000, seed=43):
    at = W.fcc_lattice(16, seed=seed, temperature=300.0)
    dt = 0.001
    fix = ephgb.FixEPH(W.fix_args(beta_file, flags=3, T_e=300.0, grid=(1, 1, 1)), at, dt=dt)
    rng = np.random.default_rng(seed)
    fric, rand = [], []
    for s in range(steps):
        if xi_source == "host":
            fix.step(1, xi=rng.standard_normal((at.n, 3)))
        else:
            fix.step(1)
        if s >= 100:
            v = fix.get("v")
            fric.append(-(fix.get("f_eph") * v).sum() * dt)
            rand.append(-(fix.get("f_rng") * v).sum() * dt)
    return np.array(fric), np.array(rand)


def test_exchange_balances_at_equal_temperatures(built, beta_file):
    """Ions and electrons both at 300 K: friction takes energy from the ions
    every step and the random force gives back as much on average
    (fluctuation-dissipation).  900 steps after 100 of settling: the mean net
    exchange per step is zero within four standard errors of the series plus
    1 % of the friction term (measured on GB300: -0.5 % +- 0.6 % over 900
    steps, -0.1 % +- 0.3 % over 2,900).  The device generator must give the
    same balance as a host Gaussian source driving the same dynamics."""
    fd, rd = exchange_series(beta_file, "device")
    fh, rh = exchange_series(beta_file, "host")
    for fric, rand in ((fd, rd), (fh, rh)):
        assert fric.mean() > 0.0 and rand.mean() < 0.0
        net = fric + rand
        stderr = net.std() / math.sqrt(len(net))
        assert abs(net.mean()) < 4.0 * stderr + 0.01 * fric.mean(), (net.mean(), stderr, fric.mean())
    ratio_d = -rd.mean() / fd.mean()
    ratio_h = -rh.mean() / fh.mean()
    err = 4.0 * math.hypot(rd.std() / fd.mean() / math.sqrt(len(rd)), rh.std() / fh.mean() / math.sqrt(len(rh)))
    assert abs(ratio_d - ratio_h) < max(err, 0.02), (ratio_d, ratio_h, err)


def test_coupled_ion_grid_energy_with_device_deviates(built, beta_file):
    """Ions at 300 K, electrons at 2,000 K on a 4^3 grid (flags 7, uniform
    C_e and kappa_e, periodic), device deviates: the ions' kinetic energy plus
    the grid's energy rho_e C_e dV sum T stays constant up to the velocity
    Verlet error of the friction/random forces (the reference's own comment,
    fix_eph.cpp:358-363: order dt^2).  600 steps of 0.5 fs: the drift stays
    under 1 % of the energy exchanged (measured on GB300: 0.05-0.4 %), and the
    grid's gain equals the fix's E_e output to rounding."""
    at = W.fcc_lattice(16, seed=44, temperature=300.0)
    words = W.fix_args(beta_file, flags=7, T_e=2000.0, grid=(4, 4, 4))
    fix = ephgb.FixEPH(words, at, dt=0.0005)
    rho_e, C_e = float(words[6]), float(words[7])
    dV = float(np.prod((at.boxhi - at.boxlo) / 4.0))

    def energies():
        v = fix.get("v")
        return 0.5 * W.MVV2E * W.NI_MASS * (v ** 2).sum(), rho_e * C_e * dV * fix.get("T").sum()

    ke0, eg0 = energies()
    E0 = fix.compute_vector(0)
    for block in range(3):
        fix.step(200)
        ke, eg = energies()
        gained = eg - eg0
        assert gained < 0.0  # the hot electrons heat the ions
        assert abs((ke - ke0) + gained) < 0.01 * abs(gained), (block, ke - ke0, gained)
        assert abs(gained - (fix.compute_vector(0) - E0)) < 1e-12 * abs(gained)
