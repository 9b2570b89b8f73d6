"""The allocation-free grid solve (eph_fdm_solve_noalloc) against the grid
solve of the fix context.

Callers that own every byte of device memory (an engine's own device pool, a
time-step loop that must not synchronise the device through cudaMalloc)
cannot let the library allocate; this entry point works on their device
arrays plus a static scratch array.  Two calls in a row must give the same
temperatures as two end_of_step calls of a context built from the same grid
file (flags 4: grid only, so end_of_step is exactly one EPH_FDM::solve).
This file is collected last so a failure here leaves every other test run."""
import ctypes as C

import numpy as np
import pytest

import ephgb
from ephgb import workloads as W
from helpers import atom_err

pytestmark = pytest.mark.gpu
TOL = 1e-12


def write_grid(path, n=(12, 10, 8), box=(0.0, 24.0, -5.0, 15.0, 1.0, 17.0), seed=3, steps=1):
    """A grid file in the reference format with DYNAMIC, CONSTANT and
    ZERO_DERIVATIVE cells and sources (`steps` substeps at least per solve);
    returns the per-cell arrays."""
    rng = np.random.default_rng(seed)
    nt = n[0] * n[1] * n[2]
    arrays = {k: np.zeros(nt) for k in ("T", "S", "rho", "C", "kappa")}
    flag = np.zeros(nt, dtype=np.int8)
    with open(path, "w") as f:
        f.write("# grid\n#\n#\n")
        f.write(f"{n[0]} {n[1]} {n[2]} {steps}\n")
        f.write(f"{box[0]:.6e} {box[1]:.6e}\n{box[2]:.6e} {box[3]:.6e}\n{box[4]:.6e} {box[5]:.6e}\nNULL\n")
        for k in range(n[2]):
            for j in range(n[1]):
                for i in range(n[0]):
                    fl = 2 if i == 0 else (0 if (j == 0 and k == 0) else 1)
                    vals = [float(f"{v:.6e}") for v in (rng.uniform(200, 2000), rng.uniform(-50, 50) if i == 4 else 0.0,
                                                        rng.uniform(0.5, 1.5), rng.uniform(1e-6, 5e-6),
                                                        rng.uniform(0.05, 0.2))]
                    f.write(f"{i} {j} {k} " + " ".join(f"{v:.6e}" for v in vals) + f" {fl} 0\n")
                    c = i + n[0] * (j + n[1] * k)
                    for key, v in zip(("T", "S", "rho", "C", "kappa"), vals):
                        arrays[key][c] = v
                    flag[c] = fl
    arrays["flag"] = flag
    return arrays


def _device_grid(g, torch):
    dev = torch.device("cuda:0")
    d = {k: torch.tensor(g[k], dtype=torch.float64, device=dev) for k in ("T", "S", "rho", "C", "kappa")}
    d["dT"] = torch.zeros_like(d["T"])
    d["flag"] = torch.tensor(g["flag"], dtype=torch.int8, device=dev)
    return d


def _solve(d, n, lo, hi, dt, steps, nsub):
    p = {k: C.c_void_p(v.data_ptr()) for k, v in d.items()}
    return ephgb.lib().eph_fdm_solve_noalloc(n[0], n[1], n[2], lo.ctypes.data_as(ephgb._dp),
                                             hi.ctypes.data_as(ephgb._dp), dt, steps, p["T"], p["dT"], p["S"],
                                             p["rho"], p["C"], p["kappa"], p["flag"], None, C.byref(nsub))


# (dt, substeps asked for in the grid file): dt 0.002 needs many stability
# substeps; dt 1e-6 is stable as asked, so one substep ends in the scratch
# buffer (copied back into T) and two end in T itself
CASES = [(0.002, 1), (1e-6, 1), (1e-6, 2)]


@pytest.mark.parametrize("dt,steps", CASES)
def test_noalloc_solve_matches_the_context(built, beta_file, tmp_path, dt, steps):
    torch = pytest.importorskip("torch")
    path = str(tmp_path / "T.in")
    g = write_grid(path, steps=steps)
    n, lo, hi = (12, 10, 8), np.array([0.0, -5.0, 1.0]), np.array([24.0, 15.0, 17.0])
    words = W.fix_args(beta_file, flags=4, T_infile=path, grid=(1, 1, 1))
    atoms = W.fcc_lattice(5, seed=9)
    fix = ephgb.FixEPH(words, atoms, dt=dt)
    want_nsub, _ = ephgb.Grid(path).substeps(dt)
    if dt < 1e-3:
        assert want_nsub == steps
    else:
        assert want_nsub > 2
    d = _device_grid(g, torch)
    nsub = C.c_uint()
    for call in range(2):
        fix.end_of_step()
        want = fix.get("T")
        torch.cuda.synchronize()
        rc = _solve(d, n, lo, hi, dt, steps, nsub)
        assert rc == ephgb.EPH_OK, rc
        got = d["T"].cpu().numpy()
        assert nsub.value == want_nsub, (call, nsub.value, want_nsub)
        assert atom_err(got, want) <= TOL, (call, atom_err(got, want))


def test_noalloc_rejects_bad_bounds_before_launching(built, tmp_path):
    """C_e of cell 0 at zero (the stability rule starts from cell 0 whatever
    its flag) and a substep count above EPH_NOALLOC_MAX_SUBSTEPS are argument
    errors; T is left as it was."""
    torch = pytest.importorskip("torch")
    g = write_grid(str(tmp_path / "T.in"))
    n, lo, hi = (12, 10, 8), np.array([0.0, -5.0, 1.0]), np.array([24.0, 15.0, 17.0])
    nsub = C.c_uint()
    bad = dict(g)
    bad["C"] = g["C"].copy()
    bad["C"][0] = 0.0
    d = _device_grid(bad, torch)
    T0 = d["T"].clone()
    assert _solve(d, n, lo, hi, 0.002, 1, nsub) == 1  # EPH_ERR_ARG
    d = _device_grid(g, torch)
    assert _solve(d, n, lo, hi, 1e-6, 1000001, nsub) == 1  # more substeps asked for than allowed
    assert _solve(d, n, lo, hi, 1e4, 1, nsub) == 1  # more substeps required than allowed
    torch.cuda.synchronize()
    assert torch.equal(d["T"], T0)


def test_noalloc_rejects_grids_above_its_scratch(built):
    torch = pytest.importorskip("torch")
    L = ephgb.lib()
    lo, hi = np.zeros(3), np.ones(3)
    buf = torch.zeros(16, dtype=torch.float64, device="cuda:0")  # the size check returns before any use
    p = C.c_void_p(buf.data_ptr())
    rc = L.eph_fdm_solve_noalloc(65, 64, 64, lo.ctypes.data_as(ephgb._dp), hi.ctypes.data_as(ephgb._dp), 1e-3, 1,
                                 p, p, p, p, p, p, p, None, None)
    assert rc == 4  # EPH_ERR_CAPACITY
