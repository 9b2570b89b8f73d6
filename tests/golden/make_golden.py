"""Writes the golden fixtures of this directory from the reference itself.

  python tests/golden/make_golden.py [REFERENCE_TREE]

Needs the reference tree (default /root/reference) and the oracle build
(oracle/_ref/libephref.so: the reference fix_eph.cpp and eph_*.h compiled
unchanged with the engine stand-in).  Writes:
  fix_<scenario>.npz   inputs (x, v, type, mask, box, fix words, the injected
                       deviates) and the reference fix's outputs after every
                       step (x, v, f, rho, f_eph, f_rng, w, array, vector, T)
  beta_tables.npz      the reference splines of the synthetic beta file
  fdm_test1.npz        the reference's own FDM golden vectors
                       (Tests/EPH_FDM/Test1/Out_Ref/T_out_*: x and T_e columns)
The synthetic beta file is regenerated from its formula by every user, so
only the knots' provenance (ephgb.workloads.write_beta_file) is recorded.
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "user-eph_gb300"))
sys.path.insert(0, os.path.join(REPO, "tests"))

from ephgb import workloads as W  # noqa: E402
from helpers import n_in_group, scenario  # noqa: E402
from oracle.bindings import RefBeta, RefFix  # noqa: E402

SCEN = {"c1_small": 3, "pka": 4, "two_elements": 2, "group": 2, "c1": 1, "ttm": 3, "coloured": 3}
EVERY_STEP = ("x", "v", "f", "rho", "vector", "T", "xi")  # the rest: last step only


def fix_fixture(name, beta_file, beta_file_2el, tmp):
    words, at, dt = scenario(name, beta_file, beta_file_2el)
    ref = RefFix(words, at, dt)
    grid = (int(words[10]), int(words[11]), int(words[12]))
    ng = n_in_group(at)
    rnd = int(words[4], 0) & 2
    rec = {k: [] for k in ("x", "v", "f", "rho", "f_eph", "f_rng", "w", "array", "vector", "T", "xi")}
    for s in range(SCEN[name]):
        xi = W.gaussian_stream(ng, 5, s) if rnd else np.zeros(0)
        ref.step(xi if rnd else None)
        rec["xi"].append(xi)
        for k in ("x", "v", "f", "rho", "f_eph", "f_rng", "w", "array", "vector"):
            rec[k].append(ref.get(k))
        rec["T"].append(ref.get_T(grid, at.boxlo, at.boxhi))
    words_rel = list(words)
    words_rel[16] = os.path.basename(words[16])
    data = {k: np.array(v) if k in EVERY_STEP else np.array(v[-1]) for k, v in rec.items()}
    np.savez_compressed(os.path.join(HERE, f"fix_{name}.npz"), x0=at.x, v0=at.v, type=at.type, mask=at.mask,
                        mass=at.mass, boxlo=at.boxlo, boxhi=at.boxhi, dt=dt, words=np.array(words_rel), **data)


def main():
    ref_tree = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    with tempfile.TemporaryDirectory() as tmp:
        bf = W.write_beta_file(os.path.join(tmp, "synth.beta"))
        bf2 = W.write_beta_file(os.path.join(tmp, "NiFe.beta"), elements=("Ni", "Fe"), numbers=(28, 26))
        for name in SCEN:
            fix_fixture(name, bf, bf2, tmp)
        b = RefBeta(bf)
        tabs = {f"t{w}": b.table(w, 0) for w in range(4)}
        rng = np.random.default_rng(1)
        r2 = rng.uniform(0, b.r_cutoff ** 2 * 0.999, 256)
        rho = rng.uniform(0, b.rho_cutoff, 256)
        np.savez_compressed(os.path.join(HERE, "beta_tables.npz"), r2=r2, rho=rho, rho_r_sq=b.eval(1, 0, r2),
                            beta=b.eval(2, 0, rho), alpha=b.eval(3, 0, rho), rc=b.r_cutoff, rho_cut=b.rho_cutoff,
                            **tabs)
    out = {}
    d = os.path.join(ref_tree, "Tests", "EPH_FDM", "Test1", "Out_Ref")
    for k in (0, 1, 2, 4, 8, 16, 32):
        a = np.loadtxt(os.path.join(d, f"T_out_{k:06d}"), skiprows=1)
        out[f"x{k}"] = a[:, 0]
        out[f"T{k}"] = a[:, 3]
    np.savez_compressed(os.path.join(HERE, "fdm_test1.npz"), **out)


if __name__ == "__main__":
    main()
