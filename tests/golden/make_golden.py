"""Writes the golden fixtures of this directory from the reference itself.

  python tests/golden/make_golden.py [REFERENCE_TREE]

The reference tree comes from the argument, else EPH_REFERENCE_TREE, else the
tree oracle/_ref/libephref.so was compiled from (oracle/_ref/tree.txt); the
oracle build (oracle/_ref/libephref.so: the reference fix_eph.cpp and eph_*.h
compiled unchanged with the engine stand-in) must exist.  Writes:
  fix_<scenario>.npz   inputs (x, v, type, mask, box, fix words, the injected
                       deviates) and the reference fix's outputs after every
                       step (x, v, f, rho, vector, T) or after the last step
                       (f_eph, f_rng, w, array)
  ref_inputs/*.xz      the reference's own input files the fix_<scenario>
                       fixtures of REF_SCEN read (beta files, a grid file, a
                       data file, an eam/alloy file), xz-compressed byte for
                       byte, so that hosts without the reference tree run them
  synth.beta.xz,       the synthetic beta files the fixtures were made from
  NiFe.beta.xz         (ephgb.workloads.write_beta_file), kept byte for byte:
                       numpy's exp may round its last bit differently on
                       another host, so they are not regenerated there
  beta_tables.npz      the reference splines of the synthetic beta file
  fdm_test1.npz        the reference's own FDM golden vectors
                       (Tests/EPH_FDM/Test1/Out_Ref/T_out_*: x and T_e columns)
"""
import lzma
import math
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
from golden_io import REF_FILES, REF_INPUTS, write_ref_input  # noqa: E402
from helpers import n_in_group, scenario  # noqa: E402
from oracle.bindings import RefBeta, RefFix, reference_tree  # noqa: E402

SCEN = {"c1_small": 3, "pka": 4, "two_elements": 2, "group": 2, "c1": 1, "ttm": 3, "coloured": 3}
# scenarios on the reference's own input files: steps run, and the steps after
# which x, v, f, rho, vector and T are recorded (their deviates are not stored:
# W.gaussian_stream(atoms in group, xi_seed, step) regenerates them)
REF_SCEN = {"md_run_deck": (3, (0, 1, 2)), "md_run": (10, (0, 3, 6, 9)), "beta_zero": (20, (0, 4, 7, 10, 13, 16, 19)),
            "nicocrfe": (6, (0, 2, 5)), "example4": (10, (0, 4, 9))}
XI_SEED = 5
EVERY_STEP = ("x", "v", "f", "rho", "vector", "T", "xi")  # the rest: last step only

# Tests/MD_Run/run.lmp:114 and Tests/EPH_Beta_zero/run.lmp (the same fix line)
DECK_WORDS = "friction all eph 1111 7 4 1.0 3.5e-6 0.1248 0.0 7 8 9 NULL 0 T_out Ni.beta Ni Ni".split()
# Examples/Example_4/run.lmp
EXAMPLE4_WORDS = "friction all eph 12345 7 4 1.0 1.0e-5 1.0e-9 300.0 9 9 9 T.in 1000 T_out Ni_model_4.beta Ni".split()
# Tests/MD_Run/run.lmp: PKA speed (A/ps) and direction; dt = 1e-3 A / speed
DECK_SPEED = 573.39111597
DECK_DIR = (0.835115, 0.543981, 0.081652)
MASSES = {"Ni": 58.69, "Co": 58.933, "Cr": 51.996, "Fe": 55.845}


def _deck_lattice(jitter, temperature, seed):
    """8^3 fcc cells with the centre atom replaced by a type-2 atom appended
    last (the deck's delete_atoms + create_atoms 2 single n/2 n/2 n/2)."""
    at = W.fcc_lattice(8, jitter=jitter, temperature=temperature, seed=seed)
    centre = np.array([4.0, 4.0, 4.0]) * W.NI_LATTICE
    d = at.x - centre
    d -= np.round(d / (at.boxhi - at.boxlo)) * (at.boxhi - at.boxlo)
    k = int(np.argmin((d ** 2).sum(axis=1)))
    keep = np.arange(at.n) != k
    x = np.vstack([at.x[keep], centre[None, :]])
    v = np.vstack([at.v[keep], np.zeros((1, 3))])
    typ = np.concatenate([at.type[keep], [2]]).astype(np.int32)
    return W.Atoms(x=x, v=v, type=typ, mask=np.ones(x.shape[0], dtype=np.int32), boxlo=at.boxlo,
                   boxhi=at.boxhi, mass=np.array([0.0, W.NI_MASS, W.NI_MASS]))


def _read_data_file(path):
    """Atoms of a LAMMPS data file with `Atoms # atomic` and `Velocities`
    sections (Examples/Example_4/struc_in.data), in id order."""
    lines = open(path).read().splitlines()
    n = int(next(ln for ln in lines if ln.strip().endswith("atoms")).split()[0])
    lo, hi = np.zeros(3), np.zeros(3)
    for ln in lines:
        for a, key in enumerate(("xlo", "ylo", "zlo")):
            if key in ln:
                p = ln.split()
                lo[a], hi[a] = float(p[0]), float(p[1])
    sec = {}
    for s in ("Masses", "Atoms", "Velocities"):
        i = next(k for k, ln in enumerate(lines) if ln.startswith(s))
        rows = []
        for ln in lines[i + 2:]:
            if not ln.strip():
                break
            rows.append(ln.split())
        sec[s] = rows
    atoms = sorted(sec["Atoms"], key=lambda r: int(r[0]))
    vel = {int(r[0]): [float(c) for c in r[1:4]] for r in sec["Velocities"]}
    x = np.array([[float(c) for c in r[2:5]] for r in atoms])
    typ = np.array([int(r[1]) for r in atoms], dtype=np.int32)
    v = np.array([vel[int(r[0])] for r in atoms])
    mass = np.zeros(len(sec["Masses"]) + 1)
    for r in sec["Masses"]:
        mass[int(r[0])] = float(r[1])
    assert x.shape[0] == n
    return W.Atoms(x=x, v=v, type=typ, mask=np.ones(n, dtype=np.int32), boxlo=lo, boxhi=hi, mass=mass)


def ref_scenario(name, tmp):
    """(words, atoms, dt) of a scenario on the reference's input files
    (written into tmp by name, as the words name them)."""
    if name == "md_run_deck":  # the deck as written: perfect lattice at rest, T_e = 0, the PKA
        at = _deck_lattice(0.0, 0.0, 1)
        at.v[-1] = DECK_SPEED * np.array(DECK_DIR)
        words = list(DECK_WORDS)
        words[16] = "MD_Run_Ni.beta"
        return words, at, 1.0e-3 / DECK_SPEED
    if name == "md_run":  # the deck's fix line on a thermal lattice (300 K, jitter 0.05 A), dt 0.5 fs
        at = _deck_lattice(0.05, 300.0, 31)
        at.v[-1] = DECK_SPEED * np.array(DECK_DIR)
        words = list(DECK_WORDS)
        words[16] = "MD_Run_Ni.beta"
        return words, at, 0.0005
    if name == "beta_zero":
        # Tests/EPH_Beta_zero: rho_cutoff = 5.0 (drho 1e-4); the deck's PKA speed
        # (1000 A/ps along x, dt 1e-4) with the PKA started 0.9 A in front of a
        # lattice atom, 0.25 A off its line: the pair's densities pass 5.0 on
        # the way in (beta = alpha = 0 there, eph_beta.h:174-197) and back out
        at = _deck_lattice(0.05, 300.0, 32)
        target = np.array([5.0, 4.0, 4.0]) * W.NI_LATTICE
        at.x[-1] = target + np.array([-0.9, 0.25, 0.0])
        at.v[-1] = np.array([1000.0, 0.0, 0.0])
        words = list(DECK_WORDS)
        words[16] = "Beta_zero_Ni.beta"
        return words, at, 1.0e-4
    if name == "nicocrfe":  # the four-element beta file, types 1-4 at random, a 1 keV knock-on atom
        at = W.fcc_lattice(6, seed=33)
        rng = np.random.default_rng(34)
        at.type = rng.integers(1, 5, at.n).astype(np.int32)
        at.mass = np.array([0.0] + [MASSES[e] for e in ("Ni", "Co", "Cr", "Fe")])
        W.add_pka(at, 1000.0, seed=35)
        words = W.fix_args("NiCoCrFe_PRB2019.beta", seed=77, grid=(6, 6, 6), elements=("Ni", "Co", "Cr", "Fe"))
        return words, at, 0.001
    if name == "example4":  # Examples/Example_4 as written: its atoms, grid file and beta file
        at = _read_data_file(os.path.join(tmp, "Example_4_struc_in.data"))
        words = list(EXAMPLE4_WORDS)
        words[13] = "Example_4_T.in"
        words[16] = "Example_4_Ni_model_4.beta"
        return words, at, 0.00005
    raise KeyError(name)


def record(ref, words, at, nsteps, xi_seed=XI_SEED, steps=None):
    """Steps the reference fix nsteps times; per step (or per step listed in
    `steps`, then without the deviates) the every-step arrays, and the rest
    after the last step."""
    grid = (int(words[10]), int(words[11]), int(words[12]))
    ng = n_in_group(at)
    rnd = int(words[4], 0) & 2
    rec = {k: [] for k in ("x", "v", "f", "rho", "f_eph", "f_rng", "w", "array", "vector", "T", "xi")}
    for s in range(nsteps):
        xi = W.gaussian_stream(ng, xi_seed, s) if rnd else np.zeros(0)
        ref.step(xi if rnd else None)
        if steps is not None and s not in steps and s != nsteps - 1:
            continue
        rec["xi"].append(xi)
        for k in ("x", "v", "f", "rho", "f_eph", "f_rng", "w", "array", "vector"):
            rec[k].append(ref.get(k))
        rec["T"].append(ref.get_T(grid, at.boxlo, at.boxhi))
    out = {k: np.array(v) if k in EVERY_STEP else np.array(v[-1]) for k, v in rec.items()}
    if steps is not None:
        del out["xi"]
        out.update(steps=np.array(steps), nsteps=nsteps, xi_seed=xi_seed)
    return out


def save_fixture(name, words, at, dt, data):
    words_rel = list(words)
    for i in (13, 15, 16):
        if words_rel[i] != "NULL":
            words_rel[i] = os.path.basename(words_rel[i])
    np.savez_compressed(os.path.join(HERE, f"fix_{name}.npz"), x0=at.x, v0=at.v, type=at.type, mask=at.mask,
                        mass=at.mass, boxlo=at.boxlo, boxhi=at.boxhi, dt=dt, words=np.array(words_rel), **data)


def fix_fixture(name, beta_file, beta_file_2el):
    words, at, dt = scenario(name, beta_file, beta_file_2el)
    save_fixture(name, words, at, dt, record(RefFix(words, at, dt), words, at, SCEN[name]))


def ref_fixture(name, tmp):
    words, at, dt = ref_scenario(name, tmp)
    words = list(words)
    for i in (13, 16):
        if words[i] != "NULL":
            words[i] = os.path.join(tmp, words[i])
    words[15] = os.path.join(tmp, "T_out")
    nsteps, steps = REF_SCEN[name]
    assert steps[-1] == nsteps - 1
    save_fixture(name, words, at, dt, record(RefFix(words, at, dt), words, at, nsteps, steps=steps))


def copy_ref_inputs(ref_tree):
    os.makedirs(REF_INPUTS, exist_ok=True)
    for name, rel in REF_FILES.items():
        data = open(os.path.join(ref_tree, rel), "rb").read()
        with open(os.path.join(REF_INPUTS, name + ".xz"), "wb") as f:
            f.write(lzma.compress(data, preset=9))


def main():
    ref_tree = sys.argv[1] if len(sys.argv) > 1 else (os.environ.get("EPH_REFERENCE_TREE") or reference_tree())
    if not ref_tree or not os.path.isdir(ref_tree):
        sys.exit("give the reference tree (argument or EPH_REFERENCE_TREE)")
    copy_ref_inputs(ref_tree)
    with tempfile.TemporaryDirectory() as tmp:
        bf = W.write_beta_file(os.path.join(tmp, "synth.beta"))
        bf2 = W.write_beta_file(os.path.join(tmp, "NiFe.beta"), elements=("Ni", "Fe"), numbers=(28, 26))
        for path in (bf, bf2):
            with open(os.path.join(HERE, os.path.basename(path) + ".xz"), "wb") as f:
                f.write(lzma.compress(open(path, "rb").read(), preset=9))
        for name in SCEN:
            fix_fixture(name, bf, bf2)
        for name in REF_FILES:
            write_ref_input(name, tmp)
        for name in REF_SCEN:
            ref_fixture(name, tmp)
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
    assert math.isfinite(float(out["T1"].sum()))


if __name__ == "__main__":
    main()
