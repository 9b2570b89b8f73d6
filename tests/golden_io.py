"""Loading the golden fixtures written by tests/golden/make_golden.py."""
import lzma
import os

import numpy as np

from ephgb import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REF_INPUTS = os.path.join(GOLDEN, "ref_inputs")
FIXTURES = ("c1_small", "pka", "two_elements", "group", "c1", "ttm", "coloured")
# fixtures on the reference's own input files (tests/golden/ref_inputs)
REF_FIXTURES = ("md_run_deck", "md_run", "beta_zero", "nicocrfe", "example4")

# the reference's input files kept in ref_inputs/<name>.xz: name -> path in the
# USER-EPH tree
REF_FILES = {
    "MD_Run_Ni.beta": "Tests/MD_Run/Ni.beta",  # 1001 rho knots, 50001 beta knots, rc 5 A, rho_cutoff 50
    "Beta_zero_Ni.beta": "Tests/EPH_Beta_zero/Ni.beta",  # the same knots with drho 1e-4: rho_cutoff 5
    "NiCoCrFe_PRB2019.beta": "Data/NiCoCrFe/NiCoCrFe_PRB2019.beta",  # four elements
    "Example_4_T.in": "Examples/Example_4/T.in",  # 9^3 grid file (current format, NULL parameter line)
    "Example_4_Ni_model_4.beta": "Examples/Example_4/Ni_model_4.beta",
    "Example_4_struc_in.data": "Examples/Example_4/struc_in.data",  # 500 atoms with velocities
    "MD_Run_Ni.eam": "Tests/MD_Run/Ni.eam",  # the decks' eam/alloy potential (setfl)
    # the LAMMPS run of that deck (fix print every 1000 steps: step, time, temp,
    # mean T_e, the knock-on atom's x y z, pe, ke, E_e, its rho and beta)
    "MD_Run_out.data": "Tests/MD_Run/Reference/out.data",
}


def ref_input_bytes(name):
    with open(os.path.join(REF_INPUTS, name + ".xz"), "rb") as f:
        return lzma.decompress(f.read())


def write_ref_input(name, tmpdir):
    """Write the reference's input file `name` into tmpdir; returns its path."""
    path = os.path.join(tmpdir, name)
    with open(path, "wb") as f:
        f.write(ref_input_bytes(name))
    return path


def write_synthetic_beta(name, tmpdir):
    """Write the synthetic beta file `name` ("synth.beta" or "NiFe.beta") the
    fixtures were made from (ephgb.workloads.write_beta_file on the host that
    made them, kept byte for byte) into tmpdir; returns its path."""
    path = os.path.join(tmpdir, name)
    with open(os.path.join(GOLDEN, name + ".xz"), "rb") as f, open(path, "wb") as out:
        out.write(lzma.decompress(f.read()))
    return path


def load_fix(name, tmpdir):
    """(words, atoms, dt, record): the beta file (synthetic or the
    reference's) and the grid file are unpacked into tmpdir, and the output
    file word points there too."""
    d = np.load(os.path.join(GOLDEN, f"fix_{name}.npz"))
    words = [str(w) for w in d["words"]]
    if words[16] in REF_FILES:
        words[16] = write_ref_input(words[16], tmpdir)
    else:
        words[16] = write_synthetic_beta(words[16], tmpdir)
    if words[13] in REF_FILES:
        words[13] = write_ref_input(words[13], tmpdir)
    words[15] = os.path.join(tmpdir, words[15])
    at = W.Atoms(x=d["x0"].copy(), v=d["v0"].copy(), type=d["type"].copy(), mask=d["mask"].copy(),
                 boxlo=d["boxlo"].copy(), boxhi=d["boxhi"].copy(), mass=d["mass"].copy())
    return words, at, float(d["dt"]), d


def fixture_steps(rec):
    """(steps to run, recorded step indices) of a fixture."""
    if "steps" in rec:
        return int(rec["nsteps"]), [int(s) for s in rec["steps"]]
    n = rec["x"].shape[0]
    return n, list(range(n))


def fixture_xi(rec, words, atoms, step, groupbit=1):
    """The deviates injected at `step` in draw order (None without random
    forces)."""
    if not int(words[4], 0) & 2:
        return None
    if "xi" in rec:
        return rec["xi"][step]
    ng = int(((atoms.mask & groupbit) != 0).sum())
    return W.gaussian_stream(ng, int(rec["xi_seed"]), step)
