"""Loading the golden fixtures written by tests/golden/make_golden.py."""
import os

import numpy as np

from ephgb import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = ("c1_small", "pka", "two_elements", "group", "c1", "ttm", "coloured")


def load_fix(name, tmpdir):
    """(words, atoms, dt, record) with the beta file regenerated in tmpdir."""
    d = np.load(os.path.join(GOLDEN, f"fix_{name}.npz"))
    words = [str(w) for w in d["words"]]
    if words[16] == "NiFe.beta":
        words[16] = W.write_beta_file(os.path.join(tmpdir, "NiFe.beta"), elements=("Ni", "Fe"), numbers=(28, 26))
    else:
        words[16] = W.write_beta_file(os.path.join(tmpdir, words[16]))
    at = W.Atoms(x=d["x0"].copy(), v=d["v0"].copy(), type=d["type"].copy(), mask=d["mask"].copy(),
                 boxlo=d["boxlo"].copy(), boxhi=d["boxhi"].copy(), mass=d["mass"].copy())
    return words, at, float(d["dt"]), d
