"""The df64 (double-float) arithmetic of the FAST pair sweeps
(user-eph_gb300/csrc/eph_df64.cuh), built for the host from the same source
and checked against long double on seeded random operands
(tests/native/df64_check.cpp): every operation within a few units of 2^-48
(u); one atom's 42 pair terms summed as the sweeps sum them (blocks of 8)
within a few u of the largest entry of M_i, and the sums of random-sign terms
(S_i, the force sweep's sum, w_i = M_i v_i - S_i) within ~60 u of their
largest component: those terms cancel to a tenth of their absolute sum, and
the same cancellation scales the FP64 reference's own rounding.  Measured:
add 1.9 u, mul 3.2, recip 4.4, displacement 27 (the bin offsets carry 2^-48
of up to one bin edge), dot3 5.0, local-form spline 1.5, M_i 4.4, S_i 63,
w_i 30, force sum 64; the EAM sweeps' square root 2.1 u, also with its FP32
seed off by 2^-22 relative (the device estimate's error class).  No GPU."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "user-eph_gb300", "csrc")
U = 2.0 ** -48
# bound per line, in units of 2^-48, with headroom over the measured values
BOUNDS = {"add": 4, "mul": 6, "recip": 8, "displacement": 60, "dot3": 10, "horner": 4, "atom_M": 12, "atom_S": 150,
          "atom_w": 80, "atom_force_sum": 150, "sqrt": 6, "sqrt_seed_2e-7": 6}


@pytest.fixture(scope="module")
def results(tmp_path_factory):
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("df64") / "df64_check")
    subprocess.run([cxx, "-O2", "-ffp-contract=off", "-fno-fast-math", "-std=c++17", "-I" + CSRC, "-o", exe,
                    os.path.join(HERE, "native", "df64_check.cpp")], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    return {ln.split()[0]: float(ln.split()[1]) for ln in out.splitlines() if ln.strip()}


def test_spline_index_estimate(results):
    """floor_estimate (the density sweep's knot index): floor(q) or one less,
    never negative, over 0 <= q < 4e6 (dense near 0, where a first version
    that rounded near 2^23 returned -1 for q < 0.5)."""
    assert results["floor_estimate_bad"] == 0


@pytest.mark.parametrize("name", sorted(BOUNDS))
def test_df64_error_bound(results, name):
    assert results[name] <= BOUNDS[name] * U, (name, results[name] / U)
