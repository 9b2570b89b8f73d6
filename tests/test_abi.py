"""The C ABI library: it loads without a GPU, exports every function that
include/eph_gb.h declares, and its host-side parts (beta file, splines, grid
files) run on the CPU."""
import os
import re

import numpy as np
import pytest

import ephgb

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "eph_gb.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(eph_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_hooks():
    names = declared_functions()
    for hook in ("eph_create", "eph_initial_integrate", "eph_post_force", "eph_final_integrate", "eph_end_of_step",
                 "eph_compute_vector", "eph_post_run", "eph_save_state", "eph_save_temperature", "eph_reset_dt"):
        assert hook in names


def test_library_exports_every_declared_symbol(built):
    L = ephgb.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_signatures_cover_the_header(built):
    assert set(declared_functions()) == set(ephgb.SIGNATURES)


def test_status_strings(built):
    L = ephgb.lib()
    assert L.eph_status_string(0) == b"ok"
    assert L.eph_status_string(4) == b"capacity exceeded"


def test_create_rejects_bad_words_without_gpu(built, beta_file):
    """Argument errors are reported before any device work (fix_eph.cpp:64)."""
    from ephgb import workloads as W

    words = W.fix_args(beta_file)[:17]
    with pytest.raises(ephgb.EphError) as e:
        ephgb.FixEPH(words, W.fcc_lattice(5))
    assert e.value.status == 1 and "too few arguments" in str(e.value)
    words = W.fix_args(beta_file, model=2)
    with pytest.raises(ephgb.EphError) as e:
        ephgb.FixEPH(words, W.fcc_lattice(5))
    assert e.value.status == 3
    words = W.fix_args(beta_file, elements=("Cu",))
    with pytest.raises(ephgb.EphError) as e:
        ephgb.FixEPH(words, W.fcc_lattice(5))
    assert "elements not found" in str(e.value)
    words = W.fix_args(beta_file, grid=(0, 4, 4))
    with pytest.raises(ephgb.EphError) as e:
        ephgb.FixEPH(words, W.fcc_lattice(5))
    assert "non-positive grid" in str(e.value)
    words = W.fix_args(os.path.join(os.path.dirname(beta_file), "missing.beta"))
    with pytest.raises(ephgb.EphError) as e:
        ephgb.FixEPH(words, W.fcc_lattice(5))
    assert e.value.status == 2
