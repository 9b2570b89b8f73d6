import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "user-eph_gb300"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built libephgb.so")


@pytest.fixture(scope="session")
def built():
    """Build the product library and the oracle once per session."""
    import __graft_entry__

    __graft_entry__.build()
    return True


@pytest.fixture(scope="session")
def beta_file(tmp_path_factory):
    """The synthetic beta file (ephgb.workloads.write_beta_file), the bytes
    the golden fixtures were made from, so every host tests the same knots."""
    from golden_io import write_synthetic_beta

    return write_synthetic_beta("synth.beta", str(tmp_path_factory.mktemp("beta")))


@pytest.fixture(scope="session")
def beta_file_2el(tmp_path_factory):
    from golden_io import write_synthetic_beta

    return write_synthetic_beta("NiFe.beta", str(tmp_path_factory.mktemp("beta2")))


def pytest_collection_modifyitems(config, items):
    """GPU tests need a device; skip them cleanly when torch sees none."""
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)
