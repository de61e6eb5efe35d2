import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "ref_fixture_l3_n250.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine library")


@pytest.fixture(scope="session")
def golden():
    d = np.load(GOLDEN)
    return {k: d[k] for k in d.files}


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle

    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def engine():
    """The engine on cuda:0; builds the library first if this checkout has none."""
    import torch

    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    import nbfmm_gb300
    from nbfmm_gb300 import _lib, build

    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    nbfmm_gb300.load_library()
    return nbfmm_gb300


def guarded_rel_err(a, ref):
    """max_i |a_i - ref_i| / max(|ref_i|, 1e-3 * median |ref|) over particles (2-vectors)."""
    a = np.asarray(a, np.float64).reshape(-1, 2)
    ref = np.asarray(ref, np.float64).reshape(-1, 2)
    mag = np.linalg.norm(ref, axis=1)
    guard = np.maximum(mag, 1e-3 * np.median(mag) if len(mag) else 0.0)
    guard[guard == 0] = 1.0
    err = np.linalg.norm(a - ref, axis=1) / guard
    return float(err.max()) if len(err) else 0.0, err
