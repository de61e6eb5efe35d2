import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "ref_fixture_l3_n250.npz")
DISPLAY_GOLDEN = os.path.join(ROOT, "tests", "golden", "ref_display_frames.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine library")


@pytest.fixture(scope="session")
def golden():
    d = np.load(GOLDEN)
    return {k: d[k] for k in d.files}


@pytest.fixture(scope="session")
def display_golden():
    """Frames drawn by the reference's displayDevice: a list of dicts (pos, w, width, height, size_scale, limits,
    frame)."""
    d = np.load(DISPLAY_GOLDEN)
    cases = []
    for k in range(int(d["num_cases"])):
        width, height = (int(v) for v in d[f"case{k}_params"])
        f = d[f"case{k}_fparams"]
        cases.append(dict(pos=d[f"case{k}_pos"], w=d[f"case{k}_w"], width=width, height=height,
                          size_scale=float(f[0]), limits=tuple(float(v) for v in f[1:]), frame=d[f"case{k}_frame"]))
    return cases


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


PARITY_TOL = 1e-5


def assert_solve_parity(eff, pos, w, num_level, limits, eps, orc, tol=PARITY_TOL):
    """Effects against the oracle's solve (p2pNaive order).

    p99.9 of the guarded relative error must be below `tol`. Its maximum must be below `tol` or, where the
    reference's own two P2P code paths -- p2pNaive and p2pBlock, chosen by N at p2p.cu:169 -- disagree by
    more than that on the same input (FP32 reordering under cancellation, e.g. uniform squares), below
    that disagreement. Returns (max, p99.9, reference disagreement)."""
    ref = orc.solve(pos, w, num_level, limits, eps)
    err, errs = guarded_rel_err(eff, ref)
    noise = guarded_rel_err(orc.solve(pos, w, num_level, limits, eps, block=True), ref)[0]
    p999 = float(np.quantile(errs, 0.999)) if len(errs) else 0.0
    assert p999 < tol, f"p99.9 guarded relative error {p999:.3e}"
    assert err < max(tol, noise), f"guarded relative error {err:.3e} (reference paths disagree by {noise:.3e})"
    return err, p999, noise
