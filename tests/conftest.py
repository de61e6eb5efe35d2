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

# Per-case parity figures of this session, printed in the terminal summary (also under -q).
PARITY_RECORDS = []


def pytest_terminal_summary(terminalreporter, exitstatus, config):
    if not PARITY_RECORDS:
        return
    tr = terminalreporter
    tr.section("effect parity against the oracle (guarded relative error; bar 1e-5)")
    tr.write_line(f"{'case':<44} {'arith':<6} {'N':>10} {'max':>10} {'p99.9':>10} {'vs block':>10} "
                  f"{'fp64 med eng/orc':>20} {'fp64 max eng/orc':>20}")
    for r in PARITY_RECORDS:
        f64 = r.get("fp64")
        med = f"{f64[0]:.3e}/{f64[1]:.3e}" if f64 else "-"
        mx = f"{f64[2]:.3e}/{f64[3]:.3e}" if f64 else "-"
        blk = f"{r['block']:.3e}" if r.get("block") is not None else "-"
        tr.write_line(f"{r['case'][:44]:<44} {r['arith']:<6} {r['n']:>10} {r['max']:>10.3e} {r['p999']:>10.3e} "
                      f"{blk:>10} {med:>20} {mx:>20}")


def fp64_errors(eff, ref, pos, w, eps, orc, targets):
    """Relative error against the FP64 all-pairs direct sum at `targets` (original indices), of the engine's
    effects and of the oracle's: (median engine, median oracle, max engine, max oracle)."""
    d = orc.direct_f64(pos, w, eps, targets)
    mag = np.linalg.norm(d, axis=1)
    mag[mag == 0] = 1.0
    e_eng = np.linalg.norm(np.asarray(eff, np.float64)[targets] - d, axis=1) / mag
    e_orc = np.linalg.norm(np.asarray(ref, np.float64)[targets] - d, axis=1) / mag
    return float(np.median(e_eng)), float(np.median(e_orc)), float(e_eng.max()), float(e_orc.max())


def assert_solve_parity(eff, pos, w, num_level, limits, eps, orc, tol=PARITY_TOL, arithmetic="fast", case="",
                        ref=None, block=None, fp64_targets=256):
    """Effects of a solve against the oracle's (the reference's stages restated in IEEE single precision, P2P in
    p2pNaive order).

    arithmetic="exact": the engine evaluates kernelFunction with the oracle's operations (correctly rounded
    sqrt and division, no contraction) in the same order, so every effect must equal the oracle's bit for bit.

    arithmetic="fast" (hardware approximations): the p99.9 of the guarded relative error must be below `tol`.
    Where the maximum is not, the error against the FP64 oracle must be equal or better than the oracle's:
    on the worst 32 particles plus `fp64_targets` random ones, the engine's median and maximum relative error
    against the FP64 all-pairs direct sum may exceed the oracle's by at most 0.1%. The disagreement with the
    reference's other P2P order (p2pBlock, its path for N <= 65,535 at p2p.cu:169) is recorded beside it.
    Returns (max, p99.9)."""
    eff = np.asarray(eff, np.float32).reshape(-1, 2)
    if ref is None:
        ref = orc.solve(pos, w, num_level, limits, eps)
    err, errs = guarded_rel_err(eff, ref)
    p999 = float(np.quantile(errs, 0.999)) if len(errs) else 0.0
    rec = dict(case=case, arith=arithmetic, n=len(eff), max=err, p999=p999, block=None, fp64=None)
    PARITY_RECORDS.append(rec)
    if arithmetic == "exact":
        bad = np.flatnonzero(~np.all((eff == ref) | (np.isnan(eff) & np.isnan(ref)), axis=1))
        assert bad.size == 0, (f"{bad.size} effects differ from the oracle's, first at {bad[:5]}: "
                               f"{eff[bad[:3]]} vs {ref[bad[:3]]}")
        return err, p999
    if block is None and len(eff) <= 1 << 17:
        block = orc.solve(pos, w, num_level, limits, eps, block=True)
    if block is not None:
        rec["block"] = guarded_rel_err(eff, block)[0]
    assert p999 < tol, f"p99.9 guarded relative error {p999:.3e}"
    if err >= tol:
        n = len(eff)
        rng = np.random.default_rng(n)
        worst = np.argsort(errs)[-32:]
        targets = np.unique(np.concatenate([worst, rng.choice(n, min(fp64_targets, n), replace=False)]))
        rec["fp64"] = fp64_errors(eff, ref, pos, w, eps, orc, targets.astype(np.int32))
        me, mo, xe, xo = rec["fp64"]
        assert me <= mo * 1.001 + 1e-7 and xe <= xo * 1.001 + 1e-7, (
            f"max guarded error {err:.3e} above {tol:.0e}, and the error against FP64 is not equal or better: "
            f"median {me:.4e} vs oracle {mo:.4e}, max {xe:.4e} vs oracle {xo:.4e}")
    return err, p999
