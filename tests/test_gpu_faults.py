"""GPU: failures made on the host, which the engine must survive with a status and without leaking: every device
allocation of each create call failing in turn (the library's injected-allocation hook), the frame raster
without its scratch, and NaN positions in a solve. Nothing here faults, traps or hangs a GPU."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NOMEM = 3
LIMITS = (ctypes.c_float * 4)(-1.0, -1.0, 1.0, 1.0)


def create(lib, kind, stars=None, path=None):
    h = ctypes.c_void_p()
    if kind == "solver":
        rc = lib.nbfmm_solver_create(4, 100_000, LIMITS, ctypes.byref(h))
    elif kind == "stars":
        rc = lib.nbfmm_stars_create(4, 100_000, 1e-3, 1.0, LIMITS, ctypes.byref(h))
    elif kind == "adjoint":
        rc = lib.nbfmm_adjoint_create(4, 50_000, LIMITS, 1e-3, 1.0, 8, 4, ctypes.byref(h))
    elif kind == "batch":
        offsets = (ctypes.c_int * 4)(0, 1000, 5000, 20_000)
        levels = (ctypes.c_int * 3)(2, 3, 4)
        limits = (ctypes.c_float * 12)(*([-1.0, -1.0, 1.0, 1.0] * 3))
        rc = lib.nbfmm_batch_create(3, offsets, levels, limits, 1e-3, 1.0, ctypes.byref(h))
    else:  # movie
        rc = lib.nbfmm_movie_open(stars, path.encode(), 320, 240, 30, 0.01, LIMITS, ctypes.byref(h))
    return rc, h


def destroy(lib, kind, h):
    {"solver": lib.nbfmm_solver_destroy, "stars": lib.nbfmm_stars_destroy, "adjoint": lib.nbfmm_adjoint_destroy,
     "batch": lib.nbfmm_batch_destroy, "movie": lib.nbfmm_movie_close}[kind](h)


@pytest.mark.parametrize("kind", ["solver", "stars", "adjoint", "batch", "movie"])
def test_every_allocation_failure_is_reported_and_released(engine, kind, tmp_path):
    import torch

    from nbfmm_gb300 import _lib

    lib = _lib.load()
    stars = None
    if kind == "movie":
        rc, stars = create(lib, "stars")
        assert rc == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    failures = 0
    for k in range(400):
        lib.nbfmm_debug_fail_allocations_after(k)
        try:
            rc, h = create(lib, kind, stars, str(tmp_path / "m.y4m"))
        finally:
            lib.nbfmm_debug_fail_allocations_after(-1)
        if rc == 0:
            destroy(lib, kind, h)
            break
        assert rc == NOMEM, lib.nbfmm_last_error().decode()
        assert not h.value
        assert b"injected" in lib.nbfmm_last_error()
        failures += 1
    assert rc == 0 and failures >= 2, (kind, failures)
    if stars is not None:
        lib.nbfmm_stars_destroy(stars)
    torch.cuda.synchronize()
    assert free0 - torch.cuda.mem_get_info()[0] < (64 << 20)  # everything a failed create took is back


def test_display_without_scratch_draws_the_same_frame(engine, orc):
    """With its bitmask scratch refused, the raster takes the byte-store kernel and draws the same frame."""
    import torch

    from nbfmm_gb300 import _lib

    rng = np.random.default_rng(3)
    n, width, height = 200_000, 640, 360
    pos = rng.uniform(-1.05, 1.05, (n, 2)).astype(np.float32)
    w = (rng.uniform(0, 9, n) * 0.01) ** 2
    p = torch.from_numpy(pos).cuda()
    m = torch.from_numpy(w.astype(np.float32)).cuda()
    frames = []
    for inject in (False, True):
        board = torch.full((engine.frame_bytes(width, height),), 7, dtype=torch.uint8, device="cuda")
        lib = _lib.load()
        lib.nbfmm_debug_fail_allocations_after(0 if inject else -1)
        try:
            engine.display(p, m, width, height, 0.01, (-1, -1, 1, 1), board, num_star=n)
        finally:
            lib.nbfmm_debug_fail_allocations_after(-1)
        torch.cuda.synchronize()
        frames.append(board.cpu().numpy())
    np.testing.assert_array_equal(frames[0], frames[1])
    np.testing.assert_array_equal(frames[0], orc.display(pos, w, width, height, 0.01, (-1, -1, 1, 1)))


def test_nan_positions_propagate_as_in_the_oracle(engine, orc):
    """NaN positions go to leaf cell 0 (the reference's index is undefined there); the NaNs then spread through
    the near and far fields exactly as in the oracle, and every finite effect keeps the parity rule."""
    import torch

    from conftest import guarded_rel_err

    rng = np.random.default_rng(9)
    n = 8192
    pos = rng.uniform(-1.0, 1.0, (n, 2)).astype(np.float32)
    w = rng.uniform(0.5, 1.5, n).astype(np.float32)
    pos[[5, 700, 4000]] = np.nan
    pos[1234, 1] = np.nan
    lim = (-1.0, -1.0, 1.0, 1.0)
    s = engine.Solver(4, n, lim, epsilon=1e-3)
    e = torch.empty(n, 2, device="cuda")
    s.solve(n, torch.from_numpy(pos).cuda(), torch.from_numpy(w).cuda(), e)
    torch.cuda.synchronize()
    eff = e.cpu().numpy()
    ref = orc.solve(pos, w, 4, lim, 1e-3)
    bad = ~np.isfinite(ref).all(1)
    np.testing.assert_array_equal(~np.isfinite(eff).all(1), bad)
    assert bad.sum() >= 4
    if (~bad).any():
        assert guarded_rel_err(eff[~bad], ref[~bad])[0] < 1e-4
