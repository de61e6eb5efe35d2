"""GPU: the allocation-free cell sort, nbfmm_sort_cells_noalloc, against the allocating entry point.

nbfmm_sort_cells_noalloc is for callers that cannot allocate device memory: a plugin whose host application
owns every device buffer, or code that must not trigger cudaMalloc's device synchronisation. Its scratch is a
fixed array inside the library, shared by every call. The tests call it through the C ABI twice in a row with
different inputs and compare each result with Solver::predo's permutation and heads (integers: exact). This
file is collected last so that a run stopping at the first failure has already run every other test; it also
passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMITS = (-1.25, -1.25, 1.25, 1.25)
MAX_PARTICLES = 1 << 18


def _noalloc(lib, level, pos, perm_out, head_out):
    import torch

    lim = (ctypes.c_float * 4)(*LIMITS)
    return lib.nbfmm_sort_cells_noalloc(level, lim, pos.shape[0], pos.data_ptr(), perm_out.data_ptr(),
                                        head_out.data_ptr(), torch.cuda.current_stream().cuda_stream)


def _system(n, seed):
    rng = np.random.default_rng(seed)
    r = np.sqrt(rng.uniform(0.01, 1.0, n))
    t = rng.uniform(0, 2 * np.pi, n)
    pos = np.stack([r * np.cos(t), r * np.sin(t)], 1).astype(np.float32)
    pos[: n // 50] = pos[n // 2]  # a pile of coincident particles: one heavy cell
    return pos, rng.uniform(0.5, 1.5, n).astype(np.float32)


def _predo(engine, level, pos, w):
    import torch

    n = pos.shape[0]
    s = engine.Solver(level, n, LIMITS)
    s.predo(n, torch.from_numpy(pos).cuda(), torch.from_numpy(w).cuda())
    torch.cuda.synchronize()
    b = s.buffers()
    return b["perm"][:n].clone(), b["head"].clone()


def test_noalloc_sort_matches_predo_on_two_calls_in_a_row(engine):
    import torch

    lib = engine.load_library()
    cases = [(MAX_PARTICLES, 6, 1), (100_003, 7, 2)]  # the second call is smaller: no stale scratch may leak
    outputs = []
    for n, level, seed in cases:
        pos, w = _system(n, seed)
        cells = (1 << (level + 1)) ** 2
        perm = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        head = torch.full((cells + 1,), -1, dtype=torch.int32, device="cuda")
        rc = _noalloc(lib, level, torch.from_numpy(pos).cuda(), perm, head)
        assert rc == 0, lib.nbfmm_last_error()
        outputs.append((n, level, pos, w, perm, head))
    torch.cuda.synchronize()
    for n, level, pos, w, perm, head in outputs:
        ref_perm, ref_head = _predo(engine, level, pos, w)
        assert torch.equal(perm, ref_perm)
        assert torch.equal(head, ref_head)
        assert int(head[-1]) == n


def test_noalloc_sort_rejects_more_than_its_scratch(engine):
    import torch

    lib = engine.load_library()
    n = MAX_PARTICLES + 1
    pos = torch.zeros(n, 2, device="cuda")
    perm = torch.zeros(n, dtype=torch.int32, device="cuda")
    head = torch.zeros((1 << 14) + 1, dtype=torch.int32, device="cuda")
    assert _noalloc(lib, 6, pos, perm, head) == 1
    assert b"exceed" in lib.nbfmm_last_error()
