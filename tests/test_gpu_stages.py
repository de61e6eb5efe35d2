"""GPU: the reference's per-stage tests (check/core/solver/*.cu) on its own fixture, through the engine's stage
entry points (the NBFMM_CHECK-public stage methods) and its workspace buffers.

Like the reference's tests, each test writes a stage's inputs into the solver's buffers, runs the stage and
compares with the known answer (golden vectors made with the reference's arithmetic) at the reference's
tolerance of 1e-4 absolute; integer outputs must match the oracle exactly.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L, B, N = 3, 16, 250
LIMITS = (0.0, -1.0, 8.0, 2.0)


def cube(a, last=2):
    return a.reshape((L, B, B, last) if last else (L, B, B))


def cube_to_compact(cube_xy, cube_w, buf):
    """Reference strided cube (level l, cell (x,y) at [l, y<<l, x<<l]) -> engine's compact float4 cells."""
    out = np.zeros((sum(d * d for d in buf["level_dim"]), 4), np.float32)
    for l, (d, off) in enumerate(zip(buf["level_dim"], buf["level_offset"])):
        s = 1 << l
        out[off:off + d * d, 0:2] = cube_xy[l, ::s, ::s].reshape(-1, 2)
        if cube_w is not None:
            out[off:off + d * d, 2] = cube_w[l, ::s, ::s].reshape(-1)
    return out


def compact_level(arr, buf, l):
    d, off = buf["level_dim"][l], buf["level_offset"][l]
    return arr[off:off + d * d].reshape(d, d, -1)


@pytest.fixture()
def solver(engine):
    s = engine.Solver(L, N, LIMITS)
    yield s
    s.close()


def to_gpu(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def test_predo(solver, golden, orc):
    import torch

    pos = golden["position"].reshape(-1, 2)
    w = golden["weight"]
    solver.predo(N, to_gpu(pos), to_gpu(w))
    torch.cuda.synchronize()
    buf = solver.buffers()
    part = buf["particle"][:N].cpu().numpy()
    perm = buf["perm"][:N].cpu().numpy()
    key = buf["cell_key"][:N].cpu().numpy()
    head = buf["head"].cpu().numpy()
    ref = orc.predo(pos, w, L, LIMITS)
    np.testing.assert_array_equal(perm, ref["perm"])                          # bit-exact order
    np.testing.assert_array_equal(head, ref["head"])
    np.testing.assert_array_equal(key, ref["index"][:, 0] + ref["index"][:, 1] * B)
    np.testing.assert_array_equal(part[:, 0:2], pos[perm])                    # predo.cu test checks
    np.testing.assert_array_equal(part[:, 2], w[perm])
    np.testing.assert_array_equal(part[:, 3].view(np.int32), perm)


@pytest.mark.parametrize("num_level,n", [(0, 5000), (1, 4097), (4, 100000), (5, 4096 * 3 + 17), (8, 700000),
                                         (9, 1000003), (10, 2000000)])
def test_predo_record_sort_across_depths(engine, orc, num_level, n):
    """predo's record sort carries (x, y, m, index) through one (depth <= 5, keys of <= 10 bits), two (depth
    6-10, keys of 12-20 bits) or three (depth 11, 22 bits) passes of up to 10-bit digits: every sorted record, key, permutation
    entry and head equals the oracle's stable counting sort, on clustered positions (some cells empty, some
    crowded, some particles on or outside the limits)."""
    import torch

    rng = np.random.default_rng(num_level * 1000 + 7)
    lim = (-1.0, -2.0, 3.0, 1.0)
    pos = np.concatenate([rng.normal(0.2, 0.4, (n // 2, 2)), rng.uniform(-1.5, 3.5, (n - n // 2, 2))])
    pos = pos.astype(np.float32)
    pos[:7] = [[-1, -2], [3, 1], [3, -2], [-1, 1], [9, 9], [-9, -9], [np.nan, 0.5]]
    w = rng.uniform(0.5, 1.5, n).astype(np.float32)
    s = engine.Solver(num_level, n, lim)
    s.predo(n, to_gpu(pos), to_gpu(w))
    torch.cuda.synchronize()
    buf = s.buffers()
    ref = orc.predo(pos, w, num_level, lim)
    b = 1 << (num_level + 1)
    perm = buf["perm"][:n].cpu().numpy()
    np.testing.assert_array_equal(perm, ref["perm"])
    np.testing.assert_array_equal(buf["head"].cpu().numpy(), ref["head"])
    np.testing.assert_array_equal(buf["cell_key"][:n].cpu().numpy(), ref["index"][:, 0] + ref["index"][:, 1] * b)
    part = buf["particle"][:n].cpu().numpy()
    np.testing.assert_array_equal(part[:, 0:2].view(np.int32), pos[perm].view(np.int32))  # NaN bits too
    np.testing.assert_array_equal(part[:, 2], w[perm])
    np.testing.assert_array_equal(part[:, 3].view(np.int32), perm)


def test_postdo(solver, golden):
    import torch

    buf = solver.buffers()
    buf["effect"][:N] = to_gpu(golden["position"].reshape(-1, 2))
    buf["perm"][:N] = torch.from_numpy(golden["perm"].astype(np.int32)).cuda()
    out = torch.zeros(N, 2, device="cuda")
    solver.postdo(N, out)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), golden["postdo_effect_origin"].reshape(-1, 2))


def _load_particles(solver, golden):
    import torch

    buf = solver.buffers()
    p = np.zeros((N, 4), np.float32)
    p[:, 0:2] = golden["position"].reshape(-1, 2)
    p[:, 2] = golden["weight"]
    buf["particle"][:N] = to_gpu(p)
    buf["head"][:] = torch.from_numpy(golden["head"].astype(np.int32)).cuda()
    return buf


def test_p2p(solver, golden):
    import torch

    buf = _load_particles(solver, golden)
    solver.p2p(N)
    torch.cuda.synchronize()
    eff = buf["effect"][:N].cpu().numpy()
    np.testing.assert_allclose(eff, golden["p2p_effect"].reshape(-1, 2), rtol=0, atol=1e-4)


def test_p2p_matches_oracle_order(solver, golden, orc):
    """Beyond the reference's 1e-4: the engine sums in p2pNaive order, so it tracks the oracle closely."""
    import torch

    buf = _load_particles(solver, golden)
    solver.p2p(N)
    torch.cuda.synchronize()
    eff = buf["effect"][:N].cpu().numpy()
    ref = orc.p2p(golden["position"].reshape(-1, 2), golden["weight"], golden["index"].reshape(-1, 2),
                  golden["head"], B, 0.1)
    from conftest import guarded_rel_err

    assert guarded_rel_err(eff, ref)[0] < 1e-5


def test_p2m(solver, golden):
    import torch

    buf = _load_particles(solver, golden)
    solver.p2m(N)
    torch.cuda.synchronize()
    c0 = compact_level(buf["cell"].cpu().numpy(), buf, 0).reshape(-1, 4)
    np.testing.assert_allclose(c0[:, 0:2], golden["p2m_cell_position"].reshape(-1, 2), rtol=0, atol=1e-4)
    np.testing.assert_allclose(c0[:, 2], golden["p2m_cell_weight"], rtol=0, atol=1e-4)


def test_m2m(solver, golden):
    import torch

    buf = solver.buffers()
    cells = cube_to_compact(cube(golden["cell_position"]), cube(golden["cell_weight"], 0), buf)
    cells[buf["level_dim"][0] ** 2:] = 0.0  # only level 0 is input (check/core/solver/m2m.cu:14-22)
    buf["cell"][:] = to_gpu(cells)
    solver.m2m()
    torch.cuda.synchronize()
    got = buf["cell"].cpu().numpy()
    ref = cube_to_compact(cube(golden["m2m_cell_position"]), cube(golden["m2m_cell_weight"], 0), buf)
    np.testing.assert_allclose(got[:, 0:3], ref[:, 0:3], rtol=0, atol=1e-4)


def test_m2l(solver, golden):
    import torch

    buf = solver.buffers()
    buf["cell"][:] = to_gpu(cube_to_compact(cube(golden["cell_position"]), cube(golden["cell_weight"], 0), buf))
    solver.m2l()
    torch.cuda.synchronize()
    got = buf["cell_effect"].cpu().numpy()
    ref = cube_to_compact(cube(golden["m2l_cell_effect"]), None, buf)[:, 0:2]
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-4)


def test_l2l(solver, golden):
    import torch

    buf = solver.buffers()
    ce = cube_to_compact(cube(golden["cell_position"]), None, buf)[:, 0:2]
    buf["cell_effect"][:] = to_gpu(ce)
    solver.l2l()
    torch.cuda.synchronize()
    got = compact_level(buf["cell_effect"].cpu().numpy(), buf, 0)
    np.testing.assert_allclose(got, golden["l2l_cell_effect0"].reshape(B, B, 2), rtol=0, atol=1e-4)


def test_l2p(solver, golden):
    import torch

    buf = solver.buffers()
    idx = golden["index"].reshape(-1, 2)
    buf["effect"][:N] = to_gpu(golden["position"].reshape(-1, 2))
    buf["cell_key"][:N] = torch.from_numpy((idx[:, 0] + idx[:, 1] * B).astype(np.int32)).cuda()
    ce = cube_to_compact(cube(golden["cell_position"]), None, buf)[:, 0:2]
    buf["cell_effect"][:] = to_gpu(ce)
    solver.l2p(N)
    torch.cuda.synchronize()
    np.testing.assert_allclose(buf["effect"][:N].cpu().numpy(), golden["l2p_effect"].reshape(-1, 2), rtol=0,
                               atol=1e-6)


def test_cell_stages_match_oracle_bit_exact(solver, golden, orc):
    """M2M and M2L round like the reference compiled for a CPU: the engine and the oracle agree exactly."""
    import torch

    buf = solver.buffers()
    cp, cw = cube(golden["cell_position"]).copy(), cube(golden["cell_weight"], 0).copy()
    cells = cube_to_compact(cp, cw, buf)
    buf["cell"][:] = to_gpu(cells)
    solver.m2m()
    solver.m2l()
    torch.cuda.synchronize()
    rp, rw = orc.m2m(cp.reshape(-1), cw.reshape(-1), L, B)
    ref_cells = cube_to_compact(cube(rp), cube(rw, 0), buf)
    np.testing.assert_array_equal(buf["cell"].cpu().numpy()[:, 0:3], ref_cells[:, 0:3])
    re = orc.m2l(rp, rw, L, B, 0.1)
    np.testing.assert_array_equal(buf["cell_effect"].cpu().numpy(), cube_to_compact(cube(re), None, buf)[:, 0:2])


def test_p2m_bit_exact_with_sequential_sums(solver, golden, orc):
    """Leaf sums are accumulated one particle at a time in sorted order, like check/core/solver/p2m.cu:36-46."""
    import torch

    buf = _load_particles(solver, golden)
    solver.p2m(N)
    torch.cuda.synchronize()
    c0 = compact_level(buf["cell"].cpu().numpy(), buf, 0).reshape(-1, 4)
    cp, cw = orc.p2m(golden["position"].reshape(-1, 2), golden["weight"], golden["head"], B)
    np.testing.assert_array_equal(c0[:, 0:2], cp)
    np.testing.assert_array_equal(c0[:, 2], cw)
