"""GPU: Solver::solve parity with the oracle (the reference's algorithm restated on the CPU).

Bar: cell order (keys, permutation, heads) bit-exact; the far field (every cell centre of mass, mass and local
effect) bit-exact; effects under the guarded relative metric max_i |a_i - a_i^ref| / max(|a_i^ref|,
1e-3 * median |a^ref|) against the oracle, which sums P2P in the reference's p2pNaive order in IEEE single
precision. With exact near-field arithmetic (correctly rounded sqrt and division, no contraction) every effect
equals the oracle's bit for bit; with the default fast arithmetic (hardware approximations, same order) the rule
of conftest.assert_solve_parity applies: p99.9 below 1e-5, and where the maximum is not, an error against the
FP64 direct sum equal to the oracle's. The per-case figures are printed in the pytest summary.
"""
import numpy as np
import pytest

from conftest import assert_solve_parity, guarded_rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-5


ARITHMETICS = ("fast", "exact")


def run_solve(engine, pos, w, num_level, limits, eps, max_n=None, arithmetic="fast"):
    import torch

    n = len(w)
    s = engine.Solver(num_level, max_n or max(n, 1), limits, epsilon=eps, arithmetic=arithmetic)
    p = torch.from_numpy(np.ascontiguousarray(pos, np.float32)).cuda()
    m = torch.from_numpy(np.ascontiguousarray(w, np.float32)).cuda()
    e = torch.full((max(n, 1), 2), float("nan"), device="cuda")
    s.solve(n, p, m, e)
    torch.cuda.synchronize()
    out = e[:n].cpu().numpy()
    return s, out


def uniform(n, seed, lo=-1.0, hi=1.0):
    rng = np.random.default_rng(seed)
    return rng.uniform(lo, hi, (n, 2)).astype(np.float32), rng.uniform(0.5, 1.5, n).astype(np.float32)


def test_reference_fixture_solve(engine, golden, orc):
    pos, w = golden["position"].reshape(-1, 2), golden["weight"]
    lim = (0.0, -1.0, 8.0, 2.0)
    s, eff = run_solve(engine, pos, w, 3, lim, 0.1)
    assert guarded_rel_err(eff, orc.solve(pos, w, 3, lim, 0.1))[0] < TOL
    # the reference's own path at this size is p2pBlock (N <= 65535); its order differs by rounding only
    assert guarded_rel_err(eff, orc.solve(pos, w, 3, lim, 0.1, block=True))[0] < 1e-4


@pytest.mark.parametrize("arithmetic", ARITHMETICS)
@pytest.mark.parametrize("n,level", [(1, 2), (2, 2), (31, 1), (1000, 0), (4095, 3), (4096, 3), (4097, 3),
                                     (12345, 4), (16384, 3), (65536, 5)])
def test_uniform_sizes(engine, orc, n, level, arithmetic):
    pos, w = uniform(n, 100 + n)
    lim = (-1.0, -1.0, 1.0, 1.0)
    s, eff = run_solve(engine, pos, w, level, lim, 1e-3, arithmetic=arithmetic)
    assert_solve_parity(eff, pos, w, level, lim, 1e-3, orc, arithmetic=arithmetic,
                        case=f"uniform n={n} L={level}")


@pytest.mark.parametrize("arithmetic", ARITHMETICS)
@pytest.mark.parametrize("scale,eps,level", [
    (1.0, 1e-3, 4),
    (200.0, 5.0, 4),    # a strongly cancelling far field
    (600.0, 50.0, 4),   # large coordinates
    (1.0, 1e-12, 3),    # tiny softening: r^3 + eps spans many binades
    (1.0, 5e9, 3),      # softening far above r^3
])
def test_scaled_fields_and_extreme_softening(engine, orc, scale, eps, level, arithmetic):
    """The near field's reciprocal arithmetic (hardware approximation and the FMA-pipe iteration) over coordinate
    scales and softenings far from the benchmark's, against the oracle."""
    rng = np.random.default_rng(int(scale * 7 + level))
    n = 20000
    r = np.sqrt(rng.uniform(0, 1, n))
    a = rng.uniform(0, 2 * np.pi, n)
    pos = (scale * np.stack([r * np.cos(a), r * np.sin(a)], 1)).astype(np.float32)
    w = rng.uniform(0.5, 1.5, n).astype(np.float32)
    lim = (-1.01 * scale, -1.01 * scale, 1.01 * scale, 1.01 * scale)
    s, eff = run_solve(engine, pos, w, level, lim, eps, arithmetic=arithmetic)
    assert np.all(np.isfinite(eff))
    assert_solve_parity(eff, pos, w, level, lim, eps, orc, arithmetic=arithmetic,
                        case=f"disk x{scale:g} eps={eps:g} L={level}")


def test_disk_against_oracle_and_fp64(engine, orc):
    from nbfmm_gb300 import workloads

    sysm = workloads.disk(1 << 18, seed=5, num_level=5)
    s, eff = run_solve(engine, sysm.position, sysm.weight, sysm.num_level, sysm.limits, sysm.epsilon)
    ref = orc.solve(sysm.position, sysm.weight, sysm.num_level, sysm.limits, sysm.epsilon)
    err, errs = guarded_rel_err(eff, ref)
    print(f"disk 262144: guarded max {err:.3e}, p99.9 {np.quantile(errs, 0.999):.3e}")
    assert err < TOL
    t = np.random.default_rng(0).choice(len(sysm.weight), 512, replace=False)
    d = orc.direct_f64(sysm.position, sysm.weight, sysm.epsilon, t)
    e_gpu = np.linalg.norm(eff[t] - d, axis=1) / np.linalg.norm(d, axis=1)
    e_orc = np.linalg.norm(ref[t] - d, axis=1) / np.linalg.norm(d, axis=1)
    print(f"vs FP64 direct sum: engine median {np.median(e_gpu):.3e}, oracle median {np.median(e_orc):.3e}")
    assert np.median(e_gpu) <= np.median(e_orc) * 1.001 + 1e-7


def series_degree(limits, num_level, eps):
    """The host rule of the fast arithmetic's reciprocal series (p2p.cu series_degree)."""
    cell = max(limits[2] - limits[0], limits[3] - limits[1]) / 2 ** (num_level + 1)
    return 2 if (2 * np.sqrt(2) * cell) ** 3 / eps <= 0.0062 else 0


@pytest.mark.parametrize("case", ["uniform", "clustered_with_outliers"])
def test_series_arithmetic_meets_the_fast_rule(engine, orc, case):
    """Where leaf cells are small against eps (r^3 << eps for every near pair), the fast arithmetic replaces
    1 / (r^3 + eps) by a series of degree 2 for part of the sources in the work items away from the grid's
    edges; the edge items, which hold the stars beyond the limits, keep the
    general path. Both must meet the fast-arithmetic rule."""
    rng = np.random.default_rng(21)
    n, level, eps = 120_000, 6, 2e-2
    lim = (-1.0, -1.0, 1.0, 1.0)
    assert series_degree(lim, level, eps) == 2
    if case == "uniform":
        pos = rng.uniform(-1, 1, (n, 2))
    else:
        pos = np.concatenate([rng.normal(0, 0.2, (n - 200, 2)), rng.uniform(-40, 40, (200, 2))])
    pos = pos.astype(np.float32)
    w = (rng.uniform(0.5, 1.5, n) / n).astype(np.float32)
    s, eff = run_solve(engine, pos, w, level, lim, eps)
    assert_solve_parity(eff, pos, w, level, lim, eps, orc, case=f"series {case}")


def test_zero_particles_is_a_no_op(engine):
    import torch

    s = engine.Solver(3, 16, (-1, -1, 1, 1))
    e = torch.full((16, 2), 7.0, device="cuda")
    s.solve(0, e, e[:, 0].contiguous(), e)
    torch.cuda.synchronize()
    assert torch.all(e == 7.0)


@pytest.mark.parametrize("arithmetic", ARITHMETICS)
def test_one_dense_cell_spans_many_chunks(engine, orc, arithmetic):
    # 1500 particles in one leaf cell (several 256-target chunks) plus a sparse background
    rng = np.random.default_rng(21)
    dense = rng.uniform(0.01, 0.11, (1500, 2)).astype(np.float32)
    sparse = rng.uniform(-1, 1, (500, 2)).astype(np.float32)
    pos = np.concatenate([dense, sparse])
    w = rng.uniform(0.5, 1.5, 2000).astype(np.float32)
    lim = (-1.0, -1.0, 1.0, 1.0)
    s, eff = run_solve(engine, pos, w, 3, lim, 1e-3, arithmetic=arithmetic)
    assert_solve_parity(eff, pos, w, 3, lim, 1e-3, orc, arithmetic=arithmetic, case="one dense cell")


@pytest.mark.parametrize("arithmetic", ARITHMETICS)
def test_boundary_outside_and_coincident_particles(engine, orc, arithmetic):
    rng = np.random.default_rng(22)
    pos, w = uniform(3000, 22)
    pos[:10] = [1.0, 1.0]           # on the upper limits: clamped into the last cell
    pos[10:20, 0] = -1.0            # on the lower x limit
    pos[20:25] = [[5.0, 0.0], [-3.0, 0.5], [0.0, 9.0], [0.2, -7.0], [2.0, 2.0]]  # outside: clamped
    pos[25:40] = pos[40]            # coincident particles contribute zero to each other
    lim = (-1.0, -1.0, 1.0, 1.0)
    s, eff = run_solve(engine, pos, w, 4, lim, 1e-3, arithmetic=arithmetic)
    assert np.all(np.isfinite(eff))
    assert_solve_parity(eff, pos, w, 4, lim, 1e-3, orc, arithmetic=arithmetic, case="boundary/outside/coincident")


def test_solve_smaller_than_capacity_and_repeat(engine, orc):
    import torch

    pos, w = uniform(5000, 23)
    lim = (-1.0, -1.0, 1.0, 1.0)
    s = engine.Solver(4, 20000, lim, epsilon=1e-3)
    p, m = torch.from_numpy(pos).cuda(), torch.from_numpy(w).cuda()
    e1 = torch.zeros(5000, 2, device="cuda")
    e2 = torch.zeros(5000, 2, device="cuda")
    s.solve(5000, p, m, e1)
    s.solve(5000, p, m, e2)
    torch.cuda.synchronize()
    assert torch.equal(e1, e2)  # deterministic
    assert_solve_parity(e1.cpu().numpy(), pos, w, 4, lim, 1e-3, orc, case="smaller than capacity")


def test_invalid_count_raises(engine):
    import torch

    s = engine.Solver(3, 100, (-1, -1, 1, 1))
    e = torch.zeros(200, 2, device="cuda")
    with pytest.raises(engine.NbfmmError):
        s.solve(101, e, e[:, 0].contiguous(), e)


def check_cell_order(buf, pos, w, num_level, limits, orc):
    """Keys, permutation and heads of the engine's sort equal the oracle's predo (a stable counting sort on the
    row-major key of floorf((x - x_min) / cell), predo.cu:37-38 and 105-135), bit for bit."""
    n = len(w)
    r = orc.predo(pos, w, num_level, limits)
    B = 1 << (num_level + 1)
    key_ref = r["index"][:, 0] + r["index"][:, 1] * B
    np.testing.assert_array_equal(buf["cell_key"][:n].cpu().numpy(), key_ref)
    np.testing.assert_array_equal(buf["perm"][:n].cpu().numpy(), r["perm"])
    np.testing.assert_array_equal(buf["head"].cpu().numpy(), r["head"])
    return r


@pytest.fixture(scope="module")
def headline(orc):
    """The three headline workloads with the oracle's cell order and effects, computed once per module:
    plain 16,384 (depth 4), one disk of 1,048,576 (depth 7), two disks of 16,777,216 (depth 9)."""
    from nbfmm_gb300 import workloads

    cache = {}

    def get(name):
        if name not in cache:
            sysm = workloads.CONFIGS[name]()
            ref = orc.solve(sysm.position, sysm.weight, sysm.num_level, sysm.limits, sysm.epsilon)
            cache[name] = (sysm, ref)
        return cache[name]

    return get


@pytest.mark.parametrize("arithmetic", ARITHMETICS)
@pytest.mark.parametrize("name", ["plain_16k", "disk_1m", "two_disks_16m"])
def test_headline_configs_order_and_effects(engine, orc, headline, name, arithmetic):
    """Each headline workload at full size: the engine's cell order equals the oracle's predo bit for bit, and
    every particle's effect is checked against the oracle's full solve (bit for bit with exact arithmetic). The
    error against the FP64 direct sum is recorded on 256 sampled targets beside the oracle's."""
    sysm, ref = headline(name)
    s, eff = run_solve(engine, sysm.position, sysm.weight, sysm.num_level, sysm.limits, sysm.epsilon,
                       arithmetic=arithmetic)
    assert np.all(np.isfinite(eff))
    check_cell_order(s.buffers(), sysm.position, sysm.weight, sysm.num_level, sysm.limits, orc)
    err, p999 = assert_solve_parity(eff, sysm.position, sysm.weight, sysm.num_level, sysm.limits, sysm.epsilon,
                                    orc, arithmetic=arithmetic, case=f"{name} (full size)", ref=ref)
    from conftest import PARITY_RECORDS, fp64_errors

    if PARITY_RECORDS[-1]["fp64"] is None:
        t = np.random.default_rng(7).choice(sysm.n, 256, replace=False).astype(np.int32)
        PARITY_RECORDS[-1]["fp64"] = fp64_errors(eff, ref, sysm.position, sysm.weight, sysm.epsilon, orc, t)
    me, mo, xe, xo = PARITY_RECORDS[-1]["fp64"]
    assert me <= mo * 1.001 + 1e-7 and xe <= xo * 1.001 + 1e-7


def test_far_field_of_a_solve_is_bit_exact(engine, orc):
    """Leaf sums in sorted order, M2M, M2L and L2L round exactly like the oracle: every cell centre of mass,
    mass and local effect of a full solve equals the oracle's bit for bit."""
    import torch

    from test_gpu_stages import cube_to_compact

    pos, w = uniform(20000, 31)
    level, lim = 5, (-1.0, -1.0, 1.0, 1.0)
    s, _ = run_solve(engine, pos, w, level, lim, 1e-3)
    buf = s.buffers()
    B = 1 << (level + 1)
    r = orc.predo(pos, w, level, lim)
    cp = np.zeros((level, B, B, 2), np.float32)
    cw = np.zeros((level, B, B), np.float32)
    p0, w0 = orc.p2m(r["position"], r["weight"], r["head"], B)
    cp[0], cw[0] = p0.reshape(B, B, 2), w0.reshape(B, B)
    cp, cw = orc.m2m(cp.reshape(-1), cw.reshape(-1), level, B)
    ce = orc.l2l(orc.m2l(cp, cw, level, B, 1e-3), level, B)
    cp, cw, ce = cp.reshape(level, B, B, 2), cw.reshape(level, B, B), ce.reshape(level, B, B, 2)
    ref_cells = cube_to_compact(cp, cw, buf)
    np.testing.assert_array_equal(buf["cell"].cpu().numpy()[:, 0:3], ref_cells[:, 0:3])
    np.testing.assert_array_equal(buf["cell_effect"].cpu().numpy(), cube_to_compact(ce, None, buf)[:, 0:2])


def test_maximum_size_solve(engine, orc):
    """The largest solve the API accepts: 2^28 particles at depth 10 (2048 x 2048 leaf cells, ~64 per cell). The
    cell order is checked over all particles (sorted keys, heads ending at N), and sampled targets against the
    oracle's full-tree solve."""
    import torch

    from conftest import guarded_rel_err

    n, level = 1 << 28, 10
    rng = np.random.default_rng(28)
    pos = rng.random((n, 2), dtype=np.float32)
    pos *= np.float32(2.0)
    pos -= np.float32(1.0)
    w = rng.random(n, dtype=np.float32)
    w += np.float32(0.5)
    lim = (-1.0, -1.0, 1.0, 1.0)
    s = engine.Solver(level, n, lim, epsilon=1e-3)
    e = torch.empty(n, 2, device="cuda")
    s.solve(n, torch.from_numpy(pos).cuda(), torch.from_numpy(w).cuda(), e)
    torch.cuda.synchronize()
    b = s.buffers()
    keys = b["cell_key"][:n]
    assert bool((keys[1:] >= keys[:-1]).all())
    head = b["head"]
    assert int(head[0]) == 0 and int(head[-1]) == n and bool((head[1:] >= head[:-1]).all())
    targets = np.sort(rng.choice(n, 256, replace=False)).astype(np.int32)
    got = e[torch.from_numpy(targets).long().cuda()].cpu().numpy()
    assert np.all(np.isfinite(got))
    ref = orc.solve_targets(pos, w, level, lim, 1e-3, targets)
    assert guarded_rel_err(got, ref)[0] < TOL
