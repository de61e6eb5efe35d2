"""GPU: the batched form. Every system of a batch must evolve bit for bit as the same system alone in a Stars
(which is itself checked against the oracle), including the pruning order, the survivor counts, systems with
no far field (num_level 0), empty systems, and state carried across update calls."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_systems(seed):
    rng = np.random.default_rng(seed)
    specs = [  # (n, num_level, limits)
        (700, 3, (-1.0, -1.0, 1.0, 1.0)),
        (0, 2, (0.0, 0.0, 1.0, 1.0)),
        (3000, 4, (-2.0, -1.0, 2.0, 3.0)),
        (130, 0, (-1.0, -1.0, 1.0, 1.0)),
        (5000, 5, (-1.25, -1.25, 1.25, 1.25)),
        (257, 1, (0.0, -5.0, 10.0, 5.0)),
        (20000, 7, (-0.5, -0.5, 0.5, 0.5)),  # fine enough for the series arithmetic at eps 1e-3 (v = 0.0014)
    ]
    systems = []
    for n, level, lim in specs:
        lo = np.array(lim[:2], np.float32)
        hi = np.array(lim[2:], np.float32)
        cur = (lo + (hi - lo) * rng.uniform(0.05, 0.95, (n, 2))).astype(np.float32)
        prev = (cur - rng.normal(0, 2e-3, (n, 2)) * (hi - lo)).astype(np.float32)
        if n > 20:  # a few stars escaping at different steps
            for k, speed in enumerate([0.3, 0.1, 0.04]):
                cur[k] = [hi[0] - 0.02 * (hi[0] - lo[0]), (lo[1] + hi[1]) / 2]
                prev[k] = cur[k] - [speed * (hi[0] - lo[0]) * 0.2, 0.0]
        w = (rng.uniform(0.5, 1.5, n) / max(n, 1)).astype(np.float32)
        systems.append((cur, prev, w, level, lim))
    return systems


def run_alone(engine, cur, prev, w, level, lim, tick, eps, calls):
    import torch

    n = len(w)
    if n == 0:
        return 0, cur, prev, w
    st = engine.Stars(level, n, tick=tick, grav_const=1.0, position_limits=lim, epsilon=eps)
    st.gpuptr_position_cur_[:] = torch.from_numpy(cur).cuda()
    st.gpuptr_position_pre_[:] = torch.from_numpy(prev).cuda()
    st.gpuptr_weight_[:] = torch.from_numpy(w).cuda()
    for k in calls:
        st.update(k)
    torch.cuda.synchronize()
    return st.num_star_, st.gpuptr_position_cur_.cpu().numpy(), st.gpuptr_position_pre_.cpu().numpy(), \
        st.gpuptr_weight_.cpu().numpy()


def run_batch(engine, systems, tick, eps, calls, arithmetic="fast", item_passes=None):
    import torch

    offsets = np.cumsum([0] + [len(s[2]) for s in systems])
    b = engine.Batch(offsets, [s[3] for s in systems], [s[4] for s in systems], tick=tick, epsilon=eps,
                     arithmetic=arithmetic)
    if item_passes is not None:
        b.set_item_passes(item_passes)
    b.position_cur[:] = torch.from_numpy(np.concatenate([s[0] for s in systems])).cuda()
    b.position_pre[:] = torch.from_numpy(np.concatenate([s[1] for s in systems])).cuda()
    b.weight[:] = torch.from_numpy(np.concatenate([s[2] for s in systems])).cuda()
    for k in calls:
        b.update(k)
    torch.cuda.synchronize()
    return b, offsets


@pytest.mark.parametrize("calls,item_passes", [([1], None), ([5], None), ([2, 3], None),
                                               ([3], [2, 4, 2, 2, 4, 2, 2])])
def test_batch_equals_systems_alone(engine, calls, item_passes):
    """Each system of a batch evolves bit for bit as the same system in a Stars of its own; with P2P work items of
    2 passes for some systems (the autotuner's tile choice) as well, which must not change any result."""
    systems = make_systems(7)
    tick, eps = 2e-3, 1e-3
    b, off = run_batch(engine, systems, tick, eps, calls, item_passes=item_passes)
    cur = b.position_cur.cpu().numpy()
    pre = b.position_pre.cpu().numpy()
    w = b.weight.cpu().numpy()
    counts = b.num_stars
    for s, (c0, p0, w0, level, lim) in enumerate(systems):
        n, c, p, ww = run_alone(engine, c0, p0, w0, level, lim, tick, eps, calls)
        assert counts[s] == n, f"system {s}"
        sl = slice(off[s], off[s + 1])
        np.testing.assert_array_equal(w[sl], ww)
        np.testing.assert_array_equal(cur[sl], c)
        np.testing.assert_array_equal(pre[sl], p)
    assert sum(counts) < sum(len(s[2]) for s in systems)  # some stars were pruned


def test_exact_arithmetic_batch_equals_the_oracle(engine, orc):
    """With exact near-field arithmetic every system of a batch, stepped 3 times, equals the oracle's three
    updates of that system alone bit for bit (positions, previous positions, weights, survivor counts)."""
    systems = make_systems(9)
    tick, eps = 2e-3, 1e-3
    b, off = run_batch(engine, systems, tick, eps, [3], arithmetic="exact")
    cur, pre, w = b.position_cur.cpu().numpy(), b.position_pre.cpu().numpy(), b.weight.cpu().numpy()
    counts = b.num_stars
    for s, (c0, p0, w0, level, lim) in enumerate(systems):
        c, p, ww, n = c0.copy(), p0.copy(), w0.copy(), len(w0)
        for _ in range(3):
            if n == 0:
                break
            k, c[:n], p[:n], ww[:n], _ = orc.stars_update(c[:n], p[:n], ww[:n], level, lim, eps, np.float32(tick))
            n = k
        sl = slice(off[s], off[s + 1])
        assert counts[s] == n, f"system {s}"
        np.testing.assert_array_equal(w[sl], ww)
        np.testing.assert_array_equal(cur[sl], c)
        np.testing.assert_array_equal(pre[sl], p)


def test_item_passes_must_be_two_or_four(engine):
    systems = make_systems(8)
    b, _ = run_batch(engine, systems, 1e-3, 1e-3, [])
    with pytest.raises(engine.NbfmmError):
        b.set_item_passes([3] * len(systems))
    with pytest.raises(ValueError):
        b.set_item_passes([2])


def test_batch_launch_count_and_profile(engine):
    systems = make_systems(8)
    b, _ = run_batch(engine, systems, 1e-3, 1e-3, [])
    b.profile_begin(3)
    b.update(3)
    ms, k = b.profile_end()
    assert k == 3 and ms > 0
    assert b.kernel_launches(3) > 3


def test_batch_continuing_steps_with_far_jumps_and_a_dense_cell(engine):
    """The steps after a call's first re-sort each system from its previous cell order with the keys the P2P
    epilogue left in the system's own grid. Stars that jump several cells per step (or leave their system's limits)
    and a cell holding more stars than the gather stages in shared memory must still give, system by system, the
    same bits as the system stepped alone (whose first step sorts in full each call)."""
    rng = np.random.default_rng(31)
    systems = []
    for n, level, lim in [(4000, 4, (-1.0, -1.0, 1.0, 1.0)), (3000, 5, (0.0, 0.0, 2.0, 2.0)),
                          (2500, 3, (-3.0, -1.0, 1.0, 3.0))]:
        lo, hi = np.array(lim[:2], np.float32), np.array(lim[2:], np.float32)
        cur = (lo + (hi - lo) * rng.uniform(0.05, 0.95, (n, 2))).astype(np.float32)
        vel = rng.uniform(-2e-3, 2e-3, (n, 2)) * (hi - lo)
        fast = rng.choice(n, n // 8, replace=False)
        vel[fast] = rng.uniform(-0.15, 0.15, (len(fast), 2)) * (hi - lo)  # several leaf cells per step
        cur[:600] = lo + (hi - lo) * rng.uniform(0.50, 0.505, (600, 2))  # one dense cell
        prev = (cur - vel).astype(np.float32)
        w = (rng.uniform(0.5, 1.5, n) / n).astype(np.float32)
        systems.append((cur, prev, w, level, lim))
    tick, eps = 1e-3, 1e-3
    calls = [4, 3]
    b, off = run_batch(engine, systems, tick, eps, calls)
    cur, pre, w = b.position_cur.cpu().numpy(), b.position_pre.cpu().numpy(), b.weight.cpu().numpy()
    counts = b.num_stars
    for s, (c0, p0, w0, level, lim) in enumerate(systems):
        n, c, p, ww = run_alone(engine, c0, p0, w0, level, lim, tick, eps, calls)
        assert counts[s] == n, f"system {s}"
        sl = slice(off[s], off[s + 1])
        np.testing.assert_array_equal(w[sl], ww)
        np.testing.assert_array_equal(cur[sl], c)
        np.testing.assert_array_equal(pre[sl], p)
    assert sum(counts) < sum(len(s[2]) for s in systems)  # the fast stars left their limits on the way
