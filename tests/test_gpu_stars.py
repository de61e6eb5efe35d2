"""GPU: the Stars update path (solve + Stormer-Verlet + prune, update.cu:47-55) against the oracle stepping the
reference's update one call at a time, including the order the reference's prune leaves the arrays in."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_stars(engine, cur, prev, w, level, limits, tick, eps, arithmetic="fast"):
    import torch

    st = engine.Stars(level, len(w), tick=tick, grav_const=1.0, position_limits=limits, epsilon=eps,
                      arithmetic=arithmetic)
    st.gpuptr_position_cur_[:] = torch.from_numpy(cur).cuda()
    st.gpuptr_position_pre_[:] = torch.from_numpy(prev).cuda()
    st.gpuptr_weight_[:] = torch.from_numpy(w).cuda()
    return st


def oracle_steps(orc, cur, prev, w, level, limits, tick, eps, steps):
    n = len(w)
    cur, prev, w = cur.copy(), prev.copy(), w.copy()
    for _ in range(steps):
        k, c2, p2, w2, _ = orc.stars_update(cur[:n], prev[:n], w[:n], level, limits, eps, tick)
        cur[:n], prev[:n], w[:n] = c2, p2, w2
        n = k
    return n, cur, prev, w


def system(n, seed, escape=()):
    rng = np.random.default_rng(seed)
    cur = rng.uniform(-0.9, 0.9, (n, 2)).astype(np.float32)
    prev = (cur - rng.normal(0, 2e-4, (n, 2))).astype(np.float32)
    w = (rng.uniform(0.5, 1.5, n) / n).astype(np.float32)
    w += np.arange(n, dtype=np.float32) * np.float32(1e-9)  # distinct weights identify stars
    for i, (idx, speed) in enumerate(escape):
        cur[idx] = [0.85, 0.0]
        prev[idx] = [0.85 - speed, 0.0]
    return cur, prev, w


def close_positions(a, b, tick, scale=1.0):
    # differences come from effect rounding (1e-5 relative) times tick^2, plus a couple of ulps
    tol = 4 * np.spacing(np.abs(b).astype(np.float32)) + 1e-5 * scale * tick * tick
    return np.all(np.abs(a - b) <= tol)


def test_one_update_matches_oracle(engine, orc):
    import torch

    cur, prev, w = system(4096, 1)
    lim, tick, eps = (-1.0, -1.0, 1.0, 1.0), 1e-3, 1e-3
    st = make_stars(engine, cur, prev, w, 3, lim, tick, eps)
    st.update(1)
    torch.cuda.synchronize()
    n, c_ref, p_ref, w_ref = oracle_steps(orc, cur, prev, w, 3, lim, tick, eps, 1)
    assert st.num_star_ == n
    c = st.gpuptr_position_cur_.cpu().numpy()
    np.testing.assert_array_equal(st.gpuptr_weight_.cpu().numpy(), w_ref)
    np.testing.assert_array_equal(st.gpuptr_position_pre_.cpu().numpy(), p_ref)
    acc_scale = np.abs(orc.solve(cur, w, 3, lim, eps)).max()
    assert close_positions(c, c_ref, tick, acc_scale)


def test_prune_order_over_several_updates(engine, orc):
    import torch

    # stars escaping after different numbers of steps; the arrays must end in the reference's order:
    # survivors in order, then the pruned ones, most recently pruned first
    escape = [(5, 0.2), (17, 0.2), (300, 0.07), (301, 0.02), (1000, 0.07), (2047, 0.2)]
    cur, prev, w = system(2048, 2, escape)
    lim, tick, eps = (-1.0, -1.0, 1.0, 1.0), 1e-3, 1e-3
    st = make_stars(engine, cur, prev, w, 3, lim, tick, eps)
    st.update(6)
    torch.cuda.synchronize()
    n, c_ref, p_ref, w_ref = oracle_steps(orc, cur, prev, w, 3, lim, tick, eps, 6)
    assert n < 2048 - 3
    assert st.num_star_ == n
    np.testing.assert_array_equal(st.gpuptr_weight_.cpu().numpy(), w_ref)  # identical layout


@pytest.mark.parametrize("n,level,steps", [(2048, 3, 8), (60000, 5, 4)])
def test_exact_arithmetic_updates_equal_the_oracle_bit_for_bit(engine, orc, n, level, steps):
    """With exact near-field arithmetic, several updates (solve, Verlet, prune, stars escaping on the way) leave
    the positions, previous positions, weights and star count exactly as the oracle's updates do."""
    import torch

    escape = [(5, 0.2), (17, 0.2), (300, 0.07), (1000, 0.07), (n - 1, 0.2)]
    cur, prev, w = system(n, 40 + level, escape)
    lim, tick, eps = (-1.0, -1.0, 1.0, 1.0), 1e-3, 1e-3
    st = make_stars(engine, cur, prev, w, level, lim, tick, eps, arithmetic="exact")
    st.update(steps)
    torch.cuda.synchronize()
    k, c_ref, p_ref, w_ref = oracle_steps(orc, cur, prev, w, level, lim, tick, eps, steps)
    assert k < n and st.num_star_ == k
    np.testing.assert_array_equal(st.gpuptr_weight_.cpu().numpy(), w_ref)
    np.testing.assert_array_equal(st.gpuptr_position_pre_.cpu().numpy(), p_ref)
    np.testing.assert_array_equal(st.gpuptr_position_cur_.cpu().numpy(), c_ref)


def test_split_calls_equal_one_call(engine):
    import torch

    escape = [(5, 0.2), (300, 0.07), (1000, 0.02)]
    cur, prev, w = system(2048, 3, escape)
    lim, tick, eps = (-1.0, -1.0, 1.0, 1.0), 1e-3, 1e-3
    a = make_stars(engine, cur, prev, w, 3, lim, tick, eps)
    b = make_stars(engine, cur, prev, w, 3, lim, tick, eps)
    a.update(7)
    b.update(3)
    b.update(4)
    torch.cuda.synchronize()
    assert a.num_star_ == b.num_star_
    assert torch.equal(a.gpuptr_weight_, b.gpuptr_weight_)
    assert torch.equal(a.gpuptr_position_cur_, b.gpuptr_position_cur_)
    assert torch.equal(a.gpuptr_position_pre_, b.gpuptr_position_pre_)


def test_initialize_forwards_tick_and_state(engine):
    import torch

    seen = {}

    def generator(n, radius, tick, cur, prev, w):
        seen["tick"] = tick
        ang = torch.linspace(0, 6.28, n, device="cuda")
        cur[:, 0] = radius * torch.cos(ang)
        cur[:, 1] = radius * torch.sin(ang)
        prev.copy_(cur)
        w.fill_(1.0 / n)

    st = engine.Stars(3, 256, tick=2e-3, grav_const=4.0, position_limits=(-1, -1, 1, 1))
    st.initialize(generator, 256, 0.5)
    assert abs(seen["tick"] - 4e-3) < 1e-9  # tick * sqrt(G) (stars.cu:31)
    st.update(2)
    torch.cuda.synchronize()
    assert st.num_star_ == 256
    assert torch.all(torch.isfinite(st.gpuptr_position_cur_))


def arrays(st):
    n = st.num_star_
    return (st.gpuptr_position_cur_[:n].cpu().numpy(), st.gpuptr_position_pre_[:n].cpu().numpy(),
            st.gpuptr_weight_[:n].cpu().numpy())


def assert_same_stars(a, b):
    assert a.num_star_ == b.num_star_
    for x, y in zip(arrays(a), arrays(b)):
        np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32))


@pytest.mark.parametrize("level", [3, 5])
def test_grouping_of_steps_into_calls_does_not_matter(engine, level):
    """Stars crossing leaf cells at every step: K steps in one call equal K calls of one step, bit for bit, and
    equal K fresh handles of one step each. A call continues from the state the last call left when the arrays
    are unchanged; a fresh handle starts from the caller's order. Both agree only if every step orders each
    leaf cell by index, as the reference's predo does (a stable sort of the caller's arrays), whatever cells
    the stars came from."""
    import torch

    rng = np.random.default_rng(level)
    n = 6000
    cur = rng.uniform(-0.8, 0.8, (n, 2)).astype(np.float32)
    prev = (cur - rng.uniform(-6e-3, 6e-3, (n, 2))).astype(np.float32)  # ~20-40% of the stars change cells each step
    w = (rng.uniform(0.5, 1.5, n) / n).astype(np.float32)
    lim, tick, eps = (-1.0, -1.0, 1.0, 1.0), 1.0, 1e-3
    a = make_stars(engine, cur, prev, w, level, lim, tick, eps)
    b = make_stars(engine, cur, prev, w, level, lim, tick, eps)
    a.update(8)
    for _ in range(8):
        b.update(1)
    c = make_stars(engine, cur, prev, w, level, lim, tick, eps)
    for _ in range(8):
        c.update(1)
        c = make_stars(engine, *arrays(c), level, lim, tick, eps)
    torch.cuda.synchronize()
    assert a.num_star_ == b.num_star_
    assert torch.equal(a.gpuptr_position_cur_, b.gpuptr_position_cur_)
    assert torch.equal(a.gpuptr_position_pre_, b.gpuptr_position_pre_)
    assert torch.equal(a.gpuptr_weight_, b.gpuptr_weight_)
    assert_same_stars(a, c)


@pytest.mark.parametrize("case", ["far", "dense", "escapes", "series"])
def test_continuing_steps_equal_full_sorts(engine, case):
    """The steps after a call's first re-sort from the previous step's cell order (stayers, immigrants counted
    per cell); a call's first step sorts in full. K steps in one call must equal K fresh handles of one step each,
    bit for bit, when stars jump several cells per step ("far"), when one cell holds far more stars than the
    gather stages in shared memory ("dense"), and when stars leave the limits on several steps of the call."""
    import torch

    rng = np.random.default_rng({"far": 11, "dense": 12, "escapes": 13, "series": 15}[case])
    n, level, steps = 8000, 5, 6
    eps = 1e-3
    if case == "series":  # leaf cells small enough for the fast arithmetic's reciprocal series
        n, level, eps = 30000, 6, 2e-2
    cur = rng.uniform(-0.8, 0.8, (n, 2)).astype(np.float32)
    vel = rng.uniform(-2e-3, 2e-3, (n, 2))
    if case == "far":
        fast = rng.choice(n, n // 10, replace=False)
        vel[fast] = rng.uniform(-0.12, 0.12, (len(fast), 2))  # up to ~4 leaf cells (0.031) per step
    if case == "dense":
        cur[:1500] = rng.uniform(0.19, 0.215, (1500, 2))  # one leaf cell, (0.1875, 0.21875) on both axes
    if case == "escapes":
        edge = rng.choice(n, 300, replace=False)
        cur[edge, 0] = rng.uniform(0.9, 0.99, len(edge))
        vel[edge, 0] = rng.uniform(0.01, 0.06, len(edge))  # out after 1 to 9 steps
    prev = (cur - vel).astype(np.float32)
    w = (rng.uniform(0.5, 1.5, n) / n).astype(np.float32)
    lim, tick = (-1.0, -1.0, 1.0, 1.0), 1e-3  # the stars move by their velocities, not by the kick
    a = make_stars(engine, cur, prev, w, level, lim, tick, eps)
    a.update(steps)
    c = make_stars(engine, cur, prev, w, level, lim, tick, eps)
    for _ in range(steps):
        c.update(1)
        c = make_stars(engine, *arrays(c), level, lim, tick, eps)
    torch.cuda.synchronize()
    if case == "escapes":
        assert n - 300 < a.num_star_ < n
    assert_same_stars(a, c)


@pytest.mark.parametrize("case", ["edit", "loss", "prune", "edit_then_prune"])
def test_a_call_resumes_only_from_its_own_export(engine, case):
    """After an update call the engine keeps its state in cell order and continues from it when the public arrays
    are bit for bit what the call exported and no star was lost. An edited star, a lost star (the last index,
    whose loss leaves every other entry in place) and a prune in between must each give exactly the result of a
    fresh handle on the same arrays."""
    import torch

    escape = [(2047, 0.2)] if case == "loss" else []
    cur, prev, w = system(2048, 4, escape)
    lim, tick, eps = (-1.0, -1.0, 1.0, 1.0), 1e-3, 1e-3
    prev = (cur - (cur - prev) * 20).astype(np.float32)  # stars change cells between calls
    if escape:
        prev[2047] = [0.85 - 0.2, 0.0]
    a = make_stars(engine, cur, prev, w, 3, lim, tick, eps)
    a.update(3)
    if case == "loss":
        assert a.num_star_ == 2047
    if case.startswith("edit"):
        a.gpuptr_position_cur_[17, 0] += 1e-3
    if case.endswith("prune"):
        a.prune()
        assert a.num_star_ == 2048
    b = make_stars(engine, *arrays(a), 3, lim, tick, eps)
    a.update(2)
    b.update(2)
    torch.cuda.synchronize()
    assert_same_stars(a, b)


def test_every_star_lost_and_an_empty_handle(engine, orc):
    """Every star leaves the limits (at different steps); the arrays hold them in the reference's order, and
    further calls on the now empty system (which cannot resume: the last call lost stars) step nothing. A handle
    created with no stars updates, prunes and draws without error."""
    import torch

    n = 64
    escape = [(i, 0.06 + 0.05 * (i % 4)) for i in range(n)]  # out after 3, 2, 1 and 1 steps
    cur, prev, w = system(n, 5, escape)
    lim, tick, eps = (-1.0, -1.0, 1.0, 1.0), 1e-3, 1e-3
    st = make_stars(engine, cur, prev, w, 2, lim, tick, eps)
    st.update(3)
    torch.cuda.synchronize()
    k, _, _, w_ref = oracle_steps(orc, cur, prev, w, 2, lim, tick, eps, 3)
    assert st.num_star_ == k == 0
    np.testing.assert_array_equal(st.gpuptr_weight_.cpu().numpy(), w_ref)
    st.update(2)
    st.prune()
    torch.cuda.synchronize()
    assert st.num_star_ == 0
    np.testing.assert_array_equal(st.gpuptr_weight_.cpu().numpy(), w_ref)  # nothing moved

    empty = engine.Stars(3, 0, 32, 24, 30, tick, 1.0, 0.01, lim, lim, epsilon=eps)
    empty.update(4)
    empty.prune()
    board = torch.full((engine.frame_bytes(32, 24),), 7, dtype=torch.uint8, device="cuda")
    empty.display(board)
    torch.cuda.synchronize()
    assert empty.num_star_ == 0
    assert torch.all(board[:32 * 24] == 0) and torch.all(board[32 * 24:] == 128)
