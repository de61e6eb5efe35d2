"""CPU: the oracle pinned against the reference's golden vectors and its CPU-compiled arithmetic.

The golden vectors come from tests/golden/make_golden.py: the fixture of check/core/solver.cu:17-69 and the
known answers of check/core/solver/*.cu, evaluated with the reference's own kernelFunction and operators.
Tolerances follow the reference's tests (CPPUNIT_ASSERT_DOUBLES_EQUAL(..., 1e-4), absolute) where the
summation order differs, and are exact where it does not.
"""
import numpy as np
import pytest

L, B, N = 3, 16, 250
LIMITS = (0.0, -1.0, 8.0, 2.0)


def cube(a, last=2):
    return a.reshape((L, B, B, last) if last else (L, B, B))


def test_kernel_function_matches_reference_samples(golden, orc):
    t = golden["kf_target"].reshape(-1, 2)
    s = golden["kf_source"].reshape(-1, 2)
    m = golden["kf_mass"]
    ref = golden["kf_effect"].reshape(-1, 2)
    got = np.array([orc.kernel_function(t[i], s[i], m[i], 0.1) for i in range(len(m))], np.float32)
    np.testing.assert_array_equal(got, ref)  # bit-exact, coincident pairs included


def test_kernel_function_matches_reference_library(orc):
    ref = orc.ref_lib()
    if ref is None:
        pytest.skip("oracle/_ref not built (reference sources absent)")
    rng = np.random.default_rng(7)
    n = 20000
    t = rng.uniform(-3, 3, (n, 2)).astype(np.float32)
    s = (t + rng.normal(0, 0.05, (n, 2))).astype(np.float32)
    m = rng.exponential(1.0, n).astype(np.float32)
    out = np.zeros((n, 2), np.float32)
    ref.ref_kernel_function_batch(n, t, s, m, out)
    got = np.array([orc.kernel_function(t[i], s[i], m[i], 0.1) for i in range(n)], np.float32)
    np.testing.assert_array_equal(got, out)


def test_row_major_key_order_matches_reference_operator(orc):
    ref = orc.ref_lib()
    if ref is None:
        pytest.skip("oracle/_ref not built (reference sources absent)")
    rng = np.random.default_rng(3)
    a = rng.integers(0, 64, (5000, 2))
    b = rng.integers(0, 64, (5000, 2))
    for (ax, ay), (bx, by) in zip(a, b):
        lt = bool(ref.ref_int2_less(int(ax), int(ay), int(bx), int(by)))
        eq = bool(ref.ref_int2_equal(int(ax), int(ay), int(bx), int(by)))
        assert lt == (ax + ay * 64 < bx + by * 64)
        assert eq == (ax + ay * 64 == bx + by * 64)


def test_predo_reference_checks(golden, orc):
    pos = golden["position"].reshape(-1, 2)
    w = golden["weight"]
    r = orc.predo(pos, w, L, LIMITS)
    cs = np.float32((LIMITS[2] - LIMITS[0]) / B), np.float32((LIMITS[3] - LIMITS[1]) / B)
    perm, idx, head = r["perm"], r["index"], r["head"]
    # check/core/solver/predo.cu:58-66
    np.testing.assert_array_equal(r["position"], pos[perm])
    np.testing.assert_array_equal(r["weight"], w[perm])
    for d in range(2):
        lo = np.float32(LIMITS[d])
        assert np.all(r["position"][:, d] >= idx[:, d].astype(np.float32) * cs[d] + lo)
        assert np.all(r["position"][:, d] < (idx[:, d] + 1).astype(np.float32) * cs[d] + lo)
    for c in range(B * B):
        seg = idx[head[c]:head[c + 1]]
        assert np.all(seg[:, 0] == c % B) and np.all(seg[:, 1] == c // B)
    # stable order: equal cells keep input order, and the permutation is a permutation
    key = idx[:, 0] + idx[:, 1] * B
    assert np.all(np.diff(key) >= 0)
    same = np.diff(key) == 0
    assert np.all(np.diff(perm)[same] > 0)
    assert sorted(perm.tolist()) == list(range(N))
    assert head[-1] == N


def test_postdo_golden(golden, orc):
    out = orc.postdo(golden["perm"], golden["position"].reshape(-1, 2))
    np.testing.assert_array_equal(out, golden["postdo_effect_origin"].reshape(-1, 2))


@pytest.mark.parametrize("block", [False, True])
def test_p2p_golden(golden, orc, block):
    eff = orc.p2p(golden["position"].reshape(-1, 2), golden["weight"], golden["index"].reshape(-1, 2),
                  golden["head"], B, 0.1, block=block)
    np.testing.assert_allclose(eff, golden["p2p_effect"].reshape(-1, 2), rtol=0, atol=1e-4)


def test_p2m_golden(golden, orc):
    cp, cw = orc.p2m(golden["position"].reshape(-1, 2), golden["weight"], golden["head"], B)
    np.testing.assert_allclose(cp, golden["p2m_cell_position"].reshape(-1, 2), rtol=0, atol=1e-4)
    np.testing.assert_allclose(cw, golden["p2m_cell_weight"], rtol=0, atol=1e-4)


def test_m2m_golden(golden, orc):
    cp = golden["cell_position"].copy()
    cw = golden["cell_weight"].copy()
    cp, cw = orc.m2m(cp, cw, L, B)
    ref_p, ref_w = cube(golden["m2m_cell_position"]), cube(golden["m2m_cell_weight"], 0)
    cp, cw = cube(cp), cube(cw, 0)
    for lv in range(L):
        s = 1 << lv
        np.testing.assert_allclose(cp[lv, ::s, ::s], ref_p[lv, ::s, ::s], rtol=0, atol=1e-4)
        np.testing.assert_allclose(cw[lv, ::s, ::s], ref_w[lv, ::s, ::s], rtol=0, atol=1e-4)


def test_m2l_golden(golden, orc):
    ce = cube(orc.m2l(golden["cell_position"], golden["cell_weight"], L, B, 0.1))
    ref = cube(golden["m2l_cell_effect"])
    for lv in range(L):
        s = 1 << lv
        np.testing.assert_allclose(ce[lv, ::s, ::s], ref[lv, ::s, ::s], rtol=0, atol=1e-4)


def test_l2l_golden(golden, orc):
    ce = cube(orc.l2l(golden["cell_position"], L, B))
    np.testing.assert_allclose(ce[0], golden["l2l_cell_effect0"].reshape(B, B, 2), rtol=0, atol=1e-4)


def test_l2p_golden(golden, orc):
    cell = cube(golden["cell_position"])
    eff = orc.l2p(golden["position"].reshape(-1, 2), golden["index"].reshape(-1, 2), cell[0], B)
    np.testing.assert_allclose(eff, golden["l2p_effect"].reshape(-1, 2), rtol=0, atol=1e-6)


def test_single_level_solve_is_direct_sum(orc):
    # num_level 0: B = 2, the 3x3 neighbourhood covers every cell and no far field runs (p2m.cu:80).
    rng = np.random.default_rng(11)
    pos = rng.uniform(-1, 1, (300, 2)).astype(np.float32)
    w = rng.uniform(0.5, 1.5, 300).astype(np.float32)
    eff = orc.solve(pos, w, 0, (-1, -1, 1, 1), eps=1e-3)
    ref = orc.direct_f64(pos, w, 1e-3)
    rel = np.linalg.norm(eff - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert rel.max() < 1e-4


def test_fmm_error_against_direct_sum_is_bounded(orc):
    rng = np.random.default_rng(12)
    pos = rng.uniform(-1, 1, (4096, 2)).astype(np.float32)
    w = rng.uniform(0.5, 1.5, 4096).astype(np.float32)
    eff = orc.solve(pos, w, 3, (-1, -1, 1, 1), eps=1e-3)
    ref = orc.direct_f64(pos, w, 1e-3)
    # The reference's method is zeroth order: monopoles at cell centres of mass, one constant local effect
    # per cell. On a uniform square (strong cancellation) that is ~14% of the RMS effect at depth 4.
    err = np.linalg.norm(eff - ref, axis=1) / np.sqrt(np.mean(np.sum(ref ** 2, axis=1)))
    assert 0.05 < np.median(err) < 0.25 and err.max() < 1.0


def test_block_and_naive_orders_agree(orc):
    rng = np.random.default_rng(13)
    pos = rng.uniform(-1, 1, (2000, 2)).astype(np.float32)
    w = rng.uniform(0.5, 1.5, 2000).astype(np.float32)
    a = orc.solve(pos, w, 3, (-1, -1, 1, 1), eps=1e-3, block=False)
    b = orc.solve(pos, w, 3, (-1, -1, 1, 1), eps=1e-3, block=True)
    from conftest import guarded_rel_err

    assert guarded_rel_err(a, b)[0] < 1e-4


def test_solve_targets_matches_solve(orc):
    rng = np.random.default_rng(14)
    pos = rng.uniform(-1, 1, (3000, 2)).astype(np.float32)
    w = rng.uniform(0.5, 1.5, 3000).astype(np.float32)
    full = orc.solve(pos, w, 4, (-1, -1, 1, 1), eps=1e-3)
    t = rng.choice(3000, 200, replace=False).astype(np.int32)
    part = orc.solve_targets(pos, w, 4, (-1, -1, 1, 1), 1e-3, t)
    np.testing.assert_array_equal(part, full[t])


def test_stars_update_prunes_stably(orc):
    # stars leaving the limits are dropped; the survivors keep their order (prune.cu:55-61)
    n = 64
    rng = np.random.default_rng(15)
    cur = rng.uniform(-0.9, 0.9, (n, 2)).astype(np.float32)
    prev = cur.copy()
    out = [3, 10, 40]
    cur[out, 0] = 0.5
    prev[out, 0] = cur[out, 0] - 1.0  # x' = 2x - x_prev = x + 1 = 1.5: leaves within a step
    w = np.full(n, 1e-6, np.float32)
    n_new, c2, p2, w2, _ = orc.stars_update(cur, prev, w, 2, (-1, -1, 1, 1), 1e-3, 1e-4)
    keep = [i for i in range(n) if i not in out]
    assert n_new == len(keep)
    np.testing.assert_array_equal(p2[:n_new], cur[keep])
    assert np.all(c2[n_new:, 0] > 1.0)


def test_cell_index_clamps_the_upper_edge(orc):
    pos = np.array([[1.0, 1.0], [-1.0, -1.0], [2.0, -5.0], [0.0, 0.0]], np.float32)
    r = orc.predo(pos, np.ones(4, np.float32), 1, (-1, -1, 1, 1))
    idx = r["index"][np.argsort(r["perm"])]
    np.testing.assert_array_equal(idx, [[3, 3], [0, 0], [3, 0], [2, 2]])


def test_display_matches_reference_golden_frames(display_golden, orc):
    """orc_display against frames drawn by the reference's own displayDevice (tests/golden)."""
    for c in display_golden:
        frame = orc.display(c["pos"], c["w"], c["width"], c["height"], c["size_scale"], c["limits"])
        assert frame.shape == c["frame"].shape
        np.testing.assert_array_equal(frame, c["frame"])


def test_display_matches_reference_library(orc):
    """orc_display against the reference's displayDevice compiled for the CPU (oracle/_ref), random fields."""
    L = orc.ref_lib()
    if L is None or not L.ref_has_display():
        pytest.skip("oracle/_ref was not built from the reference sources")
    rng = np.random.default_rng(7)
    for trial in range(25):
        width, height = int(rng.integers(1, 80)), int(rng.integers(1, 60))
        size_scale = float(rng.choice([0.1, 0.5, 1.0, 3.0]))
        limits = (-1.0, -0.5, float(rng.uniform(0.1, 2)), float(rng.uniform(0.1, 1)))
        n = int(rng.integers(0, 400))
        pos = np.stack([rng.uniform(-1.3, limits[2] + 0.3, n), rng.uniform(-0.8, limits[3] + 0.3, n)], 1)
        w = (rng.uniform(0, 10, n) * size_scale) ** 2
        frame = orc.display(pos, w, width, height, size_scale, limits)
        ref = orc.ref_display(pos, w, width, height, size_scale, limits)[0]
        np.testing.assert_array_equal(frame, ref, err_msg=f"trial {trial}: {width}x{height}")


def test_display_special_values(orc):
    """NaN, infinite and huge coordinates and weights convert as the GPU converts (saturating, NaN -> 0)."""
    pos = np.array([[np.nan, 0.0], [0.0, np.nan], [np.inf, 0.0], [-np.inf, 0.0], [1e30, 0.0], [0.0, -1e30],
                    [-0.75, -0.75]], np.float32)
    w = np.array([1.0, 1.0, 1.0, 1.0, 1.0, 1.0, -4.0], np.float32)
    frame = orc.display(pos, w, 8, 8, 1.0, (-1, -1, 1, 1))
    y = frame[:64].reshape(8, 8)
    lit = {(int(r), int(c)) for r, c in zip(*np.nonzero(y))}
    # NaN x -> column 0, row 4, size 1 (its left pixel is guarded); NaN y -> row 0, column 4 (the pixel above it
    # would be before the frame and is dropped); +-inf and 1e30 saturate off the frame; the negative weight
    # gives size floor(NaN) -> 0, the centre pixel alone (row 7, column 1).
    assert lit == {(4, 0), (4, 1), (3, 0), (5, 0), (0, 4), (0, 3), (0, 5), (1, 4), (7, 1)}
    assert np.all(frame[64:] == 128)


def test_prune_is_a_stable_partition(orc):
    rng = np.random.default_rng(3)
    n = 5000
    cur = rng.uniform(-1.5, 1.5, (n, 2)).astype(np.float32)
    cur[::97] = np.nan  # NaN is kept (the comparisons of prune.cu:40-41 are false)
    prev = rng.normal(size=(n, 2)).astype(np.float32)
    w = rng.uniform(size=n).astype(np.float32)
    limits = (-1.0, -1.0, 1.0, 1.0)
    out = (cur[:, 0] < -1) | (cur[:, 1] < -1) | (cur[:, 0] > 1) | (cur[:, 1] > 1)
    order = np.concatenate([np.flatnonzero(~out), np.flatnonzero(out)])
    ec, ep, ew = cur[order].copy(), prev[order].copy(), w[order].copy()
    kept = orc.prune(cur, prev, w, limits)
    assert kept == int((~out).sum())
    np.testing.assert_array_equal(cur, ec)
    np.testing.assert_array_equal(prev, ep)
    np.testing.assert_array_equal(w, ew)


def test_threaded_display_equals_sequential(orc):
    rng = np.random.default_rng(11)
    n = 300_000
    pos = rng.uniform(-1.1, 1.1, (n, 2)).astype(np.float32)
    w = (rng.uniform(0, 8, n) * 0.01) ** 2
    a = orc.display(pos, w, 320, 200, 0.01, (-1, -1, 1, 1))
    b = orc.display(pos, w, 320, 200, 0.01, (-1, -1, 1, 1), threads=True)
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("seed", [4, 5])
def test_prune_matches_reference_library(orc, seed):
    """The oracle's prune against the reference's own Stars::prune compiled for the CPU (oracle/_ref): its
    pruneDevice flags and thrust::sort_by_key over the zipped (cur, prev, w) arrays on thrust's host system,
    then thrust::find of the first flag (prune.cu:28-62). Same survivor count and the same arrays, bit for bit,
    with NaN, infinite and on-the-limit positions."""
    if orc.ref_prune(np.zeros((1, 2), np.float32), np.zeros((1, 2), np.float32), np.zeros(1, np.float32),
                     (-1, -1, 1, 1)) is None:
        pytest.skip("oracle/_ref not built (reference sources absent)")
    rng = np.random.default_rng(seed)
    n = 20000
    cur = rng.uniform(-1.3, 1.3, (n, 2)).astype(np.float32)
    cur[::101] = np.nan
    cur[5::211] = [np.inf, 0.0]
    cur[7::307] = [-1.0, 1.0]   # on the limits: kept (prune.cu:40-41 tests < and >)
    cur[9::401] = [0.0, -np.inf]
    prev = rng.normal(size=(n, 2)).astype(np.float32)
    w = rng.uniform(size=n).astype(np.float32)
    limits = (-1.0, -1.0, 1.0, 1.0)
    a = [cur.copy(), prev.copy(), w.copy()]
    b = [cur.copy(), prev.copy(), w.copy()]
    assert orc.prune(*a, limits) == orc.ref_prune(*b, limits)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.view(np.int32), y.view(np.int32))


MODEL_PARAMS = dict(center=(0.3, -0.2), radius=1.7, weight=1e-3, center_weight=5.0, tick=1e-3, width=2.0,
                    height=3.0, max_weight=2.0)


@pytest.mark.parametrize("kind", ["circle_center", "circle_uniform_center", "disk", "disk_center", "disk_static",
                                  "rectangle"])
def test_models_match_reference_kernels(orc, kind):
    """The oracle's model arithmetic against the reference's own generate*Device kernels compiled for the CPU
    (oracle/_ref), curand bound to the same uniform draws. Weights are equal; each coordinate is within one ulp
    of the coordinate scale (|centre| + the largest extent): the oracle rounds center + radius * cos(angle) once, as the
    CUDA compiler's fused multiply-add does, and the CPU build of the kernel rounds the product and the sum
    separately. The rectangle's x and y draws are two curand_uniform calls in one make_float2 argument list,
    whose evaluation order C++ leaves unspecified: g++ evaluates the y draw first, the oracle (and the engine)
    take the x draw first, so the reference is given the draws in that order."""
    if orc.ref_model(kind, 1, np.zeros((1, 3), np.float32), **MODEL_PARAMS) is None:
        pytest.skip("oracle/_ref not built (reference sources absent)")
    rng = np.random.default_rng(len(kind))
    n = 20000
    u = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    u_ref = u.copy()
    if kind == "rectangle":
        u_ref[:, [0, 1]] = u_ref[:, [1, 0]]
    ours = orc.model(kind, n, u, **MODEL_PARAMS)
    ref = orc.ref_model(kind, n, u_ref, **MODEL_PARAMS)
    scale = np.float32(abs(MODEL_PARAMS["center"][0]) + abs(MODEL_PARAMS["center"][1]) +
                       max(MODEL_PARAMS["radius"], MODEL_PARAMS["width"], MODEL_PARAMS["height"]))
    tol = np.spacing(scale)
    for name, a, b in zip(("cur", "prev"), ours[:2], ref[:2]):
        assert np.abs(a - b).max() <= tol, f"{name}: {np.abs(a - b).max() / np.spacing(scale):.3f} ulp"
    np.testing.assert_array_equal(ours[2], ref[2])
