"""GPU: the reference's initial-condition models. With injected draws the engine's arithmetic is compared with
the oracle's restatement (identical draws; only the device's cosf/sinf/acos rounding may differ, by a few
ulps); with curand the stream is the reference's own (curand_init(0, idx, 0)), checked for its invariants."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = {
    "circle_center": dict(n=3000, center=(0.1, -0.2), radius=0.7, weight=1e-3, center_weight=5.0, tick=2e-3),
    "circle_uniform_center": dict(n=3000, center=(0.0, 0.0), radius=0.5, weight=1e-3, center_weight=3.0, tick=1e-3),
    "disk": dict(n=4097, center=(0.25, 0.0), radius=1.0, weight=2e-4, tick=1e-3),
    "disk_center": dict(n=4097, center=(0.0, 0.3), radius=0.8, weight=2e-4, center_weight=10.0, tick=1e-3),
    "disk_static": dict(n=2049, center=(-0.1, 0.1), radius=0.6, weight=1e-3, tick=1e-3),
    "rectangle": dict(n=5000, center=(0.5, -0.5), width=2.0, height=1.0, max_weight=2.0, tick=1e-3),
    "double_disk": dict(n1=3000, n2=2000, center1=(-0.6, 0.0), center2=(0.6, 0.1), radius1=0.5, radius2=0.4,
                        weight=1e-4, eccentricity=0.3, tick=1e-3),
    "double_disk_center": dict(n1=3000, n2=2000, center1=(-0.6, 0.0), center2=(0.6, 0.1), radius1=0.5, radius2=0.4,
                               weight=1e-4, center_weight1=5.0, center_weight2=3.0, eccentricity=0.3, tick=1e-3),
}


def generate(engine, kind, p):
    import torch
    from nbfmm_gb300 import model

    n = p.get("n", p.get("n1", 0) + p.get("n2", 0))
    cur = torch.full((n, 2), float("nan"), device="cuda")
    prev = torch.full((n, 2), float("nan"), device="cuda")
    w = torch.full((n,), float("nan"), device="cuda")
    if kind == "circle_center":
        model.generateCircleCenter(n, p["center"], p["radius"], p["weight"], p["center_weight"], p["tick"], cur, prev, w)
    elif kind == "circle_uniform_center":
        model.generateCircleUniformCenter(n, p["center"], p["radius"], p["weight"], p["center_weight"], p["tick"], cur,
                                          prev, w)
    elif kind == "disk":
        model.generateDisk(n, p["center"], p["radius"], p["weight"], p["tick"], cur, prev, w)
    elif kind == "disk_center":
        model.generateDiskCenter(n, p["center"], p["radius"], p["weight"], p["center_weight"], p["tick"], cur, prev, w)
    elif kind == "disk_static":
        model.generateDiskStatic(n, p["center"], p["radius"], p["weight"], p["tick"], cur, prev, w)
    elif kind == "rectangle":
        model.generateRectangle(n, p["center"], p["width"], p["height"], p["max_weight"], p["tick"], cur, prev, w)
    elif kind == "double_disk":
        model.generateDoubleDisk(p["n1"], p["n2"], p["center1"], p["center2"], p["radius1"], p["radius2"], p["weight"],
                                 p["eccentricity"], p["tick"], cur, prev, w)
    else:
        model.generateDoubleDiskCenter(p["n1"], p["n2"], p["center1"], p["center2"], p["radius1"], p["radius2"],
                                       p["weight"], p["center_weight1"], p["center_weight2"], p["eccentricity"],
                                       p["tick"], cur, prev, w)
    torch.cuda.synchronize()
    return cur.cpu().numpy(), prev.cpu().numpy(), w.cpu().numpy()


@pytest.mark.parametrize("kind", sorted(CASES))
def test_model_arithmetic_matches_restatement(engine, orc, kind):
    import torch
    from nbfmm_gb300 import model

    p = CASES[kind]
    n = p.get("n", p.get("n1", 0) + p.get("n2", 0))
    u = np.random.default_rng(len(kind)).uniform(1e-7, 1.0, (n, 3)).astype(np.float32)
    model.set_uniforms(torch.from_numpy(u).cuda())
    try:
        cur, prev, w = generate(engine, kind, p)
    finally:
        model.set_uniforms(None)
    rc, rp, rw = orc.model(kind, p.get("n", 0), u, **{k: v for k, v in p.items() if k != "n"})
    np.testing.assert_array_equal(w, rw)
    scale = np.abs(rc).max() + 1.0
    tol = 8 * np.finfo(np.float32).eps * scale  # device cosf/sinf (and double acos) vs the host's: a few ulps
    assert np.abs(cur - rc).max() <= tol, np.abs(cur - rc).max()
    assert np.abs(prev - rp).max() <= tol, np.abs(prev - rp).max()


@pytest.mark.parametrize("kind", sorted(CASES))
def test_model_with_curand_is_deterministic_and_in_shape(engine, kind):
    p = CASES[kind]
    a = generate(engine, kind, p)
    b = generate(engine, kind, p)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    cur, prev, w = a
    assert np.all(np.isfinite(cur)) and np.all(np.isfinite(prev)) and np.all(np.isfinite(w))
    if kind in ("disk", "disk_static"):
        r = np.linalg.norm(cur - np.asarray(p["center"], np.float32), axis=1)
        expect = (np.arange(1, p["n"] + 1, dtype=np.float32) / np.float32(p["n"])) * np.float32(p["radius"])
        np.testing.assert_allclose(r, expect, rtol=1e-5, atol=1e-6)
    if kind == "rectangle":
        lo = np.asarray(p["center"]) - 0.5 * np.asarray([p["width"], p["height"]])
        hi = np.asarray(p["center"]) + 0.5 * np.asarray([p["width"], p["height"]])
        assert np.all(cur >= lo - 1e-6) and np.all(cur <= hi + 1e-6)
        assert np.all(w > 0) and np.all(w <= p["max_weight"])
    if kind == "double_disk":  # the second disk repeats the first's draws (its curand_init starts at idx 0 too)
        n2 = p["n2"]
        a1 = np.arctan2(cur[1:n2, 1] - p["center1"][1], cur[1:n2, 0] - p["center1"][0])
        a2 = np.arctan2(cur[p["n1"] + 1:p["n1"] + n2, 1] - p["center2"][1], cur[p["n1"] + 1:p["n1"] + n2, 0] - p["center2"][0])
        np.testing.assert_allclose(np.cos(a1), np.cos(a2), atol=1e-4)


def test_initialize_with_a_reference_model(engine):
    import torch
    from nbfmm_gb300 import model

    st = engine.Stars(4, 8192, tick=1e-3, grav_const=1.0, position_limits=(-1.5, -1.5, 1.5, 1.5), epsilon=1e-2)
    st.initialize(model.generateDiskCenter, 8192, (0.0, 0.0), 1.0, 1e-4, 10.0)
    st.update(10)
    torch.cuda.synchronize()
    n = st.num_star_
    assert 8000 < n <= 8192
    assert torch.all(torch.isfinite(st.gpuptr_position_cur_[:n]))
