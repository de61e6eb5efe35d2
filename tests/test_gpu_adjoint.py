"""GPU: the adjoint of the approximate method through a Verlet trajectory.

Checked against (1) FP64 central finite differences (h = 1e-6) of the same approximate method evaluated in FP64
with the cell assignment of every step frozen (the oracle's orc_traj_fmm64), on sampled gradient components,
and (2) the exact FP64 adjoint of the all-pairs dynamics (how close the method's gradient is to the true one).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIM = (-1.25, -1.25, 1.25, 1.25)


def disk_system(n, seed, dt):
    from nbfmm_gb300 import workloads

    s = workloads.disk(n, seed=seed, num_level=3)
    rng = np.random.default_rng(seed + 100)
    return s.position.astype(np.float64), s.velocity.astype(np.float64), s.weight.astype(np.float64), rng


def gpu_grads(engine, x0, v0, m, target, level, eps, dt, steps, k=20):
    import torch
    from nbfmm_gb300.adjoint import Adjoint

    n = len(m)
    adj = Adjoint(level, n, LIM, tick=dt, max_steps=steps, checkpoint_interval=k, epsilon=eps)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
    X0, V0, M, T = t(x0), t(v0), t(m), t(target)
    xT = torch.empty_like(X0)
    gx, gv, gm, terms = torch.empty_like(X0), torch.empty_like(V0), torch.empty_like(M), torch.empty_like(M)
    adj.forward(steps, X0, V0, M, xT)
    adj.backward(T, gx, gv, gm, terms)
    torch.cuda.synchronize()
    return gx.cpu().numpy().astype(np.float64), gv.cpu().numpy().astype(np.float64), \
        gm.cpu().numpy().astype(np.float64), float(terms.double().sum()), xT.cpu().numpy()


def fd_grads(orc, x0, v0, m, target, level, eps, tau, steps, comps_x, comps_v, comps_m, h=1e-6):
    f32 = lambda a: a.astype(np.float32).astype(np.float64)  # the engine starts from the FP32 inputs
    x0, v0, m, target = f32(x0), f32(v0), f32(m), f32(target)
    loss, keys = orc.traj_fmm64(x0, v0, m, level, LIM, eps, tau, steps, target)

    def L(x=x0, v=v0, mm=m):
        return orc.traj_fmm64(x, v, mm, level, LIM, eps, tau, steps, target, keys)[0]

    gx = []
    for c in comps_x:
        xp, xm = x0.copy(), x0.copy()
        xp[c] += h
        xm[c] -= h
        gx.append((L(x=xp) - L(x=xm)) / (2 * h))
    gv = []
    for c in comps_v:
        vp, vm = v0.copy(), v0.copy()
        vp[c] += h
        vm[c] -= h
        gv.append((L(v=vp) - L(v=vm)) / (2 * h))
    gm = []
    for i in comps_m:
        hm = h * m[i]
        mp, mm_ = m.copy(), m.copy()
        mp[i] += hm
        mm_[i] -= hm
        gm.append((L(mm=mp) - L(mm=mm_)) / (2 * hm))
    return loss, np.array(gx), np.array(gv), np.array(gm)


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


# At dt = 1e-4 the gradient is mostly m (x(T) - x*) with |x(T) - x*| ~ 1e-3 while the FP32 positions (~0.5)
# carry ulps of 6e-8 over 10 steps: the FP32 trajectory itself limits agreement to a few 1e-4. At dt = 5e-3 the
# force terms dominate and the agreement is ~1e-6.
@pytest.mark.parametrize("dt,tol", [(1e-4, 1e-3), (5e-3, 1e-4)])
def test_adjoint_matches_fp64_finite_differences(engine, orc, dt, tol):
    """N = 1,024 rotating disk, 10 steps, h = 1e-6; dt = 1e-4 (the measured configuration's step) and a larger
    dt where the force terms dominate the gradient."""
    x0, v0, m, rng = disk_system(1024, 5, dt)
    steps, level, eps = 10, 3, 1e-3
    target = x0 + v0 * dt * steps + rng.normal(0, 1e-3, x0.shape)
    gx, gv, gm, loss, _ = gpu_grads(engine, x0, v0, m, target, level, eps, dt, steps)
    cx = [tuple(c) for c in np.stack([rng.choice(1024, 24, replace=False), rng.integers(0, 2, 24)], 1)]
    cv = [tuple(c) for c in np.stack([rng.choice(1024, 24, replace=False), rng.integers(0, 2, 24)], 1)]
    cm = list(rng.choice(1024, 24, replace=False)) + [0]  # include the central mass
    floss, fx, fv, fm = fd_grads(orc, x0, v0, m, target, level, eps, np.float32(dt), steps, cx, cv, cm)
    assert abs(loss - floss) <= 1e-4 * floss
    ex = rel([gx[c] for c in cx], fx)
    ev = rel([gv[c] for c in cv], fv)
    em = rel([gm[i] for i in cm], fm)
    print(f"dt {dt}: relative gradient error vs FP64 FD: x0 {ex:.2e}  v0 {ev:.2e}  m {em:.2e}")
    assert ex < tol and ev < tol and em < tol


def test_adjoint_against_exact_direct_sum_adjoint(engine, orc):
    """The method's gradient against the exact FP64 gradient of the all-pairs dynamics: the difference is the
    method's own approximation (percent level), reported and bounded loosely."""
    dt, steps, level, eps = 5e-3, 10, 3, 1e-3
    x0, v0, m, rng = disk_system(1024, 6, dt)
    target = x0 + v0 * dt * steps + rng.normal(0, 1e-3, x0.shape)
    gx, gv, gm, loss, _ = gpu_grads(engine, x0, v0, m, target, level, eps, dt, steps)
    dl, dx, dv, dm = orc.traj_direct64_grad(x0.astype(np.float32).astype(np.float64),
                                            v0.astype(np.float32).astype(np.float64),
                                            m.astype(np.float32).astype(np.float64),
                                            eps, float(np.float32(dt)), steps,
                                            target.astype(np.float32).astype(np.float64))
    print(f"method vs exact gradient: x0 {rel(gx, dx):.2e} v0 {rel(gv, dv):.2e} m {rel(gm, dm):.2e}, "
          f"loss {loss:.4e} vs {dl:.4e}")
    assert rel(gx, dx) < 0.5 and rel(gv, dv) < 0.5 and rel(gm, dm) < 0.5


def test_checkpoint_interval_does_not_change_gradients(engine):
    x0, v0, m, rng = disk_system(2048, 7, 1e-3)
    target = x0 + rng.normal(0, 1e-3, x0.shape)
    ref = gpu_grads(engine, x0, v0, m, target, 3, 1e-3, 1e-3, 12, k=12)
    for k in (1, 5):
        got = gpu_grads(engine, x0, v0, m, target, 3, 1e-3, 1e-3, 12, k=k)
        for a, b in zip(got[:3], ref[:3]):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("steps", [1, 5])
def test_final_state_matches_stars_update(engine, steps):
    """The adjoint's forward trajectory is the Stars update without pruning. One step is bit-identical; later
    steps agree to rounding (Stars keeps its state in the previous step's cell order, which reorders the P2P
    sums within a cell)."""
    import torch

    x0, v0, m, rng = disk_system(4096, 8, 1e-4)
    _, _, _, _, xT = gpu_grads(engine, x0, v0, m, x0, 3, 1e-3, 1e-4, steps)
    st = engine.Stars(3, 4096, tick=1e-4, grav_const=1.0, position_limits=LIM, epsilon=1e-3)
    f = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
    x0f = x0.astype(np.float32)
    st.gpuptr_position_cur_[:] = f(x0f)
    st.gpuptr_position_pre_[:] = f(x0f - v0.astype(np.float32) * np.float32(1e-4))
    st.gpuptr_weight_[:] = f(m)
    st.update(steps)
    torch.cuda.synchronize()
    assert st.num_star_ == 4096
    got = st.gpuptr_position_cur_.cpu().numpy()
    if steps == 1:
        np.testing.assert_array_equal(got, xT)
    else:
        assert np.abs(got - xT).max() < 1e-6


def test_autograd_wrapper(engine):
    import torch
    from nbfmm_gb300.adjoint import Adjoint, trajectory_loss

    x0, v0, m, rng = disk_system(1024, 9, 1e-3)
    target = x0 + rng.normal(0, 1e-3, x0.shape)
    gx, gv, gm, loss, _ = gpu_grads(engine, x0, v0, m, target, 3, 1e-3, 1e-3, 6)
    adj = Adjoint(3, 1024, LIM, tick=1e-3, max_steps=6, checkpoint_interval=20, epsilon=1e-3)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda().requires_grad_(True)
    X0, V0, M = t(x0), t(v0), t(m)
    out = trajectory_loss(X0, V0, M, t(target).detach(), adj, 6)
    out.backward()
    np.testing.assert_array_equal(X0.grad.cpu().numpy(), gx.astype(np.float32))
    np.testing.assert_array_equal(M.grad.cpu().numpy(), gm.astype(np.float32))
    assert abs(float(out.detach()) - loss) <= 1e-6 * abs(loss)
