"""Reverse mode of the engine's approximate method through a Stormer-Verlet trajectory (include/nbfmm_gb300.h,
nbfmm_adjoint_*). `Adjoint` mirrors the C ABI; `TrajectoryLoss` is a thin torch.autograd.Function over it, for
checking gradients against torch tooling only -- the computation is the CUDA library's."""
import ctypes

from . import _lib, _check, _limits, _ptr, _stream


class Adjoint:
    def __init__(self, num_level, num_particle, position_limits, tick, grav_const=1.0, max_steps=200,
                 checkpoint_interval=20, epsilon=0.1):
        lib = _lib.load()
        h = ctypes.c_void_p()
        _check(lib.nbfmm_adjoint_create(int(num_level), int(num_particle), _limits(position_limits), float(tick),
                                        float(grav_const), int(max_steps), int(checkpoint_interval), ctypes.byref(h)))
        self._h = h
        self.num_particle = int(num_particle)
        _check(lib.nbfmm_adjoint_set_epsilon(self._h, float(epsilon)))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().nbfmm_adjoint_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, num_steps, position0, velocity0, weight, position_final, stream=None):
        _check(_lib.load().nbfmm_adjoint_forward(self._h, int(num_steps), _ptr(position0), _ptr(velocity0),
                                                 _ptr(weight), _ptr(position_final), _stream(stream)))

    def backward(self, target, grad_position0, grad_velocity0, grad_weight, loss_terms=None, stream=None):
        _check(_lib.load().nbfmm_adjoint_backward(self._h, _ptr(target), _ptr(grad_position0), _ptr(grad_velocity0),
                                                  _ptr(grad_weight), _ptr(loss_terms), _stream(stream)))


def _autograd_function():
    import torch

    class TrajectoryLoss(torch.autograd.Function):
        """loss = 0.5 sum m |x(T) - target|^2 of an `Adjoint` trajectory; gradients for x0, v0 and m."""

        @staticmethod
        def forward(ctx, x0, v0, m, target, adj, num_steps):
            x0, v0, m, target = (t.detach().contiguous() for t in (x0, v0, m, target))
            xT = torch.empty_like(x0)
            adj.forward(num_steps, x0, v0, m, xT)
            gx, gv, gm = torch.empty_like(x0), torch.empty_like(v0), torch.empty_like(m)
            terms = torch.empty_like(m)
            adj.backward(target, gx, gv, gm, terms)
            ctx.save_for_backward(gx, gv, gm)
            return terms.double().sum().to(x0.dtype)

        @staticmethod
        def backward(ctx, grad_out):
            gx, gv, gm = ctx.saved_tensors
            return grad_out * gx, grad_out * gv, grad_out * gm, None, None, None

    return TrajectoryLoss


def trajectory_loss(x0, v0, m, target, adj, num_steps):
    return _autograd_function().apply(x0, v0, m, target, adj, num_steps)
