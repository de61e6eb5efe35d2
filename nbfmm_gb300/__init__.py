"""nbfmm_gb300 -- GB300-native (sm_103a) 2D fast-multipole N-body engine behind nbfmm's Solver / Stars API.

Host mirror of the reference's C++ classes over the C ABI in include/nbfmm_gb300.h:

  nbfmm::Solver  (include/nbfmm/core/solver.hpp)    -> Solver(num_level, max_num_particle, position_limits)
                                                        .solve(num_particle, position, weight, effect)
                                                        .predo/.p2p/.p2m/.m2m/.m2l/.l2l/.l2p/.postdo
  nbfmm::Stars   (include/nbfmm/display/stars.hpp)  -> Stars(fmm_level, num_star, ..., tick, grav_const, ...,
                                                              position_limits, ...)
                                                        .initialize(func, *args), .update()

Device arrays are torch CUDA tensors (float32, contiguous) or raw device addresses (int). Positions and
effects are (n, 2) float32, weights (n,) float32, limits (x_min, y_min, x_max, y_max). Errors raise
NbfmmError where the reference asserts. The compute path is the CUDA library only; there is no CPU path.
"""
import ctypes

from . import _lib

__all__ = ["NbfmmError", "Solver", "Stars", "Batch", "Movie", "display", "frame_bytes", "load_library"]


class NbfmmError(RuntimeError):
    """A failed engine call; `code` is the NBFMM_ERR_* status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"nbfmm error {code}: {message}")
        self.code = code


def load_library():
    return _lib.load()


def _check(rc: int):
    if rc != _lib.NBFMM_OK:
        raise NbfmmError(rc, _lib.load().nbfmm_last_error().decode())


def _ptr(x, dtype: str = "float32"):
    if x is None:
        return None
    if isinstance(x, int):
        return x
    import torch

    if not isinstance(x, torch.Tensor):
        raise TypeError("expected a torch CUDA tensor or a device address")
    if not x.is_cuda:
        raise ValueError("tensor must live on the GPU")
    if x.dtype != getattr(torch, dtype):
        raise TypeError(f"tensor must be {dtype}, got {x.dtype}")
    if not x.is_contiguous():
        raise ValueError("tensor must be contiguous")
    return x.data_ptr()


def _stream(stream):
    if stream is None:
        try:
            import torch

            if torch.cuda.is_available():
                return torch.cuda.current_stream().cuda_stream
        except ImportError:
            pass
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def _limits(position_limits):
    vals = [float(v) for v in position_limits]
    if len(vals) != 4:
        raise ValueError("position_limits must be (x_min, y_min, x_max, y_max)")
    return (ctypes.c_float * 4)(*vals)


ARITHMETIC = {"fast": _lib.NBFMM_ARITH_FAST, "exact": _lib.NBFMM_ARITH_EXACT}


def _arithmetic(name: str) -> int:
    if name not in ARITHMETIC:
        raise ValueError(f"arithmetic must be one of {sorted(ARITHMETIC)}")
    return ARITHMETIC[name]


class _DeviceView:
    """Exposes a device range through __cuda_array_interface__ so torch can wrap it without a copy."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (ptr, False),
                                         "version": 2, "strides": None}


def _as_tensor(ptr, shape, typestr):
    import torch

    return torch.as_tensor(_DeviceView(ptr, shape, typestr), device="cuda")


class Solver:
    """nbfmm::Solver (include/nbfmm/core/solver.hpp:22-209) on the GB300 engine."""

    def __init__(self, num_level: int, max_num_particle: int, position_limits, epsilon: float = 0.1,
                 arithmetic: str = "fast"):
        lib = _lib.load()
        h = ctypes.c_void_p()
        _check(lib.nbfmm_solver_create(int(num_level), int(max_num_particle), _limits(position_limits),
                                       ctypes.byref(h)))
        self._h = h
        self.num_level = int(num_level)
        self.base_dim = 1 << (self.num_level + 1)
        self.max_num_particle = int(max_num_particle)
        self.position_limits = tuple(float(v) for v in position_limits)
        self.set_epsilon(epsilon)
        self.set_arithmetic(arithmetic)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().nbfmm_solver_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_epsilon(self, epsilon: float):
        _check(_lib.load().nbfmm_solver_set_epsilon(self._h, float(epsilon)))
        self.epsilon = float(epsilon)

    def set_arithmetic(self, arithmetic: str):
        """Near-field arithmetic: "fast" (hardware approximations, the default) or "exact" (correctly rounded
        sqrt and division, no fused multiply-add: the oracle's IEEE single-precision rounding)."""
        _check(_lib.load().nbfmm_solver_set_arithmetic(self._h, _arithmetic(arithmetic)))
        self.arithmetic = arithmetic

    def solve(self, num_particle, position, weight, effect, stream=None):
        """Solver::solve (solve.cu:11-27): effects of `num_particle` particles, caller order in and out."""
        _check(_lib.load().nbfmm_solver_solve(self._h, int(num_particle), _ptr(position), _ptr(weight), _ptr(effect),
                                              _stream(stream)))

    # Stage methods (public under NBFMM_CHECK in the reference, solver.hpp:24-28).
    def predo(self, num_particle, position, weight, stream=None):
        _check(_lib.load().nbfmm_solver_predo(self._h, int(num_particle), _ptr(position), _ptr(weight),
                                              _stream(stream)))

    def p2p(self, num_particle, stream=None):
        _check(_lib.load().nbfmm_solver_p2p(self._h, int(num_particle), _stream(stream)))

    def p2m(self, num_particle, stream=None):
        _check(_lib.load().nbfmm_solver_p2m(self._h, int(num_particle), _stream(stream)))

    def m2m(self, stream=None):
        _check(_lib.load().nbfmm_solver_m2m(self._h, _stream(stream)))

    def m2l(self, stream=None):
        _check(_lib.load().nbfmm_solver_m2l(self._h, _stream(stream)))

    def l2l(self, stream=None):
        _check(_lib.load().nbfmm_solver_l2l(self._h, _stream(stream)))

    def l2p(self, num_particle, stream=None):
        _check(_lib.load().nbfmm_solver_l2p(self._h, int(num_particle), _stream(stream)))

    def postdo(self, num_particle, effect, stream=None):
        _check(_lib.load().nbfmm_solver_postdo(self._h, int(num_particle), _ptr(effect), _stream(stream)))

    def buffers(self):
        """The workspace as torch tensors sharing device memory (the reference's gpuptr_* members)."""
        b = _lib.SolverBuffers()
        _check(_lib.load().nbfmm_solver_get_buffers(self._h, ctypes.byref(b)))
        n = b.max_num_particle
        cells = b.base_dim * b.base_dim
        return {
            "particle": _as_tensor(b.particle, (n, 4), "<f4"),
            "effect": _as_tensor(b.effect, (n, 2), "<f4"),
            "cell_key": _as_tensor(b.cell_key, (n,), "<i4"),
            "perm": _as_tensor(b.perm, (n,), "<i4"),
            "head": _as_tensor(b.head, (cells + 1,), "<i4"),
            "cell": _as_tensor(b.cell, (b.total_cells, 4), "<f4"),
            "cell_effect": _as_tensor(b.cell_effect, (b.total_cells, 2), "<f4"),
            "level_dim": list(b.level_dim[: b.num_cell_levels]),
            "level_offset": list(b.level_offset[: b.num_cell_levels]),
        }


class Stars:
    """nbfmm::Stars (include/nbfmm/display/stars.hpp:22-134), update path.

    Accepts the reference's constructor arguments (fmm_level, num_star, width, height, fps, tick, grav_const,
    size_scale, position_limits, display_limits); the display ones are used by display() and checked as the
    reference asserts them. display_limits defaults to position_limits. `epsilon` is the kernel softening (the
    reference fixes 1e-1).
    """

    def __init__(self, fmm_level, num_star, width=1, height=1, fps=1, tick=None, grav_const=1.0, size_scale=1.0,
                 position_limits=None, display_limits=None, *, epsilon: float = 0.1, arithmetic: str = "fast"):
        if tick is None or position_limits is None:
            raise ValueError("tick and position_limits are required")
        if int(width) <= 0 or int(height) <= 0 or int(fps) <= 0 or not float(size_scale) > 0:
            raise ValueError("width, height, fps and size_scale must be > 0 (stars.cu:37-41)")
        lib = _lib.load()
        h = ctypes.c_void_p()
        _check(lib.nbfmm_stars_create(int(fmm_level), int(num_star), float(tick), float(grav_const),
                                      _limits(position_limits), ctypes.byref(h)))
        self._h = h
        self.fmm_level = int(fmm_level)
        self.position_limits = tuple(float(v) for v in position_limits)
        self.display_limits = tuple(float(v) for v in (display_limits if display_limits is not None
                                                        else position_limits))
        if not (self.display_limits[0] < self.display_limits[2] and self.display_limits[1] < self.display_limits[3]):
            raise ValueError("display limits must satisfy x_min < x_max, y_min < y_max (stars.cu:43)")
        self.width_, self.height_, self.fps_ = int(width), int(height), int(fps)
        self.size_scale_ = float(size_scale)
        self.max_num_star = int(num_star)
        import numpy as np

        # tick_ = tick * sqrt(grav_const) in FP32 (stars.cu:31)
        self.tick_ = float(np.float32(tick) * np.sqrt(np.float32(grav_const)))
        self.set_epsilon(epsilon)
        self.set_arithmetic(arithmetic)
        cur, pre, w = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        _check(lib.nbfmm_stars_state(self._h, ctypes.byref(cur), ctypes.byref(pre), ctypes.byref(w)))
        self._ptrs = (cur.value, pre.value, w.value)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().nbfmm_stars_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_epsilon(self, epsilon: float):
        _check(_lib.load().nbfmm_stars_set_epsilon(self._h, float(epsilon)))
        self.epsilon = float(epsilon)

    def set_arithmetic(self, arithmetic: str):
        """Near-field arithmetic of the update's solves: "fast" (default) or "exact" (Solver.set_arithmetic)."""
        _check(_lib.load().nbfmm_stars_set_arithmetic(self._h, _arithmetic(arithmetic)))
        self.arithmetic = arithmetic

    @property
    def gpuptr_position_cur_(self):
        return _as_tensor(self._ptrs[0], (self.max_num_star, 2), "<f4")

    @property
    def gpuptr_position_pre_(self):
        return _as_tensor(self._ptrs[1], (self.max_num_star, 2), "<f4")

    @property
    def gpuptr_weight_(self):
        return _as_tensor(self._ptrs[2], (self.max_num_star,), "<f4")

    @property
    def num_star_(self) -> int:
        n = ctypes.c_int()
        _check(_lib.load().nbfmm_stars_num_star(self._h, ctypes.byref(n)))
        return n.value

    def initialize(self, func, *args):
        """Stars::initialize (stars.hpp:111-114): func(*args, tick_, cur, prev, weight)."""
        return func(*args, self.tick_, self.gpuptr_position_cur_, self.gpuptr_position_pre_, self.gpuptr_weight_)

    def update(self, num_steps: int = 1, stream=None):
        """`num_steps` x Stars::update() (update.cu:47-55) without host synchronisation."""
        _check(_lib.load().nbfmm_stars_update(self._h, int(num_steps), _stream(stream)))

    def prune(self, stream=None):
        """Stars::prune (prune.cu:28-62) on the public arrays."""
        _check(_lib.load().nbfmm_stars_prune(self._h, _stream(stream)))

    def display(self, board, stream=None):
        """Stars::display(board) (display.cu:219-229): draw the frame (uint8 CUDA tensor or device address of
        frame_bytes(width, height) bytes), then prune."""
        _check(_lib.load().nbfmm_stars_display(self._h, self.width_, self.height_, self.size_scale_,
                                               _limits(self.display_limits), _ptr(board, "uint8"), _stream(stream)))

    # Engine instrumentation (no reference counterpart).
    def profile_begin(self, max_steps: int):
        """Time the P2P launch of each of the next `max_steps` steps with CUDA events on the update stream."""
        _check(_lib.load().nbfmm_stars_profile_begin(self._h, int(max_steps)))

    def profile_end(self):
        """(total P2P milliseconds, timed launches) of the session; synchronises."""
        ms, k = ctypes.c_float(), ctypes.c_int()
        _check(_lib.load().nbfmm_stars_profile_end(self._h, ctypes.byref(ms), ctypes.byref(k)))
        return float(ms.value), int(k.value)

    def kernel_launches(self, num_steps: int) -> int:
        """Engine kernels one update(num_steps) call launches."""
        out = ctypes.c_longlong()
        _check(_lib.load().nbfmm_stars_kernel_launches(self._h, int(num_steps), ctypes.byref(out)))
        return int(out.value)


class Batch:
    """Many independent systems stepped together (the batched form; no counterpart in the reference).

    System s owns particles [particle_offsets[s], particle_offsets[s+1]) of the shared state arrays, its own
    `position_limits[s]` = (x_min, y_min, x_max, y_max) and tree depth `num_levels[s]`. Each update step of
    each system is one Stars::update of that system alone.
    """

    def __init__(self, particle_offsets, num_levels, position_limits, tick, grav_const=1.0, epsilon: float = 0.1,
                 arithmetic: str = "fast"):
        import numpy as np

        off = np.ascontiguousarray(particle_offsets, dtype=np.int32)
        lev = np.ascontiguousarray(num_levels, dtype=np.int32)
        lim = np.ascontiguousarray(position_limits, dtype=np.float32).reshape(-1)
        self.num_systems = int(len(lev))
        if len(off) != self.num_systems + 1 or len(lim) != 4 * self.num_systems:
            raise ValueError("need num_systems+1 offsets and 4 limits per system")
        lib = _lib.load()
        h = ctypes.c_void_p()
        _check(lib.nbfmm_batch_create(self.num_systems, off.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                      lev.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                      lim.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), float(tick),
                                      float(grav_const), ctypes.byref(h)))
        self._h = h
        self.particle_offsets = off.tolist()
        self.num_particles = int(off[-1])
        self.set_epsilon(epsilon)
        self.set_arithmetic(arithmetic)
        cur, pre, w = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        _check(lib.nbfmm_batch_state(self._h, ctypes.byref(cur), ctypes.byref(pre), ctypes.byref(w)))
        self._ptrs = (cur.value, pre.value, w.value)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().nbfmm_batch_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_epsilon(self, epsilon: float):
        _check(_lib.load().nbfmm_batch_set_epsilon(self._h, float(epsilon)))
        self.epsilon = float(epsilon)

    def set_arithmetic(self, arithmetic: str):
        """Near-field arithmetic of every system's solves: "fast" (default) or "exact" (Solver.set_arithmetic)."""
        _check(_lib.load().nbfmm_batch_set_arithmetic(self._h, _arithmetic(arithmetic)))
        self.arithmetic = arithmetic

    def set_item_passes(self, passes_per_item):
        """P2P work-item size of each system: 2 or 4 passes of 32 target stars (a tile shape; results do not
        depend on it)."""
        import numpy as np

        p = np.ascontiguousarray(passes_per_item, dtype=np.int32)
        if len(p) != self.num_systems:
            raise ValueError("one value per system")
        _check(_lib.load().nbfmm_batch_set_item_passes(self._h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))

    @property
    def position_cur(self):
        return _as_tensor(self._ptrs[0], (max(self.num_particles, 1), 2), "<f4")[: self.num_particles]

    @property
    def position_pre(self):
        return _as_tensor(self._ptrs[1], (max(self.num_particles, 1), 2), "<f4")[: self.num_particles]

    @property
    def weight(self):
        return _as_tensor(self._ptrs[2], (max(self.num_particles, 1),), "<f4")[: self.num_particles]

    @property
    def num_stars(self):
        out = (ctypes.c_int * self.num_systems)()
        _check(_lib.load().nbfmm_batch_num_stars(self._h, out))
        return list(out)

    def update(self, num_steps: int = 1, stream=None):
        _check(_lib.load().nbfmm_batch_update(self._h, int(num_steps), _stream(stream)))

    def profile_begin(self, max_steps: int):
        _check(_lib.load().nbfmm_batch_profile_begin(self._h, int(max_steps)))

    def profile_end(self):
        ms, k = ctypes.c_float(), ctypes.c_int()
        _check(_lib.load().nbfmm_batch_profile_end(self._h, ctypes.byref(ms), ctypes.byref(k)))
        return float(ms.value), int(k.value)

    def kernel_launches(self, num_steps: int) -> int:
        out = ctypes.c_longlong()
        _check(_lib.load().nbfmm_batch_kernel_launches(self._h, int(num_steps), ctypes.byref(out)))
        return int(out.value)


def frame_bytes(width: int, height: int) -> int:
    """Bytes of one YUV 4:2:0 frame, width*height*3/2 (main.cu:234)."""
    return int(_lib.load().nbfmm_frame_bytes(int(width), int(height)))


def display(position, weight, width, height, size_scale, display_limits, board, num_star=None, stream=None):
    """The raster of Stars::display (display.cu:29-221) for any device arrays: position (n, 2) float32, weight
    (n,) float32, board uint8 of frame_bytes(width, height) bytes."""
    n = int(num_star if num_star is not None else (weight.shape[0] if hasattr(weight, "shape") else 0))
    _check(_lib.load().nbfmm_display(n, int(width), int(height), float(size_scale), _limits(display_limits),
                                     _ptr(position), _ptr(weight), _ptr(board, "uint8"), _stream(stream)))


class Movie:
    """The .y4m movie of main.cu:228-259 for one Stars: frame() is Stars::display into the next frame (with its
    prune); the file write of a frame overlaps the GPU work queued before the next frame() or close()."""

    def __init__(self, stars: Stars, path: str):
        h = ctypes.c_void_p()
        _check(_lib.load().nbfmm_movie_open(stars._h, str(path).encode(), stars.width_, stars.height_, stars.fps_,
                                            stars.size_scale_, _limits(stars.display_limits), ctypes.byref(h)))
        self._h = h
        self._stars = stars

    def frame(self, stream=None):
        _check(_lib.load().nbfmm_movie_frame(self._h, _stream(stream)))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            h, self._h = self._h, None
            _check(_lib.load().nbfmm_movie_close(h))
        self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
