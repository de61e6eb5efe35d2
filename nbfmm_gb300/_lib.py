"""ctypes binding of libnbfmm_gb300.so (include/nbfmm_gb300.h). Loading fails loudly when the library is
missing: there is no CPU fallback."""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libnbfmm_gb300.so")

NBFMM_OK = 0
NBFMM_ERR_INVALID = 1
NBFMM_ERR_CUDA = 2
NBFMM_ERR_NOMEM = 3
NBFMM_ARITH_FAST = 0
NBFMM_ARITH_EXACT = 1

_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_float_p = ctypes.POINTER(ctypes.c_float)
_vp = ctypes.c_void_p

# name -> (restype, argtypes); every symbol include/nbfmm_gb300.h declares.
SIGNATURES = {
    "nbfmm_last_error": (ctypes.c_char_p, []),
    "nbfmm_version": (ctypes.c_int, []),
    "nbfmm_solver_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _c_float_p, ctypes.POINTER(_vp)]),
    "nbfmm_solver_destroy": (ctypes.c_int, [_vp]),
    "nbfmm_solver_set_epsilon": (ctypes.c_int, [_vp, ctypes.c_float]),
    "nbfmm_solver_set_arithmetic": (ctypes.c_int, [_vp, ctypes.c_int]),
    "nbfmm_solver_solve": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, _vp, _vp]),
    "nbfmm_solver_predo": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, _vp]),
    "nbfmm_solver_p2p": (ctypes.c_int, [_vp, ctypes.c_int, _vp]),
    "nbfmm_solver_p2m": (ctypes.c_int, [_vp, ctypes.c_int, _vp]),
    "nbfmm_solver_m2m": (ctypes.c_int, [_vp, _vp]),
    "nbfmm_solver_m2l": (ctypes.c_int, [_vp, _vp]),
    "nbfmm_solver_l2l": (ctypes.c_int, [_vp, _vp]),
    "nbfmm_solver_l2p": (ctypes.c_int, [_vp, ctypes.c_int, _vp]),
    "nbfmm_solver_postdo": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp]),
    "nbfmm_solver_get_buffers": (ctypes.c_int, [_vp, _vp]),
    "nbfmm_stars_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float, _c_float_p,
                                          ctypes.POINTER(_vp)]),
    "nbfmm_stars_destroy": (ctypes.c_int, [_vp]),
    "nbfmm_stars_set_epsilon": (ctypes.c_int, [_vp, ctypes.c_float]),
    "nbfmm_stars_set_arithmetic": (ctypes.c_int, [_vp, ctypes.c_int]),
    "nbfmm_stars_state": (ctypes.c_int, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp)]),
    "nbfmm_stars_num_star": (ctypes.c_int, [_vp, _c_int_p]),
    "nbfmm_stars_update": (ctypes.c_int, [_vp, ctypes.c_int, _vp]),
    "nbfmm_stars_prune": (ctypes.c_int, [_vp, _vp]),
    "nbfmm_debug_fail_allocations_after": (ctypes.c_int, [ctypes.c_int]),
    "nbfmm_device_malloc": (ctypes.c_int, [ctypes.c_ulonglong, ctypes.POINTER(_vp)]),
    "nbfmm_device_free": (ctypes.c_int, [_vp]),
    "nbfmm_memcpy_to_device": (ctypes.c_int, [_vp, _vp, ctypes.c_ulonglong]),
    "nbfmm_memcpy_to_host": (ctypes.c_int, [_vp, _vp, ctypes.c_ulonglong]),
    "nbfmm_frame_bytes": (ctypes.c_longlong, [ctypes.c_int, ctypes.c_int]),
    "nbfmm_display": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, _c_float_p, _vp, _vp,
                                     _vp, _vp]),
    "nbfmm_stars_display": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_float, _c_float_p, _vp, _vp]),
    "nbfmm_movie_open": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_float, _c_float_p, ctypes.POINTER(_vp)]),
    "nbfmm_movie_frame": (ctypes.c_int, [_vp, _vp]),
    "nbfmm_movie_close": (ctypes.c_int, [_vp]),
    "nbfmm_batch_create": (ctypes.c_int, [ctypes.c_int, _c_int_p, _c_int_p, _c_float_p, ctypes.c_float,
                                          ctypes.c_float, ctypes.POINTER(_vp)]),
    "nbfmm_batch_destroy": (ctypes.c_int, [_vp]),
    "nbfmm_batch_set_epsilon": (ctypes.c_int, [_vp, ctypes.c_float]),
    "nbfmm_batch_set_arithmetic": (ctypes.c_int, [_vp, ctypes.c_int]),
    "nbfmm_batch_set_item_passes": (ctypes.c_int, [_vp, _c_int_p]),
    "nbfmm_batch_state": (ctypes.c_int, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp)]),
    "nbfmm_batch_num_stars": (ctypes.c_int, [_vp, _c_int_p]),
    "nbfmm_batch_update": (ctypes.c_int, [_vp, ctypes.c_int, _vp]),
    "nbfmm_batch_profile_begin": (ctypes.c_int, [_vp, ctypes.c_int]),
    "nbfmm_batch_profile_end": (ctypes.c_int, [_vp, _c_float_p, _c_int_p]),
    "nbfmm_batch_kernel_launches": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)]),
    "nbfmm_adjoint_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _c_float_p, ctypes.c_float, ctypes.c_float,
                                            ctypes.c_int, ctypes.c_int, ctypes.POINTER(_vp)]),
    "nbfmm_adjoint_destroy": (ctypes.c_int, [_vp]),
    "nbfmm_adjoint_set_epsilon": (ctypes.c_int, [_vp, ctypes.c_float]),
    "nbfmm_adjoint_forward": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, _vp, _vp, _vp]),
    "nbfmm_adjoint_backward": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "nbfmm_model_circle_center": (ctypes.c_int, [ctypes.c_int, _c_float_p] + [ctypes.c_float] * 4 + [_vp] * 4),
    "nbfmm_model_circle_uniform_center": (ctypes.c_int, [ctypes.c_int, _c_float_p] + [ctypes.c_float] * 4 + [_vp] * 4),
    "nbfmm_model_disk": (ctypes.c_int, [ctypes.c_int, _c_float_p] + [ctypes.c_float] * 3 + [_vp] * 4),
    "nbfmm_model_disk_center": (ctypes.c_int, [ctypes.c_int, _c_float_p] + [ctypes.c_float] * 4 + [_vp] * 4),
    "nbfmm_model_disk_static": (ctypes.c_int, [ctypes.c_int, _c_float_p] + [ctypes.c_float] * 3 + [_vp] * 4),
    "nbfmm_model_double_disk": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _c_float_p, _c_float_p] + [ctypes.c_float] * 5 + [_vp] * 4),
    "nbfmm_model_double_disk_center": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _c_float_p, _c_float_p] + [ctypes.c_float] * 7 + [_vp] * 4),
    "nbfmm_model_rectangle": (ctypes.c_int, [ctypes.c_int, _c_float_p] + [ctypes.c_float] * 4 + [_vp] * 4),
    "nbfmm_model_set_uniforms": (ctypes.c_int, [_vp]),
    "nbfmm_sort_cells_noalloc": (ctypes.c_int, [ctypes.c_int, _c_float_p, ctypes.c_int, _vp, _vp, _vp, _vp]),
    "nbfmm_stars_profile_begin": (ctypes.c_int, [_vp, ctypes.c_int]),
    "nbfmm_stars_profile_end": (ctypes.c_int, [_vp, _c_float_p, _c_int_p]),
    "nbfmm_stars_kernel_launches": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)]),
}


class SolverBuffers(ctypes.Structure):
    _fields_ = [
        ("num_level", ctypes.c_int),
        ("base_dim", ctypes.c_int),
        ("max_num_particle", ctypes.c_int),
        ("num_cell_levels", ctypes.c_int),
        ("level_dim", ctypes.c_int * 11),
        ("level_offset", ctypes.c_int * 11),
        ("total_cells", ctypes.c_int),
        ("particle", _vp),
        ("effect", _vp),
        ("cell_key", _vp),
        ("perm", _vp),
        ("head", _vp),
        ("cell", _vp),
        ("cell_effect", _vp),
    ]


_lib = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Loads the engine library (once) and declares every entry point. Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"nbfmm_gb300: {path} is missing; build it with `python -m nbfmm_gb300.build` "
                           "(the engine has no CPU fallback)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
