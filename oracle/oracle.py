"""Python binding of the CPU oracle (oracle/libnbfmm_oracle.so) -- TEST INFRASTRUCTURE ONLY.

Only the tests, __graft_entry__.smoke() and the CPU-baseline leg of bench.py import this module, as the
checker; the engine never does. Arrays are numpy; positions/effects (n, 2) float32, cell cubes in the
reference's strided layout (num_level, B, B[, 2]).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libnbfmm_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libnbfmm_refcpu.so")

_f = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_d = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_u8 = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_lib = None


def build():
    subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        c_int, c_float = ctypes.c_int, ctypes.c_float
        sig = {
            "orc_kernel_function": (None, [c_float] * 6 + [ctypes.POINTER(c_float)] * 2),
            "orc_base_dim": (c_int, [c_int]),
            "orc_predo": (None, [c_int, c_int, _f, _f, _f, _i, _i, _i, _f, _f]),
            "orc_p2p_naive": (None, [c_int, c_int, _f, _f, _i, _i, c_float, _f]),
            "orc_p2p_block": (None, [c_int, c_int, _f, _f, _i, _i, c_float, _f]),
            "orc_p2m": (None, [c_int, c_int, _f, _f, _i, _f, _f]),
            "orc_m2m": (None, [c_int, c_int, _f, _f]),
            "orc_m2l": (None, [c_int, c_int, _f, _f, c_float, _f]),
            "orc_l2l": (None, [c_int, c_int, _f]),
            "orc_l2p": (None, [c_int, c_int, _i, _f, _f]),
            "orc_postdo": (None, [c_int, _i, _f, _f]),
            "orc_solve": (c_int, [c_int, c_int, _f, c_float, c_int, _f, _f, _f]),
            "orc_solve_targets": (c_int, [c_int, c_int, _f, c_float, _f, _f, _i, c_int, _f]),
            "orc_prune": (c_int, [c_int, _f, _f, _f, _f]),
            "orc_display": (None, [c_int, c_int, c_int, c_float, _f, _f, _f, _u8]),
            "orc_display_threads": (None, [c_int, c_int, c_int, c_float, _f, _f, _f, _u8]),
            "orc_stars_update": (c_int, [c_int, c_int, _f, c_float, c_int, c_float, _f, _f, _f, _f]),
            "orc_direct_f64": (None, [c_int, _f, _f, ctypes.c_double, ctypes.c_void_p, c_int, _d]),
            "orc_direct_f32": (None, [c_int, _f, _f, ctypes.c_float, ctypes.c_void_p, c_int, _f]),
            "orc_p2p_pairs": (ctypes.c_longlong, [c_int, _i]),
            "orc_num_threads": (c_int, []),
            "orc_model_circle": (None, [c_int] + [c_float] * 6 + [c_int, _f, _f, _f, _f]),
            "orc_model_disk": (None, [c_int] + [c_float] * 6 + [c_int, c_int, _f, _f, _f, _f]),
            "orc_model_rectangle": (None, [c_int] + [c_float] * 5 + [_f, _f, _f, _f]),
            "orc_model_double_disk": (None, [c_int, c_int] + [c_float] * 11 + [c_int, _f, _f, _f, _f]),
            "orc_traj_fmm64": (ctypes.c_double, [c_int, c_int, _f, ctypes.c_double, ctypes.c_double, c_int, _d, _d, _d,
                                                 ctypes.c_void_p, ctypes.c_void_p, _d, ctypes.c_void_p]),
            "orc_traj_direct64_grad": (ctypes.c_double, [c_int, ctypes.c_double, ctypes.c_double, c_int, _d, _d, _d, _d,
                                                         _d, _d, _d]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def lim(limits):
    return f32(np.asarray(limits, dtype=np.float32).reshape(4))


def kernel_function(t, s, m, eps=0.1):
    ax, ay = ctypes.c_float(), ctypes.c_float()
    lib().orc_kernel_function(float(t[0]), float(t[1]), float(s[0]), float(s[1]), float(m), float(eps),
                              ctypes.byref(ax), ctypes.byref(ay))
    return np.float32(ax.value), np.float32(ay.value)


def predo(pos, w, num_level, limits):
    n = len(w)
    B = 1 << (num_level + 1)
    index = np.zeros((n, 2), np.int32)
    perm = np.zeros(n, np.int32)
    head = np.zeros(B * B + 1, np.int32)
    ps = np.zeros((n, 2), np.float32)
    ws = np.zeros(n, np.float32)
    lib().orc_predo(n, num_level, lim(limits), f32(pos), f32(w), index, perm, head, ps, ws)
    return dict(index=index, perm=perm, head=head, position=ps, weight=ws)


def p2p(pos, w, index, head, base_dim, eps=0.1, block=False):
    n = len(w)
    eff = np.zeros((n, 2), np.float32)
    fn = lib().orc_p2p_block if block else lib().orc_p2p_naive
    fn(n, base_dim, f32(pos), f32(w), i32(index), i32(head), float(eps), eff)
    return eff


def p2m(pos, w, head, base_dim):
    C = base_dim * base_dim
    cp = np.zeros((C, 2), np.float32)
    cw = np.zeros(C, np.float32)
    lib().orc_p2m(len(w), base_dim, f32(pos), f32(w), i32(head), cp, cw)
    return cp, cw


def m2m(cell_pos, cell_w, num_level, base_dim):
    cp, cw = f32(cell_pos).copy(), f32(cell_w).copy()
    lib().orc_m2m(num_level, base_dim, cp, cw)
    return cp, cw


def m2l(cell_pos, cell_w, num_level, base_dim, eps=0.1):
    ce = np.zeros_like(f32(cell_pos))
    lib().orc_m2l(num_level, base_dim, f32(cell_pos), f32(cell_w), float(eps), ce)
    return ce


def l2l(cell_eff, num_level, base_dim):
    ce = f32(cell_eff).copy()
    lib().orc_l2l(num_level, base_dim, ce)
    return ce


def l2p(eff, index, cell_eff, base_dim):
    e = f32(eff).copy()
    lib().orc_l2p(len(e), base_dim, i32(index), f32(cell_eff), e)
    return e


def postdo(perm, eff):
    out = np.zeros_like(f32(eff))
    lib().orc_postdo(len(perm), i32(perm), f32(eff), out)
    return out


def solve(pos, w, num_level, limits, eps=0.1, block=False):
    n = len(w)
    eff = np.zeros((n, 2), np.float32)
    if n:
        rc = lib().orc_solve(n, num_level, lim(limits), float(eps), int(block), f32(pos), f32(w), eff)
        assert rc == 0
    return eff


def solve_targets(pos, w, num_level, limits, eps, targets):
    targets = i32(targets)
    eff = np.zeros((len(targets), 2), np.float32)
    rc = lib().orc_solve_targets(len(w), num_level, lim(limits), float(eps), f32(pos), f32(w), targets,
                                 len(targets), eff)
    assert rc == 0
    return eff


def stars_update(cur, prev, w, num_level, limits, eps, tick_scaled, block=False):
    """One Stars::update; returns (n_new, cur, prev, w, acc) with arrays of the input length."""
    cur, prev, w = f32(cur).copy(), f32(prev).copy(), f32(w).copy()
    acc = np.zeros_like(cur)
    n = lib().orc_stars_update(len(w), num_level, lim(limits), float(eps), int(block), float(tick_scaled), cur, prev,
                               w, acc)
    assert n >= 0
    return n, cur, prev, w, acc


def direct_f64(pos, w, eps, targets=None):
    n = len(w)
    nt = n if targets is None else len(targets)
    eff = np.zeros((nt, 2), np.float64)
    if targets is None:
        lib().orc_direct_f64(n, f32(pos), f32(w), float(eps), None, 0, eff)
    else:
        t = i32(targets)
        lib().orc_direct_f64(n, f32(pos), f32(w), float(eps), t.ctypes.data_as(ctypes.c_void_p), nt, eff)
    return eff


def direct_f32(pos, w, eps, targets=None):
    """All-pairs direct sum in FP32 (kernelFunction's operations, sources in index order)."""
    n = len(w)
    nt = n if targets is None else len(targets)
    eff = np.zeros((nt, 2), np.float32)
    if targets is None:
        lib().orc_direct_f32(n, f32(pos), f32(w), float(eps), None, 0, eff)
    else:
        t = i32(targets)
        lib().orc_direct_f32(n, f32(pos), f32(w), float(eps), t.ctypes.data_as(ctypes.c_void_p), nt, eff)
    return eff


def p2p_pairs(head, base_dim):
    return int(lib().orc_p2p_pairs(base_dim, i32(head)))


def num_threads():
    return int(lib().orc_num_threads())


def ref_lib():
    """The reference's own kernelFunction/operators compiled for the CPU (oracle/_ref), or None."""
    if not os.path.exists(REF_LIB):
        return None
    L = ctypes.CDLL(REF_LIB)
    L.ref_kernel_function_batch.argtypes = [ctypes.c_int, _f, _f, _f, _f]
    L.ref_kernel_function_batch.restype = None
    L.ref_int2_less.argtypes = [ctypes.c_int] * 4
    L.ref_int2_less.restype = ctypes.c_int
    L.ref_int2_equal.argtypes = [ctypes.c_int] * 4
    L.ref_int2_equal.restype = ctypes.c_int
    L.ref_weighted_position.argtypes = [ctypes.c_int, _f, _f, _f]
    L.ref_weighted_position.restype = None
    L.ref_has_display.argtypes = []
    L.ref_has_display.restype = ctypes.c_int
    if L.ref_has_display():
        L.ref_display_device.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, _f, _f, _f, _u8]
        L.ref_display_device.restype = None
    L.ref_has_prune.restype = ctypes.c_int
    if L.ref_has_prune():
        L.ref_prune.argtypes = [ctypes.c_int, _f, _f, _f, _f]
        L.ref_prune.restype = ctypes.c_int
    L.ref_has_models.restype = ctypes.c_int
    if L.ref_has_models():
        f = ctypes.c_float
        for name, nf in (("circle_center", 6), ("circle_uniform_center", 6), ("disk", 5), ("disk_center", 6),
                         ("disk_static", 4), ("rectangle", 6)):
            fn = getattr(L, "ref_model_" + name)
            fn.argtypes = [ctypes.c_int] + [f] * nf + [_f, _f, _f, _f]
            fn.restype = None
    return L


def frame_bytes(width, height):
    return width * height * 3 // 2


def display(pos, w, width, height, size_scale, limits, threads=False):
    """Stars::display without its prune: one YUV 4:2:0 frame (uint8, width*height*3/2 bytes); threads=True
    splits the stars over the OpenMP threads (the same frame)."""
    pos = f32(pos).reshape(-1)
    board = np.empty(frame_bytes(width, height), np.uint8)
    fn = lib().orc_display_threads if threads else lib().orc_display
    fn(len(pos) // 2, width, height, float(size_scale), lim(limits), pos, f32(w), board)
    return board


def ref_display(pos, w, width, height, size_scale, limits, pad_rows=8):
    """The reference's displayDevice compiled for the CPU (oracle/_ref), on a frame cleared as
    Stars::display clears it; returns (frame, bytes written before it, bytes written after it), or None."""
    L = ref_lib()
    if L is None or not L.ref_has_display():
        return None
    pad = pad_rows * width + 8
    fb = frame_bytes(width, height)
    buf = np.full(pad + fb + pad, 7, np.uint8)
    buf[pad:pad + width * height] = 0
    buf[pad + width * height:pad + fb] = 128
    pos = f32(pos).reshape(-1)
    view = buf[pad:]
    L.ref_display_device(len(pos) // 2, width, height, float(size_scale), lim(limits), pos, f32(w), view)
    return buf[pad:pad + fb].copy(), int(np.count_nonzero(buf[:pad] != 7)), int(np.count_nonzero(buf[pad + fb:] != 7))


def ref_prune(cur, prev, w, limits):
    """The reference's Stars::prune (pruneDevice + thrust::sort_by_key on thrust's host system, oracle/_ref) in
    place; returns the number of survivors, or None when oracle/_ref was not built."""
    L = ref_lib()
    if L is None or not L.ref_has_prune():
        return None
    return L.ref_prune(len(w), lim(limits), cur.reshape(-1), prev.reshape(-1), w)


def ref_model(kind, n, u, **p):
    """The reference's generate*Device kernel of one model (oracle/_ref) on draws u (n x 3): (cur, prev, w), or
    None when oracle/_ref was not built. The double disks are two disks plus host-side offsets: not here."""
    L = ref_lib()
    if L is None or not L.ref_has_models():
        return None
    cur = np.zeros((n, 2), np.float32)
    prev = np.zeros((n, 2), np.float32)
    w = np.zeros(n, np.float32)
    uu = f32(u).reshape(-1)
    c = p["center"]
    if kind in ("circle_center", "circle_uniform_center"):
        args = (*c, p["radius"], p["weight"], p["center_weight"], p["tick"])
    elif kind == "disk":
        args = (*c, p["radius"], p["weight"], p["tick"])
    elif kind == "disk_center":
        args = (*c, p["radius"], p["weight"], p["center_weight"], p["tick"])
    elif kind == "disk_static":
        args = (*c, p["radius"], p["weight"])
    elif kind == "rectangle":
        args = (*c, p["width"], p["height"], p["max_weight"], p["tick"])
    else:
        raise ValueError(kind)
    getattr(L, "ref_model_" + kind)(n, *[float(a) for a in args], uu, cur.reshape(-1), prev.reshape(-1), w)
    return cur, prev, w


def prune(cur, prev, w, limits):
    """Stars::prune: stable partition in place; returns the number of survivors."""
    return lib().orc_prune(len(w), lim(limits), cur.reshape(-1), prev.reshape(-1), w)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def traj_fmm64(x0, v0, m, num_level, limits, eps, tau, steps, target, keys=None):
    """FP64 loss of the approximate method's trajectory; returns (loss, keys used (steps, n))."""
    n = len(m)
    keys_out = np.zeros((steps, n), np.int32) if keys is None else None
    kin = None if keys is None else i32(keys).ctypes.data_as(ctypes.c_void_p)
    kout = None if keys_out is None else keys_out.ctypes.data_as(ctypes.c_void_p)
    loss = lib().orc_traj_fmm64(n, num_level, lim(limits), float(eps), float(tau), steps, f64(x0).reshape(-1),
                                f64(v0).reshape(-1), f64(m), kin, kout, f64(target).reshape(-1), None)
    return loss, (keys if keys is not None else keys_out)


def traj_direct64_grad(x0, v0, m, eps, tau, steps, target):
    """(loss, dL/dx0, dL/dv0, dL/dm) of the exact all-pairs FP64 dynamics."""
    n = len(m)
    gx, gv, gm = np.zeros(2 * n), np.zeros(2 * n), np.zeros(n)
    loss = lib().orc_traj_direct64_grad(n, float(eps), float(tau), steps, f64(x0).reshape(-1), f64(v0).reshape(-1),
                                        f64(m), f64(target).reshape(-1), gx, gv, gm)
    return loss, gx.reshape(n, 2), gv.reshape(n, 2), gm


def model(kind, n, u, **p):
    """CPU restatement of one reference model for draws u (n x 3, float32); returns (cur, prev, w)."""
    total = n if kind not in ("double_disk", "double_disk_center") else p["n1"] + p["n2"]
    cur = np.zeros((total, 2), np.float32)
    prev = np.zeros((total, 2), np.float32)
    w = np.zeros(total, np.float32)
    uu = f32(u).reshape(-1)
    L = lib()
    if kind in ("circle_center", "circle_uniform_center"):
        L.orc_model_circle(n, *p["center"], p["radius"], p["weight"], p["center_weight"], p["tick"],
                           int(kind == "circle_uniform_center"), uu, cur, prev, w)
    elif kind in ("disk", "disk_center", "disk_static"):
        L.orc_model_disk(n, *p["center"], p["radius"], p["weight"], p.get("center_weight", 0.0), p["tick"],
                         int(kind == "disk_center"), int(kind == "disk_static"), uu, cur, prev, w)
    elif kind == "rectangle":
        L.orc_model_rectangle(n, *p["center"], p["width"], p["height"], p["max_weight"], uu, cur, prev, w)
    else:
        center = kind == "double_disk_center"
        L.orc_model_double_disk(p["n1"], p["n2"], *p["center1"], *p["center2"], p["radius1"], p["radius2"],
                                p["weight"], p.get("center_weight1", 0.0), p.get("center_weight2", 0.0),
                                p["eccentricity"], p["tick"], int(center), uu, cur, prev, w)
    return cur, prev, w
