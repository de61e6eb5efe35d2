"""CPU: the C-ABI library loads, exports every entry point include/nbfmm_gb300.h declares, and rejects the
arguments the reference asserts on -- all without touching a GPU."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "nbfmm_gb300.h")


@pytest.fixture(scope="module")
def lib():
    from nbfmm_gb300 import _lib, build

    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    return _lib.load()


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nbfmm_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ["nbfmm_solver_create", "nbfmm_solver_solve", "nbfmm_solver_destroy", "nbfmm_stars_update"]:
        assert required in names


def test_library_exports_every_declared_symbol(lib):
    from nbfmm_gb300 import _lib

    names = declared_functions()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(_lib.SIGNATURES), "ctypes signatures and header disagree"


def test_version(lib):
    assert lib.nbfmm_version() == 1


def _limits(*v):
    return (ctypes.c_float * 4)(*v)


@pytest.mark.parametrize("level,maxn,limits", [
    (-1, 10, (0, 0, 1, 1)),
    (11, 10, (0, 0, 1, 1)),
    (3, 0, (0, 0, 1, 1)),
    (3, 10, (1, 0, 0, 1)),
    (3, 10, (0, 1, 1, 1)),
    (3, 10, (0, 0, float("nan"), 1)),
])
def test_create_rejects_invalid_arguments(lib, level, maxn, limits):
    h = ctypes.c_void_p()
    rc = lib.nbfmm_solver_create(level, maxn, _limits(*limits), ctypes.byref(h))
    assert rc == 1 and not h.value
    assert lib.nbfmm_last_error()


def test_null_handles_are_errors_not_crashes(lib):
    assert lib.nbfmm_solver_solve(None, 1, None, None, None, None) == 1
    assert lib.nbfmm_solver_destroy(None) == 0
    assert lib.nbfmm_stars_update(None, 1, None) == 1
    assert lib.nbfmm_stars_destroy(None) == 0
    assert b"null" in lib.nbfmm_last_error()


def test_stars_create_rejects_bad_tick(lib):
    h = ctypes.c_void_p()
    assert lib.nbfmm_stars_create(3, 10, 0.0, 1.0, _limits(0, 0, 1, 1), ctypes.byref(h)) == 1
    assert lib.nbfmm_stars_create(3, 10, 1e-3, -1.0, _limits(0, 0, 1, 1), ctypes.byref(h)) == 1
    assert lib.nbfmm_stars_create(3, -1, 1e-3, 1.0, _limits(0, 0, 1, 1), ctypes.byref(h)) == 1


def test_python_mirror_raises_without_the_library(tmp_path):
    from nbfmm_gb300 import _lib

    saved = _lib._lib
    try:
        _lib._lib = None
        with pytest.raises(RuntimeError, match="no CPU fallback"):
            _lib.load(str(tmp_path / "missing.so"))
    finally:
        _lib._lib = saved


def build_facade_check(out_path):
    """Compiles tests/cxx/facade_check.cpp against the C++ facade and links it to the library."""
    import shutil
    import subprocess

    from nbfmm_gb300 import build

    cxx = shutil.which(os.environ.get("CXX", "g++"))
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    if cxx is None or not os.path.exists(os.path.join(cuda_inc, "vector_types.h")):
        pytest.skip("needs g++ and the CUDA headers")
    if not os.path.exists(build.LIB):
        build.build()
    src = os.path.join(ROOT, "tests", "cxx", "facade_check.cpp")
    cmd = [cxx, "-std=c++17", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"), "-I" + cuda_inc, src,
           "-o", out_path, "-L" + os.path.dirname(build.LIB), "-lnbfmm_gb300",
           "-Wl,-rpath," + os.path.dirname(build.LIB)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out_path


def test_cxx_facade_compiles_and_links(tmp_path):
    """include/nbfmm_gb300.hpp: reference-style code (Solver, Stars.initialize with a model, update, display)
    compiles against the facade and links to the library."""
    assert os.path.exists(build_facade_check(str(tmp_path / "facade_check")))
