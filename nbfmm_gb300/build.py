"""Builds libnbfmm_gb300.so in-tree from nbfmm_gb300/csrc/*.cu for sm_103a (GB300), and the command-line
programs nbfmm_gb300/bin/nbfmm_main and nbfmm_demo from nbfmm_gb300/cli/*.cpp.

Each translation unit is compiled in parallel with nvcc, then linked into one shared library with the CUDA
runtime linked statically. The programs are plain C++ on the library's C ABI. `python -m nbfmm_gb300.build`
or `build()` from Python.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnbfmm_gb300.so")
CLI = os.path.join(HERE, "cli")
BIN = os.path.join(HERE, "bin")
INCLUDE = os.path.join(HERE, "..", "include")
PROGRAMS = {"nbfmm_main": "main.cpp", "nbfmm_demo": "demo.cpp"}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "-Xcompiler", "-ffp-contract=off",  # host arithmetic rounds the same on x86 and Arm
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, extra_flags=None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "nbfmm_gb300.h"))
    flags = NVCC_FLAGS + list(extra_flags or [])
    jobs = []
    objs = []
    for src in sources():
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([nvcc()] + ARCH + flags + ["-c", src, "-o", obj])
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda cmd: subprocess.run(cmd, capture_output=True, text=True), jobs))
    for cmd, r in zip(jobs, results):
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {cmd[-3]}")
    if _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-Xlinker", "-z", "-Xlinker", "defs", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("link of libnbfmm_gb300.so failed")
    build_programs(verbose)
    return LIB


def program(name: str) -> str:
    return os.path.join(BIN, name)


def build_programs(verbose: bool = False):
    """The command-line programs, linked against the in-tree library (rpath $ORIGIN/..)."""
    os.makedirs(BIN, exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    for name, src in PROGRAMS.items():
        out, src = program(name), os.path.join(CLI, src)
        if not _stale(out, [src, LIB, os.path.join(INCLUDE, "nbfmm_gb300.h")]):
            continue
        cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-Wall", "-I" + INCLUDE, src, "-o", out,
               "-L" + HERE, "-lnbfmm_gb300", "-Wl,-rpath,$ORIGIN/.."]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"build of {name} failed")


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
