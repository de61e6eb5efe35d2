"""Regenerates tests/golden/ref_fixture_l3_n250.npz from the reference's test fixture.

Compiles make_golden.cpp against the reference headers (kernelFunction and the vector operators are the
reference's own code), runs it, and packs the raw arrays into one .npz. Needs the reference sources
(NBFMM_REFERENCE, default /root/reference) and g++; the committed .npz is what the tests read.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "ref_fixture_l3_n250.npz")


def main() -> int:
    ref = os.environ.get("NBFMM_REFERENCE", "/root/reference")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    if not os.path.isfile(os.path.join(ref, "include/nbfmm/core/kernel_function.hpp")):
        print(f"make_golden: reference sources not found at {ref}", file=sys.stderr)
        return 1
    with tempfile.TemporaryDirectory() as tmp:
        inc = os.path.join(tmp, "include", "nbfmm")
        os.makedirs(inc)
        with open(os.path.join(inc, "config.hpp"), "w") as f:
            f.write("#pragma once\n")
        exe = os.path.join(tmp, "make_golden")
        subprocess.check_call([
            "g++", "-std=c++14", "-O2", "-ffp-contract=off", "-Wno-deprecated-declarations",
            "-I" + os.path.join(tmp, "include"), "-I" + os.path.join(ref, "include"), "-I" + os.path.join(cuda, "include"),
            os.path.join(HERE, "make_golden.cpp"), "-o", exe,
        ])
        outdir = os.path.join(tmp, "out")
        os.makedirs(outdir)
        subprocess.check_call([exe, outdir])
        arrays = {}
        with open(os.path.join(outdir, "manifest.txt")) as f:
            for line in f:
                name, dtype, count = line.split()
                arrays[name] = np.fromfile(os.path.join(outdir, name + ".bin"), dtype="<" + dtype, count=int(count))
    np.savez(OUT, **arrays)
    print(f"make_golden: wrote {OUT} ({len(arrays)} arrays)")
    return 0


if __name__ == "__main__":
    sys.exit(main())
