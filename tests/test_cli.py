"""The command-line programs' argument handling (main/main.cu:25-37 and the per-model checks), which runs before
any GPU call: the reference's usage lines and abort()."""
import os
import signal
import subprocess

import pytest


@pytest.fixture(scope="module")
def main_program():
    from nbfmm_gb300 import build

    exe = build.program("nbfmm_main")
    if not os.path.exists(exe):
        if os.path.exists(build.LIB):
            build.build_programs()
        else:
            build.build()
    return exe


def run(exe, *args):
    return subprocess.run([exe, *map(str, args)], capture_output=True, text=True, timeout=60)


def test_usage_without_arguments(main_program):
    r = run(main_program)
    assert r.returncode == -signal.SIGABRT
    assert r.stdout == (
        "NBFMM 1.2.0\n\n"
        f"Usage: {main_program} <output file> <width> <height> <fps> <time (second)> <FMM level> <number of stars>"
        " <position width> <position height> <display scale> <grav_const> <size_scale> <model> [model parameters]"
        " ...\n\n")


def test_usage_with_twelve_arguments(main_program):
    r = run(main_program, "out.y4m", 64, 48, 10, 1, 3, 100, 16, 12, 0.5, 1, 1)
    assert r.returncode == -signal.SIGABRT and "Usage:" in r.stdout


def test_launch_presets_match_reference_scripts():
    from nbfmm_gb300 import launch

    assert launch.preset("circle")[:11] == "1024 768 60 10 4 256 16 12 0.5 1 1".split()
    assert launch.preset("circle")[11:] == ["circle", "0.75", "1", "16384"]
    assert launch.preset("disk")[11:] == ["disk", "0.75", "1"]
    dd = launch.preset("double_disk")
    assert dd[5] == "10000" and dd[8] == "0.8" and dd[11:14] == ["double-disk", "5", "3"]
    assert abs(float(dd[14]) - 0.375) < 1e-12 and abs(float(dd[15]) - 0.225) < 1e-12
    assert launch.preset("rectangle")[11:] == ["rectangle", "12.8", "9.600000000000001", "16"]
    assert launch.preset("disk", num_star=500, num_second=1)[3:6] == ["1", "4", "500"]
