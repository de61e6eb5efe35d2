"""The reference's launcher scripts (main/script/circle.py, disk.py, double_disk.py, rectangle.py) for
nbfmm_main: each runs the movie program on one preset model.

    python -m nbfmm_gb300.launch <circle|disk|double_disk|rectangle> <output.y4m> [--seconds S] [--stars N]

The presets are the reference scripts' values (1024 x 768 at 60 fps for 10 s, FMM level 4, a 16 x 12 domain,
gravitational constant 1, size scale 1); --seconds and --stars shorten a run.
"""
import argparse
import os
import subprocess
import sys

from . import build

COMMON = dict(width=1024, height=768, fps=60, num_second=10, fmm_level=4, pos_width=16, pos_height=12,
              grav_const=1, size_scale=1)


def preset(model: str, num_star=None, num_second=None):
    """argv (after the program name and output file) of one reference script."""
    c = dict(COMMON)
    if num_second is not None:
        c["num_second"] = num_second
    pw, ph = c["pos_width"], c["pos_height"]
    if model == "circle":
        c.update(num_star=256, display_scale=0.5)
        n = num_star or c["num_star"]
        params = ["circle", min(pw, ph) * c["display_scale"] / 8, 1, n * 64]
    elif model == "disk":
        c.update(num_star=10000, display_scale=0.5)
        params = ["disk", min(pw, ph) * c["display_scale"] / 8, 1]
    elif model == "double_disk":
        c.update(num_star=10000, display_scale=0.8)
        p1, p2 = 5, 3
        radius = min(pw, ph) * c["display_scale"] / 16
        params = ["double-disk", p1, p2, radius * p1 / (p1 + p2), radius * p2 / (p1 + p2), 1, 1]
    elif model == "rectangle":
        c.update(num_star=10000, display_scale=0.8)
        params = ["rectangle", pw * c["display_scale"], ph * c["display_scale"], 16]
    else:
        raise ValueError(f"unknown preset {model}")
    if num_star is not None:
        c["num_star"] = num_star
    args = [c["width"], c["height"], c["fps"], c["num_second"], c["fmm_level"], c["num_star"], pw, ph,
            c["display_scale"], c["grav_const"], c["size_scale"]] + params
    return [str(a) for a in args]


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("model", choices=["circle", "disk", "double_disk", "rectangle"])
    ap.add_argument("output")
    ap.add_argument("--seconds", type=int, default=None)
    ap.add_argument("--stars", type=int, default=None)
    a = ap.parse_args(argv)
    exe = build.program("nbfmm_main")
    if not os.path.exists(exe):
        build.build()
    return subprocess.call([exe, a.output] + preset(a.model, a.stars, a.seconds))


if __name__ == "__main__":
    sys.exit(main())
