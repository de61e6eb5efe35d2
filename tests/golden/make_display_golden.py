"""Regenerates tests/golden/ref_display_frames.npz: frames drawn by the reference's own displayDevice.

Builds oracle/_ref (oracle/build_ref.sh compiles source/nbfmm/display/stars/display.cu:29-214 for the CPU from
the reference sources), draws seeded star fields on frames cleared as Stars::display clears them
(display.cu:220-221) and stores inputs and frames. The stars include the edge cases of the raster: every size
0..9, the first and last columns and rows, and stars one row below the display limits, which the reference
accepts as row `height` (display.cu:53). The reference writes before the frame for stars on its top rows; the
frame buffer is padded so those writes land outside it, and the frame itself is what is stored.
Needs the reference sources (NBFMM_REFERENCE, default /root/reference); the committed .npz is what the tests read.
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "ref_display_frames.npz")

# (width, height, size_scale, display limits, number of random stars)
CASES = [
    (96, 64, 1.0, (-1.5, -1.0, 1.5, 1.0), 600),
    (33, 17, 0.5, (-2.0, -1.0, 2.0, 1.0), 120),
    (160, 90, 0.25, (-8.0, -4.5, 8.0, 4.5), 5000),
]


def stars_for(rng, width, height, size_scale, limits, count):
    x0, y0, x1, y1 = limits
    uw, uh = (x1 - x0) / width, (y1 - y0) / height
    pos = [np.stack([rng.uniform(x0 - 0.1 * (x1 - x0), x1 + 0.1 * (x1 - x0), count),
                     rng.uniform(y0 - 0.1 * (y1 - y0), y1 + 0.1 * (y1 - y0), count)], 1)]
    size = [rng.integers(0, 10, count)]
    # Edge pixels: columns 0..4 and width-5..width-1 against rows 0..4, height-5..height (row `height` lies
    # half a row below y_min), every size.
    cols = list(range(5)) + list(range(width - 5, width))
    rows = list(range(5)) + list(range(height - 5, height + 1))
    ex, ey = np.meshgrid(cols, rows)
    ex, ey = ex.ravel(), ey.ravel()
    pos.append(np.stack([x0 + (ex + 0.5) * uw, y1 - (ey + 0.5) * uh], 1))
    size.append(np.arange(len(ex)) % 10)
    pos = np.concatenate(pos).astype(np.float32)
    size = np.concatenate(size)
    w = ((size + 0.5) * size_scale) ** 2
    return pos, w.astype(np.float32)


def main() -> int:
    subprocess.check_call(["sh", os.path.join(ROOT, "oracle", "build_ref.sh")])
    sys.path.insert(0, ROOT)
    from oracle import oracle as O

    L = O.ref_lib()
    if L is None or not L.ref_has_display():
        print("make_display_golden: the reference's displayDevice was not built", file=sys.stderr)
        return 1
    rng = np.random.default_rng(20160611)
    arrays = {}
    for k, (width, height, size_scale, limits, count) in enumerate(CASES):
        pos, w = stars_for(rng, width, height, size_scale, limits, count)
        frame, before, after = O.ref_display(pos, w, width, height, size_scale, limits)
        arrays[f"case{k}_pos"] = pos
        arrays[f"case{k}_w"] = w
        arrays[f"case{k}_params"] = np.array([width, height], np.int32)
        arrays[f"case{k}_fparams"] = np.array([size_scale, *limits], np.float32)
        arrays[f"case{k}_frame"] = frame
        arrays[f"case{k}_outside_writes"] = np.array([before, after], np.int32)
    arrays["num_cases"] = np.array(len(CASES), np.int32)
    np.savez_compressed(OUT, **arrays)
    print(f"make_display_golden: wrote {OUT} ({len(CASES)} frames)")
    return 0


if __name__ == "__main__":
    sys.exit(main())
