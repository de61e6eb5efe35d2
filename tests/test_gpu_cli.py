"""GPU: the movie program (main/main.cu) and the demo (main/demo.cu) on the engine.

nbfmm_main's printed lines are checked against the reference's formats, its .y4m against the same run made
through the Python API (Stars, model, Movie), and every model's command line once."""
import os
import re
import signal
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def programs(engine):
    from nbfmm_gb300 import build

    build.build_programs()
    return build.program("nbfmm_main"), build.program("nbfmm_demo")


def run(exe, *args):
    # Bytes decoded here: text mode would turn the progress bar's carriage return into a newline.
    r = subprocess.run([exe, *map(str, args)], capture_output=True, timeout=600)
    return subprocess.CompletedProcess(r.args, r.returncode, r.stdout.decode(), r.stderr.decode())


def f32(v):
    return float(np.float32(v))


def test_disk_movie_matches_python_api(engine, programs, tmp_path):
    import torch
    from nbfmm_gb300 import model

    exe = programs[0]
    width, height, fps, seconds, level, n = 160, 120, 8, 2, 4, 3000
    pw, ph, ds, g, ss, radius, weight = 16.0, 12.0, 0.5, 1.0, 1.0, 0.75, 1.0
    out = os.path.join(str(tmp_path), "cli.y4m")
    r = run(exe, out, width, height, fps, seconds, level, n, pw, ph, ds, g, ss, "disk", radius, weight)
    assert r.returncode == 0, r.stderr
    tick = f32(0.05 / fps)
    frames = seconds * fps
    lines = r.stdout.split("\n")
    assert lines[0] == "NBFMM 1.2.0" and lines[1] == ""
    assert lines[2] == f"{width} x {height} pixel, {fps} fps, {seconds} sec / {frames} frame"
    assert lines[3] == f"{level} FMM level, {n} stars, tick = {tick:.6f}, grav const = {g:.2f}, scale size = {ss:.2f}"
    assert lines[4] == f"position size = {pw:.2f} x {ph:.2f}, display scale = {ds:.2f}"
    assert lines[5] == ("position range = [-8.00, 8.00] x [-6.00, 6.00], "
                        "display range = [-4.00, 4.00] x [-3.00, 3.00]")
    assert lines[7] == f"Model Disk: radius = {radius:.2f}, weight = {weight:.2f}"
    progress, bar = 0, ""
    for j in range(1, frames):  # main.cu:252-255
        if 100 * j > progress * frames:
            progress += 1
            bar += ">"
    assert lines[9] == "=" * 100 + "\r" + bar and lines[10:] == ["", ""]

    pos_lim = (-8.0, -6.0, 8.0, 6.0)
    disp_lim = (-4.0, -3.0, 4.0, 3.0)
    st = engine.Stars(level, n, width, height, fps, tick, g, ss, pos_lim, disp_lim)
    st.initialize(model.generateDisk, n, (0.0, 0.0), radius, weight)
    ref = os.path.join(str(tmp_path), "api.y4m")
    with engine.Movie(st, ref) as mv:
        mv.frame()
        for _ in range(1, frames):
            st.update(1)
            mv.frame()
    torch.cuda.synchronize()
    a, b = open(out, "rb").read(), open(ref, "rb").read()
    header = f"YUV4MPEG2 W{width} H{height} F{fps}:1 Ip A1:1 C420\n".encode()
    assert a.startswith(header) and len(a) == len(header) + frames * (6 + width * height * 3 // 2)
    assert a == b


@pytest.mark.parametrize("model_args", [
    ["circle", 0.75, 1, 16384],
    ["circle-uniform", 0.75, 1, 16384],
    ["disk-center", 0.75, 1, 5000],
    ["disk-static", 0.75, 1],
    ["double-disk", 5, 3, 0.375, 0.225, 1, 1],
    ["double-disk-center", 5, 3, 0.375, 0.225, 1, 500, 300, 1],
    ["rectangle", 12.8, 9.6, 16],
])
def test_every_model_runs(programs, tmp_path, model_args):
    out = os.path.join(str(tmp_path), "m.y4m")
    r = run(programs[0], out, 96, 64, 5, 1, 4, 2000, 16, 12, 0.8, 1, 1, *model_args)
    assert r.returncode == 0, r.stderr
    data = open(out, "rb").read()
    header = b"YUV4MPEG2 W96 H64 F5:1 Ip A1:1 C420\n"
    assert data.startswith(header) and len(data) == len(header) + 5 * (6 + 96 * 64 * 3 // 2)
    frame0 = np.frombuffer(data[len(header) + 6:len(header) + 6 + 96 * 64], np.uint8)
    assert np.count_nonzero(frame0) > 0  # stars are on screen


def test_model_usage_and_unknown_model(programs, tmp_path):
    out = os.path.join(str(tmp_path), "u.y4m")
    base = [out, 96, 64, 5, 1, 4, 2000, 16, 12, 0.8, 1, 1]
    r = run(programs[0], *base, "disk", 0.75)
    assert r.returncode == -signal.SIGABRT and "... disk <radius> <weight>" in r.stdout
    r = run(programs[0], *base, "double-disk-center", 5, 3, 0.375, 0.225, 1, 500, 300)
    assert r.returncode == -signal.SIGABRT and "double-disk-center <proportion 1>" in r.stdout
    r = run(programs[0], *base, "spiral", 1)
    assert r.returncode == -signal.SIGABRT and "Unknown model spiral." in r.stdout


def test_demo(programs, orc):
    r = run(programs[1])
    assert r.returncode == 0, r.stderr
    lines = r.stdout.split("\n")
    assert lines[0] == "NBFMM 1.2.0 demo"
    rows = [ln for ln in lines if ln.startswith("(")]
    assert len(rows) == 250
    num = re.compile(r"-?\d+(?:\.\d+)?")
    vals = np.array([[float(v) for v in num.findall(ln)] for ln in rows])
    assert vals.shape == (250, 9)
    x, y, w, ix, iy = vals[:, 0], vals[:, 1], vals[:, 2], vals[:, 3], vals[:, 4]
    assert np.all((0 <= x) & (x <= 8) & (-1 <= y) & (y <= 3) & (w > 0))
    # Leaf cells of a depth-4 tree (32 x 32 over [0, 8] x [-1, 3]); the printed positions are rounded.
    away = (np.abs(x / 0.25 - np.round(x / 0.25)) > 1e-3) & (np.abs((y + 1) / 0.125 - np.round((y + 1) / 0.125)) > 1e-3)
    assert np.all(ix[away] == np.floor(x[away] / 0.25)) and np.all(iy[away] == np.floor((y[away] + 1) / 0.125))
    cpu, fmm = vals[:, 5:7], vals[:, 7:9]
    rel = np.linalg.norm(cpu - fmm, axis=1) / np.linalg.norm(cpu, axis=1).max()
    assert np.median(rel) < 0.05  # the method's own error at depth 4 with monopoles


def test_cxx_facade_runs_like_the_python_api(engine, tmp_path):
    """Reference-style C++ (include/nbfmm_gb300.hpp) gives the numbers the Python API gives for the same run."""
    import sys

    import torch
    from nbfmm_gb300 import model

    sys.path.insert(0, os.path.dirname(__file__))
    from test_abi import build_facade_check

    exe = build_facade_check(str(tmp_path / "facade_check"))
    r = run(exe)
    assert r.returncode == 0, r.stderr
    esum, n_after, lit = r.stdout.split()
    n = 4096
    st = engine.Stars(4, n, 64, 48, 30, 1e-3, 1.0, 0.05, (-2, -2, 2, 2), (-1.5, -1.5, 1.5, 1.5))
    st.initialize(model.generateDiskCenter, n, (0.0, 0.0), 1.0, 1e-4, 5.0)
    solver = engine.Solver(4, n, (-2, -2, 2, 2))
    eff = torch.empty(n, 2, device="cuda")
    solver.solve(n, st.gpuptr_position_cur_, st.gpuptr_weight_, eff)
    st.update(5)
    board = torch.empty(engine.frame_bytes(64, 48), dtype=torch.uint8, device="cuda")
    st.display(board)
    torch.cuda.synchronize()
    e = eff.cpu().numpy().astype(np.float64).ravel()
    assert abs(float(esum) - e.sum()) <= 1e-9 * np.abs(e).sum()
    assert int(n_after) == st.num_star_
    assert int(lit) == int((board[:64 * 48] == 255).sum())
