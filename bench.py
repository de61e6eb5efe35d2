"""Throughput of the nbfmm hot path on GB300: Stars::update steps (solve + Stormer-Verlet + prune).

Default workload: two colliding disks, N = 16,777,216, depth 9 (num_level 8, 512 x 512 leaf cells), eps 5e-4,
dt 5e-5 (seeded synthetic particles). One step = one reference Stars::update (update.cu:47-55). Prints one JSON
line (metric particle-steps/s). `--impl reference` times the reference's algorithm on the host cores instead
(the oracle's CPU restatement; the reference itself has no CPU path), on a bounded sample of the workload.

Multi-GPU (torchrun): every rank steps its own replica of the workload (the path has no exchange step);
value = all particles stepped on all ranks / max-over-ranks time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

FLOP_PER_PAIR = 15  # 2 sub, 3 for r^2, 1 sqrt, 1 for r*r^2 (+eps fused: 2), 1 rcp, 1 mul by m, 4 for 2 FMAs
SMS, FP32_LANES, MUFU_LANES = 152, 128, 16
# Transcendental-unit operations per pair in p2p_kernel's packed passes: the square root always, plus the
# hardware reciprocal on the sources that do not take an FMA-pipe form -- 10 of every 16 beside the Newton
# iteration (NBFMM_P2P_NEWTON_MASK = 0x9249), 7 of 16 beside the degree-2 reciprocal series
# (NBFMM_P2P_SERIES_MASK = 0x5AB5) in the work items away from the leaf grid's edges, when
# (2 sqrt(2) cell)^3 / eps is at most SERIES_MAX_V: the rule of p2p.cu's series_degree.
P2P_MUFU_PER_PAIR = 1 + 10 / 16
P2P_MUFU_PER_PAIR_SERIES = {2: 1 + 7 / 16}
SERIES_MAX_V = 0.0062


def series_degree(sysm, arithmetic):
    b = 2 ** (sysm.num_level + 1)
    lim = sysm.limits
    cell = max(float(np.float32(lim[2] - lim[0]) / np.float32(b)), float(np.float32(lim[3] - lim[1]) / np.float32(b)))
    if arithmetic != "fast" or not sysm.epsilon > 0:
        return 0
    return 2 if (2 * np.sqrt(2) * cell) ** 3 / sysm.epsilon <= SERIES_MAX_V else 0


WINDOW_CELLS = 32  # side of the CPU sample window, in leaf cells
# DRAM bytes (read + write) of one P2P launch per particle: ncu's dram__bytes_read.sum (134.96 MB) and
# dram__bytes_write.sum (73.99 MB) for one p2p_kernel<kVerlet> launch of the two-disk step at N = 4,194,304,
# depth 8 (the same particles per leaf cell as the 16.8M workload); traffic grows with the particles of a launch
# (it equals the algorithmic 48 B/particle), so a full launch is this times N.
P2P_DRAM_BYTES_PER_PARTICLE = (134.964992e6 + 73.988864e6) / 4194304


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: the workload's own step count; 200 for the frame modes)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="two_disks_16m")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the side measurements of the default run (batched, adjoint, exact, CPU direct sums)")
    ap.add_argument("--arithmetic", default="fast", choices=["fast", "exact"],
                    help="near-field arithmetic of the engine (exact: correctly rounded, the oracle's rounding)")
    return ap.parse_args()


def workload_name(sysm):
    depth = sysm.num_level + 1
    b = 1 << depth
    return (f"{sysm.name}: N={sysm.n:,}, depth {depth} ({b}x{b} leaf cells), eps {sysm.epsilon:g}, "
            f"dt {sysm.dt:g}, G {sysm.grav_const:g}, limits {list(sysm.limits)}")


# ---- CPU side (oracle = the reference's algorithm restated on the host) --------------------------------------

def window_sample(sysm):
    """A WINDOW_CELLS x WINDOW_CELLS leaf-cell window of the system at full density: same cell size and
    particles per cell as the full workload, so the cost per particle-step matches it."""
    b = 1 << (sysm.num_level + 1)
    cell = (sysm.limits[2] - sysm.limits[0]) / b
    side = WINDOW_CELLS * cell
    # centre the window on the disk material: the median position of a seeded subset
    rng = np.random.default_rng(0)
    sub = sysm.position[rng.choice(sysm.n, min(sysm.n, 4096), replace=False)]
    cx, cy = float(np.median(sub[:, 0])), float(np.median(sub[:, 1]))
    if sysm.name == "two_disks":
        cx, cy = -0.35, 0.0  # on the ring of the left disk, away from its centre mass
    lim = (cx - side / 2, cy - side / 2, cx + side / 2, cy + side / 2)
    p = sysm.position
    m = (p[:, 0] >= lim[0]) & (p[:, 0] < lim[2]) & (p[:, 1] >= lim[1]) & (p[:, 1] < lim[3])
    level = int(np.log2(WINDOW_CELLS)) - 1
    prev = sysm.previous()
    return p[m].copy(), prev[m].copy(), sysm.weight[m].copy(), lim, level


def cpu_steps(sysm, steps, budget_s=None):
    """Steps the window sample with the oracle's Stars::update; returns (particle-steps/s, threads, n, steps)."""
    from oracle import oracle

    cur, prev, w, lim, level = window_sample(sysm)
    n = len(w)
    tick = sysm.tick()
    done, t0 = 0, time.perf_counter()
    while True:
        k, cur[:n], prev[:n], w[:n], _ = oracle.stars_update(cur[:n], prev[:n], w[:n], level, lim, sysm.epsilon, tick)
        done += n
        n = k
        steps -= 1
        el = time.perf_counter() - t0
        if steps <= 0 or (budget_s is not None and el >= budget_s):
            break
    return done / el, oracle.num_threads(), len(w), el


def cpu_sample_text(sysm, n, steps):
    return (f"{steps} oracle Stars::update steps of a {WINDOW_CELLS}x{WINDOW_CELLS}-leaf-cell window of the "
            f"workload ({n:,} particles at full density, same cell size, num_level "
            f"{int(np.log2(WINDOW_CELLS)) - 1}), OpenMP over the host cores")


def run_reference_arm(args, sysm, rank):
    if rank != 0:
        return
    from oracle import oracle

    oracle.lib()
    cur, prev, w, lim, level = window_sample(sysm)
    n0 = len(w)
    tick = sysm.tick()
    n = n0
    for _ in range(args.warmup):
        # the new count is bound last: the slices on the left take the count the step started with
        k, cur[:n], prev[:n], w[:n], _ = oracle.stars_update(cur[:n], prev[:n], w[:n], level, lim, sysm.epsilon, tick)
        n = k
    done, t0 = 0, time.perf_counter()
    for _ in range(args.steps):
        k, cur[:n], prev[:n], w[:n], _ = oracle.stars_update(cur[:n], prev[:n], w[:n], level, lim, sysm.epsilon, tick)
        done += n
        n = k
    el = time.perf_counter() - t0
    v = done / el
    out = {
        "impl": "reference", "metric": "particle-steps/s", "value": v, "unit": "particle-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": workload_name(sysm), "sample_particles": n0, "parallelism": "host threads"},
        "cpu_baseline": {"value": v, "unit": "particle-steps/s", "cores": oracle.num_threads(), "kind": "port",
                         "sample": cpu_sample_text(sysm, n0, args.steps)},
        "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def run_reference_mode(args):
    """The reference arm of the modes outside the Stars step: the raster has a CPU restatement; the batched form
    and the adjoint have no counterpart in the reference."""
    if args.config != "display_16m":
        why = {"batched_512": "the reference has no batched form (it steps one system per Stars)",
               "adjoint_262k": "the reference has no adjoint",
               "models_16m": "the reference's models run only on a GPU (curand); the oracle restates their "
                             "arithmetic for the gb300 line's cpu_baseline",
               "movie_disk": "the reference's movie program runs only on a GPU; the gb300 line's cpu_baseline "
                             "times the oracle's frame loop"}.get(args.config, f"unknown config {args.config}")
        print(json.dumps({"impl": "reference", "unavailable": why}), flush=True)
        return
    from nbfmm_gb300 import workloads
    from oracle import oracle

    oracle.lib()
    sysm = workloads.two_disks()
    n, width, height, size_scale = sysm.n, 1920, 1080, 1e-4
    for _ in range(args.warmup):
        oracle.display(sysm.position, sysm.weight, width, height, size_scale, sysm.limits, threads=True)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.display(sysm.position, sysm.weight, width, height, size_scale, sysm.limits, threads=True)
    el = time.perf_counter() - t0
    v = n * args.steps / el
    print(json.dumps({
        "impl": "reference", "metric": "stars/s", "value": v, "unit": "stars/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": f"display: the two-disk state, N={n:,}, into a {width}x{height} YUV 4:2:0 frame",
                   "parallelism": "host threads"},
        "cpu_baseline": {"value": v, "unit": "stars/s", "cores": oracle.num_threads(), "kind": "port",
                         "sample": f"{args.steps} frames of the whole workload"},
        "e2e": {"value": v, "unit": "stars/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


# ---- GPU side --------------------------------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_id):
        self.proc = None
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", device_id, "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for name, val in zip(names, f[4:8]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_sm_mhz():
    """Median SM clock under load recorded in MEASURED_PEAKS.json, when the run sampled none itself."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(path))["clocks_under_load"]["sm_mhz_median"])
    except (OSError, KeyError, ValueError):
        return 1900.0


def p2p_pairs(torch, head, base_dim):
    """Algorithmic P2P pair count of one solve: each target against its 3x3 leaf cells, self excluded."""
    n = (head[1:base_dim * base_dim + 1] - head[:base_dim * base_dim]).double().reshape(1, 1, base_dim, base_dim)
    ns = torch.nn.functional.conv2d(n, torch.ones(1, 1, 3, 3, dtype=n.dtype, device=n.device), padding=1)
    return int((n * (ns - 1)).clamp(min=0).sum().item())


def stage_bandwidth(torch, solver, pos, w, n, num_level, reps=5):
    """The solve's stages run one by one through the stage entry points (the reference's NBFMM_CHECK-public
    methods) on `n` particles in caller order, each timed with CUDA events on the current stream (median of
    `reps` after a warm-up), against its algorithmic bytes: HBM-bound sweeps reported in GB/s and as a fraction
    of the measured copy bandwidth. P2P (compute-bound) is the step's roofline and is left out here."""
    b = 1 << (num_level + 1)
    c = b * b
    levels = num_level if num_level > 0 else 1
    dims = [b >> l for l in range(levels)]
    key_bits = 2 * (num_level + 1)
    passes = 1 if key_bits <= 10 else -(-key_bits // 10)  # record-sort passes of at most 10 bits
    # Record sort: the first pass reads positions twice (keys for the tile counts, then for ranking: 8 B each)
    # and weights once (4 B), and writes key + record (20 B); each later pass reads keys twice (4 B each) and
    # the record (16 B) and writes key + record (20 B); the last pass also writes the permutation (4 B). Then
    # heads (4 B per cell, binary searches in cache), the work list and the leaf sums (16 B read per particle,
    # 16 B written per leaf cell).
    sort_bytes = 40 + 44 * (passes - 1) + 4
    bytes_ = {
        "predo": n * (sort_bytes + 16) + c * 28,
        "p2m": n * 16 + c * 20,
        "m2m": sum((dims[l - 1] ** 2 + dims[l] ** 2) * 16 for l in range(1, levels)),
        "m2l": sum(d * d * (16 + 8) for d in dims),
        "l2l": sum(dims[l + 1] ** 2 * 8 + dims[l] ** 2 * 16 for l in range(levels - 1)),
        "l2p": n * 20 + c * 8,
        "postdo": n * 20,
    }
    eff = torch.empty(n, 2, device="cuda")
    calls = {
        "predo": lambda: solver.predo(n, pos, w), "p2m": lambda: solver.p2m(n), "m2m": solver.m2m,
        "m2l": solver.m2l, "l2l": solver.l2l, "l2p": lambda: solver.l2p(n), "postdo": lambda: solver.postdo(n, eff),
    }
    solver.predo(n, pos, w)
    solver.p2p(n)  # sorted effects for l2p / postdo
    peak = measured_hbm_gbs()
    out = {"workload": "one solve from caller order, stage by stage", "hbm_peak_gbs": peak}
    for name, fn in calls.items():
        fn()
        times = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        ms = statistics.median(times)
        gbs = bytes_[name] / (ms / 1e3) / 1e9
        out[name] = {"ms": ms, "bytes": bytes_[name], "gbs": gbs, "frac": gbs / peak if peak else None}
        if name == "predo":
            # the task's own minimum (read x, y, m; write the sorted x, y, m and the permutation; heads)
            task = n * 28 + (c + 1) * 4
            out[name].update(task_bytes=task, task_frac=task / (ms / 1e3) / 1e9 / peak if peak else None)
    del eff
    return out


def measured_hbm_gbs():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        return 6800.0  # fallback: one earlier STREAM-style copy on a GB300


def fp64_direct(torch, pos, w, eps, targets):
    """FP64 all-pairs direct sum on the GPU for the listed targets (the error reference of every result)."""
    p = pos.double()
    m = w.double()
    out = []
    for t in targets.split(8):
        d = p[None, :, :] - p[t][:, None, :]  # (8, n, 2)
        r = torch.sqrt((d * d).sum(-1))
        s = m[None, :] / (r * r * r + eps)
        s[torch.arange(len(t), device=p.device), t] = 0.0
        out.append((d * s[..., None]).sum(1))
    return torch.cat(out)


def rel_error_stats(torch, got, ref):
    e = torch.linalg.norm(got.double() - ref, dim=1) / torch.linalg.norm(ref, dim=1)
    return {"median": float(e.median()), "p99": float(torch.quantile(e, 0.99)), "max": float(e.max()),
            "targets": int(len(ref))}


def fp64_error(torch, pos, w, eff, eps, targets):
    """Relative error of the engine's effects against the FP64 all-pairs direct sum, on the GPU, for targets."""
    return rel_error_stats(torch, eff[targets], fp64_direct(torch, pos, w, eps, targets))


def cpu_direct_baselines():
    """OpenMP all-pairs direct sums on the host cores (the oracle library), FP32 (kernelFunction's operations)
    and FP64, at N = 16,384 (every target) and N = 1,048,576 (2,048 sampled targets; the rate extrapolates to
    a whole solve of N (N - 1) pairs)."""
    from nbfmm_gb300 import workloads
    from oracle import oracle

    oracle.lib()
    out = {"cores": oracle.num_threads(), "kind": "port",
           "how": "orc_direct_f32 / orc_direct_f64, OpenMP over targets, all sources in index order"}
    for name, sysm in (("plain_16k", workloads.plain(16384, 1, 3)), ("disk_1m", workloads.disk(1 << 20, 2, 6))):
        n = sysm.n
        targets = None if n <= 16384 else np.sort(np.random.default_rng(0).choice(n, 2048, replace=False))
        nt = n if targets is None else len(targets)
        for prec, fn in (("f32", oracle.direct_f32), ("f64", oracle.direct_f64)):
            t0 = time.perf_counter()
            fn(sysm.position, sysm.weight, sysm.epsilon, targets)
            el = time.perf_counter() - t0
            rate = nt * (n - 1) / el
            solve_s = n * (n - 1) / rate
            out[f"{name}_{prec}"] = {"pairs_per_s": rate, "solve_s": solve_s, "particle_steps_per_s": n / solve_s,
                                     "targets_timed": nt}
    return out


def measure_exact(torch, nbfmm_gb300, sysm, pos, prev, w, steps, warmup):
    """The same Stars steps with exact near-field arithmetic (correctly rounded sqrt and division, no
    contraction: bit for bit the oracle's IEEE single-precision rounding)."""
    st = nbfmm_gb300.Stars(sysm.num_level, sysm.n, tick=sysm.dt, grav_const=sysm.grav_const,
                           position_limits=sysm.limits, epsilon=sysm.epsilon, arithmetic="exact")
    st.gpuptr_position_cur_.copy_(pos)
    st.gpuptr_position_pre_.copy_(prev)
    st.gpuptr_weight_.copy_(w)
    st.update(warmup)
    torch.cuda.synchronize()
    st.profile_begin(steps)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    st.update(steps)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    p2p_ms, k = st.profile_end()
    st.close()
    return {"value": sysm.n * steps / (ms / 1e3), "unit": "particle-steps/s", "steps": steps, "warmup": warmup,
            "ms_per_step": ms / steps, "p2p_ms_per_launch": p2p_ms / max(k, 1),
            "what": "the same workload and Stars steps with Stars.set_arithmetic('exact')"}


def run_batched(args):
    """The batched form against looped single-system updates on the same systems and depths."""
    print(json.dumps(measure_batched(args.steps, args.warmup)), flush=True)


def measure_batched(steps, warmup):
    """The 512-system batched step against looped Stars updates of the same systems, depths and steps."""
    import torch

    import nbfmm_gb300
    from nbfmm_gb300 import autotune, workloads

    sysb = workloads.batched()
    levels, passes, report = autotune.tune(nbfmm_gb300, sysb)
    levels_d, report_d = autotune.tune_levels(nbfmm_gb300, sysb)
    prev = sysb.previous()
    n = sysb.n
    clocks = ClockSampler("0")

    def run(lv, item_passes, profile):
        b = nbfmm_gb300.Batch(sysb.offsets, lv, sysb.limits, tick=sysb.dt, grav_const=sysb.grav_const,
                              epsilon=sysb.epsilon)
        if item_passes is not None:
            b.set_item_passes(item_passes)
        b.position_cur[:] = torch.from_numpy(sysb.position).cuda()
        b.position_pre[:] = torch.from_numpy(prev).cuda()
        b.weight[:] = torch.from_numpy(sysb.weight).cuda()
        b.update(warmup)
        torch.cuda.synchronize()
        if profile:
            b.profile_begin(steps)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        b.update(steps)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        p2p = b.profile_end()[0] if profile else None
        launches = b.kernel_launches(steps)
        b.close()
        return ms, p2p, launches

    batched_ms, p2p_ms, launches = run(levels, passes, True)
    depth_only_ms, _, _ = run(levels_d, None, False)
    clk = clocks.stop()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    stars = []
    for s in range(sysb.num_systems):
        lo, hi = int(sysb.offsets[s]), int(sysb.offsets[s + 1])
        st = nbfmm_gb300.Stars(int(levels[s]), hi - lo, tick=sysb.dt, grav_const=sysb.grav_const,
                               position_limits=tuple(float(v) for v in sysb.limits[s]), epsilon=sysb.epsilon)
        st.gpuptr_position_cur_[:] = torch.from_numpy(sysb.position[lo:hi]).cuda()
        st.gpuptr_position_pre_[:] = torch.from_numpy(prev[lo:hi]).cuda()
        st.gpuptr_weight_[:] = torch.from_numpy(sysb.weight[lo:hi]).cuda()
        st.update(warmup)
        stars.append(st)
    torch.cuda.synchronize()
    e0.record()
    for st in stars:
        st.update(steps)
    e1.record()
    torch.cuda.synchronize()
    looped_ms = e0.elapsed_time(e1)
    value = n * steps / (batched_ms / 1e3)
    looped = n * steps / (looped_ms / 1e3)
    out = {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": 1,
        "steps": steps, "warmup": warmup, "ms_per_step": batched_ms / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded; nbfmm_gb300/workloads.py batched)",
        "config": {"workload": f"batched: {sysb.num_systems} systems, N lognormal(median 20k, sd 0.8) clipped to "
                               f"[2k, 262k], {n:,} particles, squares and disks, eps {sysb.epsilon:g}, "
                               f"dt {sysb.dt:g}", "autotune": report},
        "depth_only_tuning": {"value": n * steps / (depth_only_ms / 1e3), "ms_per_step": depth_only_ms / steps,
                              "how": "tree depth chosen per bucket, P2P items of 4 passes", "autotune": report_d},
        "looped": {"value": looped, "ms_per_step": looped_ms / steps,
                   "how": "one Stars per system with the same depths; update(K) per system, one after another"},
        "speedup_vs_looped": value / looped,
        "p2p_share_of_step": p2p_ms / batched_ms, "gpu_launches": launches, "clocks": clk,
    }
    return out


def run_adjoint(args):
    print(json.dumps(measure_adjoint(args.steps, args.warmup)), flush=True)


def measure_adjoint(steps, warmup):
    """Adjoint through the trajectory: forward pass and backward pass of the 262,144-particle disk (depth 6),
    dt 1e-4, checkpoints every 20 steps; targets = forward final positions + N(0, 1e-3)."""
    import torch

    import nbfmm_gb300
    from nbfmm_gb300 import workloads
    from nbfmm_gb300.adjoint import Adjoint

    sysm = workloads.disk(1 << 18, seed=5, num_level=5)
    n = sysm.n
    f = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
    x0, v0, m = f(sysm.position), f(sysm.velocity), f(sysm.weight)
    adj = Adjoint(sysm.num_level, n, sysm.limits, tick=sysm.dt, max_steps=steps, checkpoint_interval=20,
                  epsilon=sysm.epsilon)
    xT = torch.empty_like(x0)
    adj.forward(steps, x0, v0, m, xT)
    torch.cuda.synchronize()
    g = torch.Generator(device="cpu").manual_seed(5)
    target = (xT.cpu() + 1e-3 * torch.randn(xT.shape, generator=g)).cuda()
    gx, gv, gm, terms = torch.empty_like(x0), torch.empty_like(v0), torch.empty_like(m), torch.empty_like(m)
    for _ in range(max(1, warmup)):
        adj.forward(steps, x0, v0, m, xT)
        adj.backward(target, gx, gv, gm, terms)
    torch.cuda.synchronize()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    clocks = ClockSampler("0")
    e[0].record()
    adj.forward(steps, x0, v0, m, xT)
    e[1].record()
    adj.backward(target, gx, gv, gm, terms)
    e[2].record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    fwd = e[0].elapsed_time(e[1])
    bwd = e[1].elapsed_time(e[2])
    # the graph-replayed Stars step of the same system, for reference
    st = nbfmm_gb300.Stars(sysm.num_level, n, tick=sysm.dt, position_limits=sysm.limits, epsilon=sysm.epsilon)
    st.gpuptr_position_cur_.copy_(x0)
    st.gpuptr_position_pre_.copy_(f(sysm.previous()))
    st.gpuptr_weight_.copy_(m)
    st.update(3)
    torch.cuda.synchronize()
    e[0].record()
    st.update(steps)
    e[1].record()
    torch.cuda.synchronize()
    stars_ms = e[0].elapsed_time(e[1])
    out = {
        "metric": "adjoint/forward time", "value": bwd / fwd, "unit": "ratio", "higher_is_better": False,
        "n_gpus": 1, "steps": steps, "warmup": warmup, "dtype": "f32", "data": "synthetic (seeded disk)",
        "config": {"workload": f"adjoint: disk N={n:,}, depth 6, dt {sysm.dt:g}, eps {sysm.epsilon:g}, "
                               f"{steps} steps, checkpoint every 20, loss 0.5 sum m |x(T) - x*|^2"},
        "forward_ms_per_step": fwd / steps, "backward_ms_per_step": bwd / steps,
        "adjoint_total_over_forward": (fwd + bwd) / fwd,
        "stars_update_ms_per_step": stars_ms / steps, "backward_over_stars_step": bwd / stars_ms,
        "particle_steps_per_s_forward": n * steps / (fwd / 1e3), "clocks": clk,
    }
    return out


# DRAM bytes (read + write) of one raster_bits_kernel launch per star: ncu's dram__bytes_read.sum (201.60 MB) and
# dram__bytes_write.sum (3.42 MB) for one launch on the display workload itself (N = 16,777,216, 1920x1080).
DISPLAY_DRAM_BYTES_PER_STAR = (201.596928e6 + 3.421184e6) / 16777216


def run_display(args):
    """The frame raster of Stars::display (display.cu:29-221): the 16.8M two-disk state drawn into one 1920 x 1080
    YUV 4:2:0 frame per step. value = stars drawn per second on the device; e2e = the same through the movie
    writer (raster, prune, frame copy to pinned host memory, file write)."""
    import tempfile

    import torch

    import nbfmm_gb300
    from nbfmm_gb300 import workloads

    sysm = workloads.two_disks()
    n, width, height, size_scale = sysm.n, 1920, 1080, 1e-4
    lim = sysm.limits
    pos = torch.from_numpy(sysm.position).cuda()
    w = torch.from_numpy(sysm.weight).cuda()
    fb = nbfmm_gb300.frame_bytes(width, height)
    board = torch.empty(fb, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(max(3, args.warmup)):
        nbfmm_gb300.display(pos, w, width, height, size_scale, lim, board)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * args.steps)]
    clocks = ClockSampler("0")
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for k in range(args.steps):
        ev[2 * k].record(stream)
        nbfmm_gb300.display(pos, w, width, height, size_scale, lim, board)
        ev[2 * k + 1].record(stream)
    t1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    total_ms = t0.elapsed_time(t1)
    launch_ms = statistics.mean(ev[2 * k].elapsed_time(ev[2 * k + 1]) for k in range(args.steps))
    lit = int((board[:width * height] == 255).sum())

    # e2e: the movie writer on a Stars holding the same state (its first frame prunes nothing: all stars are
    # inside the limits).
    st = nbfmm_gb300.Stars(sysm.num_level, n, width, height, 30, sysm.dt, sysm.grav_const, size_scale, lim, lim,
                           epsilon=sysm.epsilon)
    st.gpuptr_position_cur_.copy_(pos)
    st.gpuptr_position_pre_.copy_(torch.from_numpy(sysm.previous()).cuda())
    st.gpuptr_weight_.copy_(w)
    torch.cuda.synchronize()
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "frames.y4m")
        with nbfmm_gb300.Movie(st, path) as mv:
            for _ in range(max(3, args.warmup)):
                mv.frame()
            torch.cuda.synchronize()
            w0 = time.perf_counter()
            for _ in range(args.steps):
                mv.frame()
            mv.close()
            e2e_s = time.perf_counter() - w0
        file_bytes = os.path.getsize(path)

    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle

        oracle.lib()
        reps = 3
        c0 = time.perf_counter()
        for _ in range(reps):
            ref = oracle.display(sysm.position, sysm.weight, width, height, size_scale, lim, threads=True)
        cpu_s = (time.perf_counter() - c0) / reps
        cpu = {"value": n / cpu_s, "unit": "stars/s", "cores": oracle.num_threads(), "kind": "port",
               "sample": f"the whole workload ({n:,} stars, one 1920x1080 frame), {reps} frames, oracle raster "
                         "(C, OpenMP over the host cores)",
               "frame_equal": bool(np.array_equal(ref, board.cpu().numpy()))}

    peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    alg_bytes = 12 * n + fb
    achieved = alg_bytes / (launch_ms / 1e3) / 1e9
    out = {
        "metric": "stars/s", "value": n * args.steps / (total_ms / 1e3), "unit": "stars/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded; nbfmm_gb300/workloads.py)",
        "config": {"workload": f"display: the two-disk state, N={n:,}, into a {width}x{height} YUV 4:2:0 frame, "
                               f"size_scale {size_scale:g}, display limits = position limits {list(lim)}",
                   "l2": "inputs larger than L2 (positions and weights 12 B/star = 201 MB)", "lit_pixels": lit},
        "roofline": {"kernel": "raster_bits_kernel + expand_kernel (the whole frame)", "bound": "hbm", "unit": "GB/s",
                     "achieved": achieved, "peak": peak, "frac": achieved / peak,
                     "traffic": (DISPLAY_DRAM_BYTES_PER_STAR * n if DISPLAY_DRAM_BYTES_PER_STAR else None),
                     "algorithmic_bytes": alg_bytes, "launch_ms": launch_ms,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of raster_bits_kernel on "
                                       "this workload",
                     "note": "the raster issues IEEE-exact pixel arithmetic and shared-memory atomics per star; it "
                             "is bound by SIMT issue, not by HBM",
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)"},
        "e2e": {"value": n * args.steps / e2e_s, "unit": "stars/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": fb, "api": "Movie.frame(): Stars.display (raster + prune), frame copy to "
                "pinned host memory, .y4m file write; wall clock", "file_bytes": file_bytes},
        "cpu_baseline": cpu, "gpu_launches": args.steps, "clocks": clk,
    }
    print(json.dumps(out), flush=True)


def run_models(args):
    """The reference's initial-condition models (source/nbfmm/model): the centred double disk of the movie program
    generated for 16.8M stars on the device (curand_init(0, idx, 0) per star, then the orbit arithmetic)."""
    import torch

    import nbfmm_gb300
    from nbfmm_gb300 import model

    n1, n2 = 10_485_760, 6_291_456  # 5:3, as the double-disk script
    n = n1 + n2
    cur = torch.empty(n, 2, device="cuda")
    prev = torch.empty(n, 2, device="cuda")
    w = torch.empty(n, device="cuda")
    c1, c2, r1, r2, tick = (-0.5, 0.0), (0.5, 0.0), 0.3, 0.2, 5e-5

    def gen():
        model.generateDoubleDiskCenter(n1, n2, c1, c2, r1, r2, 1.0 / n, 10.0, 6.0, 1.0, tick, cur, prev, w)

    for _ in range(max(3, args.warmup)):
        gen()
    torch.cuda.synchronize()
    clocks = ClockSampler("0")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        gen()
    e1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle

        oracle.lib()
        m = 1 << 20
        u = np.random.default_rng(0).uniform(1e-7, 1.0, (m, 3)).astype(np.float32)
        t0 = time.perf_counter()
        oracle.model("double_disk_center", 0, u, n1=m * 5 // 8, n2=m * 3 // 8, center1=c1, center2=c2, radius1=r1,
                     radius2=r2, weight=1.0 / n, center_weight1=10.0, center_weight2=6.0, eccentricity=1.0,
                     tick=tick)
        el = time.perf_counter() - t0
        cpu = {"value": m / el, "unit": "stars/s", "cores": 1, "kind": "port",
               "sample": f"{m:,} stars of the same model, the oracle's arithmetic on host-drawn uniforms "
                         "(no CPU code reproduces curand's stream)"}
    out = {
        "metric": "stars/s", "value": n / (ms / 1e3), "unit": "stars/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "generated (the model itself)",
        "config": {"workload": f"generateDoubleDiskCenter: {n1:,} + {n2:,} stars, radii {r1}/{r2}, centre weights 10/6"},
        "roofline": {"kernel": "disk_kernel (curand_init + orbit arithmetic) x2 + shift_kernel x2", "bound": "hbm",
                     "unit": "GB/s", "achieved": 20 * n / (ms / 1e3) / 1e9,
                     "peak": json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"],
                     "frac": 20 * n / (ms / 1e3) / 1e9 / json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"],
                     "traffic": None, "note": "20 B written per star; bound by curand_init's skip-ahead per star"},
        "cpu_baseline": cpu, "gpu_launches": 4 * args.steps, "clocks": clk,
        "e2e": {"value": n / (ms / 1e3), "unit": "stars/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                "api": "model.generateDoubleDiskCenter on device arrays (no host data)"},
    }
    print(json.dumps(out), flush=True)


def run_movie(args):
    """The movie program on the reference's disk script preset (main/script/disk.py: 10,000 stars, 1024 x 768,
    60 fps, FMM level 4, a 16 x 12 domain at display scale 0.5). value = frames per second of the frame loop
    (update, display, frame copy, file write) through the Python API, timed on the device; e2e = frames per second
    of the nbfmm_main process itself, wall clock, start to exit."""
    import tempfile

    import torch

    import nbfmm_gb300
    from nbfmm_gb300 import build, launch, model

    frames = max(60, args.steps)
    argv = launch.preset("disk", num_second=1)
    argv[2] = str(frames)  # fps = frames, 1 second: `frames` frames
    width, height, fps, _, level, n, pw, ph, ds, g, ss = (float(a) for a in argv[:11])
    width, height, fps, level, n = int(width), int(height), int(fps), int(level), int(n)
    radius, weight = float(argv[12]), float(argv[13])
    tick = float(np.float32(0.05 / fps))
    plim = (-pw / 2, -ph / 2, pw / 2, ph / 2)
    dlim = tuple(v * ds for v in plim)
    with tempfile.TemporaryDirectory() as tmp:
        st = nbfmm_gb300.Stars(level, n, width, height, fps, tick, g, ss, plim, dlim)
        st.initialize(model.generateDisk, n, (0.0, 0.0), radius, weight)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with nbfmm_gb300.Movie(st, os.path.join(tmp, "api.y4m")) as mv:
            mv.frame()
            for _ in range(min(args.warmup, frames - 1)):
                st.update(1)
                mv.frame()
            torch.cuda.synchronize()
            e0.record()
            for _ in range(frames):
                st.update(1)
                mv.frame()
            e1.record()
            mv.close()
        torch.cuda.synchronize()
        api_ms = e0.elapsed_time(e1)
        exe = build.program("nbfmm_main")
        if not os.path.exists(exe):
            build.build()
        w0 = time.perf_counter()
        r = subprocess.run([exe, os.path.join(tmp, "cli.y4m")] + argv, capture_output=True)
        cli_s = time.perf_counter() - w0
        assert r.returncode == 0, r.stderr[-500:]
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle

        oracle.lib()
        rng = np.random.default_rng(1)
        rr = radius * np.sqrt(rng.uniform(0.01, 1.0, n))
        a = rng.uniform(0, 2 * np.pi, n)
        cur = np.stack([rr * np.cos(a), rr * np.sin(a)], 1).astype(np.float32)
        prev, w = cur.copy(), np.full(n, weight, np.float32)
        k, t0 = n, time.perf_counter()
        cframes = 30
        with open(os.devnull, "wb") as f:
            for _ in range(cframes):
                k2, cur[:k], prev[:k], w[:k], _ = oracle.stars_update(cur[:k], prev[:k], w[:k], level, plim, 0.1, tick)
                k = k2
                f.write(b"FRAME\n")
                f.write(oracle.display(cur[:k], w[:k], width, height, ss, dlim).tobytes())
        el = time.perf_counter() - t0
        cpu = {"value": cframes / el, "unit": "frames/s", "cores": oracle.num_threads(), "kind": "port",
               "sample": f"{cframes} frames of {n:,} stars: the oracle's Stars::update and raster, frames written"}
    out = {
        "metric": "frames/s", "value": frames / (api_ms / 1e3), "unit": "frames/s", "n_gpus": 1, "steps": frames,
        "warmup": args.warmup, "ms_per_step": api_ms / frames, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "generated (the reference's disk model)",
        "config": {"workload": f"movie: disk script preset, {n:,} stars, {width}x{height}, FMM level {level}, "
                               f"{frames} frames", "argv": argv},
        "e2e": {"value": frames / cli_s, "unit": "frames/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": width * height * 3 // 2,
                "api": "nbfmm_main process, wall clock from start to exit (library load, CUDA start-up, model, "
                       "frames, file)"},
        "cpu_baseline": cpu, "gpu_launches": None,
    }
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    from nbfmm_gb300 import workloads

    if args.steps is None:
        own = {"batched_512": 100, "adjoint_262k": 200}
        if args.config in own:
            args.steps = own[args.config]
        elif args.config in workloads.CONFIGS:
            args.steps = workloads.CONFIGS[args.config]().steps
        else:
            args.steps = 200
    if args.config == "batched_512" and args.impl == "gb300":
        return run_batched(args)
    if args.config == "adjoint_262k" and args.impl == "gb300":
        return run_adjoint(args)
    if args.config == "display_16m" and args.impl == "gb300":
        return run_display(args)
    if args.config == "models_16m" and args.impl == "gb300":
        return run_models(args)
    if args.config == "movie_disk" and args.impl == "gb300":
        return run_movie(args)

    from nbfmm_gb300 import replicas

    rank, world, local = replicas.rank_info()
    if args.impl == "reference" and args.config not in workloads.CONFIGS:
        if rank == 0:
            run_reference_mode(args)
        return
    sysm = workloads.CONFIGS[args.config]()

    if args.impl == "reference":
        run_reference_arm(args, sysm, rank)
        return

    import torch

    import nbfmm_gb300

    torch.cuda.set_device(local)
    dist = replicas.init(world, "nccl")
    dev_id = str(local)
    try:
        dev_id = "GPU-" + str(torch.cuda.get_device_properties(local).uuid)
    except Exception:
        pass

    n = sysm.n
    pos = torch.from_numpy(sysm.position).cuda()
    w = torch.from_numpy(sysm.weight).cuda()
    prev = torch.from_numpy(sysm.previous()).cuda()

    # One solve of the initial state: the P2P pair count and the error against the FP64 direct sum.
    solver = nbfmm_gb300.Solver(sysm.num_level, n, sysm.limits, epsilon=sysm.epsilon, arithmetic=args.arithmetic)
    eff = torch.empty(n, 2, device="cuda")
    solver.solve(n, pos, w, eff)
    torch.cuda.synchronize()
    b = 1 << (sysm.num_level + 1)
    pairs0 = p2p_pairs(torch, solver.buffers()["head"], b)
    g = torch.Generator(device="cpu").manual_seed(1234)
    targets = torch.randperm(n, generator=g)[:512].cuda()
    ref64 = fp64_direct(torch, pos, w, sysm.epsilon, targets)
    err64 = rel_error_stats(torch, eff[targets], ref64)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the oracle's solve (the reference's algorithm in IEEE single precision) at the same targets
        from oracle import oracle

        t_sorted, order = torch.sort(targets)
        ref_orc = oracle.solve_targets(sysm.position, sysm.weight, sysm.num_level, sysm.limits, sysm.epsilon,
                                       t_sorted.cpu().numpy().astype(np.int32))
        got_orc = torch.empty(len(targets), 2, dtype=torch.float32, device="cuda")
        got_orc[order] = torch.from_numpy(ref_orc).cuda()
        err64 = {"engine": err64, "oracle": rel_error_stats(torch, got_orc, ref64)}
    del eff
    torch.cuda.empty_cache()  # return the FP64 check's temporaries
    stages = stage_bandwidth(torch, solver, pos, w, n, sysm.num_level)

    stars = nbfmm_gb300.Stars(sysm.num_level, n, tick=sysm.dt, grav_const=sysm.grav_const,
                              position_limits=sysm.limits, epsilon=sysm.epsilon, arithmetic=args.arithmetic)
    stars.gpuptr_position_cur_.copy_(pos)
    stars.gpuptr_position_pre_.copy_(prev)
    stars.gpuptr_weight_.copy_(w)
    stream = torch.cuda.current_stream()
    stars.update(args.warmup)
    torch.cuda.synchronize()

    # ---- timed region: K steps in one update call, P2P timed per launch with CUDA events ----
    stars.profile_begin(args.steps)
    replicas.barrier(dist)
    torch.cuda.synchronize()
    clocks = ClockSampler(dev_id)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    stars.update(args.steps)
    ev1.record(stream)
    torch.cuda.synchronize()
    replicas.barrier(dist)
    clk = clocks.stop()
    elapsed_ms = replicas.max_over_ranks(ev0.elapsed_time(ev1), dist, "cuda")
    p2p_ms, p2p_launches = stars.profile_end()
    n_end = stars.num_star_

    # Pair count at the end of the timed steps (the system moves); the roofline uses the mean of both ends.
    cur_now = stars.gpuptr_position_cur_[:n_end].clone()
    solver.solve(n_end, cur_now, stars.gpuptr_weight_[:n_end].clone(), torch.empty(n_end, 2, device="cuda"))
    torch.cuda.synchronize()
    pairs1 = p2p_pairs(torch, solver.buffers()["head"], b)
    pairs = 0.5 * (pairs0 + pairs1)

    # ---- e2e: the same steps through the public API with host buffers. A second Stars restarts from the initial
    # state, runs the same warm-up steps untimed, then the same K steps; every step copies the state in from
    # pinned host memory, runs update(1) and copies the state out. ----
    e2e_steps = args.steps
    st2 = nbfmm_gb300.Stars(sysm.num_level, n, tick=sysm.dt, grav_const=sysm.grav_const,
                            position_limits=sysm.limits, epsilon=sysm.epsilon, arithmetic=args.arithmetic)
    h_cur = torch.empty(n, 2, pin_memory=True)
    h_prev = torch.empty(n, 2, pin_memory=True)
    h_w = torch.empty(n, pin_memory=True)
    h_cur.copy_(pos)
    h_prev.copy_(prev)
    h_w.copy_(w)
    pub = (st2.gpuptr_position_cur_[:n], st2.gpuptr_position_pre_[:n], st2.gpuptr_weight_[:n])
    host = (h_cur, h_prev, h_w)

    def e2e_step(marks=None):
        if marks:
            marks[0].record(stream)
        for d, h in zip(pub, host):
            d.copy_(h, non_blocking=True)
        if marks:
            marks[1].record(stream)
        st2.update(1)
        if marks:
            marks[2].record(stream)
        for d, h in zip(pub, host):
            h.copy_(d, non_blocking=True)
        if marks:
            marks[3].record(stream)

    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    replicas.barrier(dist)
    parts = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(e2e_steps)]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2e_clocks = ClockSampler(dev_id)
    e0.record(stream)
    for k in range(e2e_steps):
        e2e_step(parts[k])
    e1.record(stream)
    torch.cuda.synchronize()
    replicas.barrier(dist)
    e2e_clk = e2e_clocks.stop()
    e2e_ms = replicas.max_over_ranks(e0.elapsed_time(e1), dist, "cuda")
    e2e_parts = {name: statistics.median(parts[k][j].elapsed_time(parts[k][j + 1]) for k in range(e2e_steps))
                 for j, name in enumerate(("copy_in_ms", "update_ms", "copy_out_ms"))}
    del st2
    io_bytes = n * (8 + 8 + 4)

    launches = stars.kernel_launches(args.steps)
    extras = {}
    if rank == 0 and world == 1 and not args.no_extras and args.config == "two_disks_16m":
        extras["exact_arithmetic"] = measure_exact(torch, nbfmm_gb300, sysm, pos, prev, w, 10, 2)
        del stars
        torch.cuda.empty_cache()
        extras["batched"] = measure_batched(100, 3)
        extras["adjoint"] = measure_adjoint(200, 1)
        if not args.no_cpu_baseline:
            extras["cpu_direct"] = cpu_direct_baselines()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, cores, ns, el = cpu_steps(sysm, 1000, budget_s=15.0)
        steps_done = max(1, int(round(v * el / max(ns, 1))))
        cpu = {"value": v, "unit": "particle-steps/s", "cores": cores, "kind": "port",
               "sample": cpu_sample_text(sysm, ns, steps_done)}

    if rank != 0:
        return
    value = replicas.whole_job_rate(n * args.steps, world, elapsed_ms)
    p2p_s = p2p_ms / max(p2p_launches, 1) / 1e3
    sm_mhz = clk["sm_mhz"] or measured_sm_mhz()
    fp32_peak = SMS * FP32_LANES * 2 * sm_mhz * 1e6 / 1e12
    achieved = FLOP_PER_PAIR * pairs / p2p_s / 1e12
    series = series_degree(sysm, args.arithmetic)
    mufu = P2P_MUFU_PER_PAIR_SERIES[series] if series else P2P_MUFU_PER_PAIR
    out = {
        "metric": "particle-steps/s",
        "value": value,
        "unit": "particle-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": elapsed_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded; nbfmm_gb300/workloads.py)",
        "config": {"workload": workload_name(sysm), "N": n, "num_level": sysm.num_level,
                   "arithmetic": args.arithmetic, "steps_per_call": args.steps, "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (state + sorted copy ~ 0.9 GB at N=16.8M)",
                   "stars_after_timed_steps": n_end},
        "roofline": {
            "kernel": "p2p_kernel<kVerlet> (near field + L2P + Verlet epilogue)",
            "bound": "fp32", "unit": "TFLOP/s",
            "achieved": achieved, "peak": fp32_peak, "frac": achieved / fp32_peak,
            "traffic": P2P_DRAM_BYTES_PER_PARTICLE * n,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the N=4,194,304 capture, "
                              "scaled by particles per launch",
            "peak_source": f"nominal FP32 FMA rate {SMS} SMs x {FP32_LANES} lanes x 2 at the median sampled SM clock "
                           f"({sm_mhz:.0f} MHz); MEASURED_PEAKS.json has no SIMT FP32 figure",
            "flop_per_pair": FLOP_PER_PAIR, "pairs_per_launch": pairs, "p2p_ms_per_launch": p2p_s * 1e3,
            "p2p_share_of_step": p2p_ms / max(elapsed_ms, 1e-9),
            "pairs_per_s": pairs / p2p_s,
            "series_degree": series,
            "mufu_ops_per_pair": mufu,
            "mufu_bound_pairs_per_s": SMS * MUFU_LANES * sm_mhz * 1e6 / mufu,
        },
        "e2e": {"value": replicas.whole_job_rate(n * e2e_steps, world, e2e_ms), "unit": "particle-steps/s",
                "median_parts": e2e_parts, "clocks": e2e_clk,
                "h2d_bytes_per_step": io_bytes, "d2h_bytes_per_step": io_bytes,
                "api": "Stars.update(1) per step, state copied in from and out to pinned host memory; the same "
                       "warm-up and timed steps as the device-timed value, from the same initial state"},
        "stages": stages,
        "cpu_baseline": cpu,
        "gpu_launches": launches,
        "clocks": clk,
        "error_vs_fp64": err64,
    }
    out.update(extras)
    print(json.dumps(out), flush=True)
    replicas.finish(dist)


if __name__ == "__main__":
    main()
