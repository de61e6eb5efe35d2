"""Per-size-bucket tree depth and P2P tile shape for the batched form, chosen by measurement.

Systems are bucketed by size (powers of two). For each bucket the candidate depths are those giving between
MIN_PER_CELL and MAX_PER_CELL particles per leaf cell (nominal n / B^2, B = 2^(num_level+1)); the band keeps
the method's accuracy in the range of the reference's own configurations (its far-field error grows with
depth). The tile shape is the P2P work item: 2 or 4 passes of 32 target stars per item (ITEM_PASSES), a
trade between reusing each loaded source for more targets and spreading a system's cells over more warps; it
does not change any result. Each candidate is timed on a mini-batch of the bucket's own systems (up to `sample`
of them, a few steps after a warm-up, CUDA events), and the fastest is used for every system of the bucket.
tune_levels chooses the depth alone (items of 4 passes); tune chooses depth and tile together.
"""
import numpy as np

MIN_PER_CELL = 16
MAX_PER_CELL = 256
ITEM_PASSES = (2, 4)


def candidate_levels(n: int, max_level: int = 10):
    out = []
    for level in range(0, max_level + 1):
        per_cell = n / float(4 ** (level + 1))
        if MIN_PER_CELL <= per_cell <= MAX_PER_CELL:
            out.append(level)
    if not out:  # tiny or huge systems: the depth closest to the band
        target = np.sqrt(MIN_PER_CELL * MAX_PER_CELL)
        out.append(int(np.clip(round(np.log(max(n, 1) / target) / np.log(4) - 1), 0, max_level)))
    return out


def _time_batch(engine, sysb, idx, level, steps, warmup, passes=4):
    import torch

    sizes = sysb.sizes()[idx]
    offsets = np.concatenate([[0], np.cumsum(sizes)])
    parts = [slice(int(sysb.offsets[i]), int(sysb.offsets[i + 1])) for i in idx]
    b = engine.Batch(offsets, [level] * len(idx), sysb.limits[idx], tick=sysb.dt, grav_const=sysb.grav_const,
                     epsilon=sysb.epsilon)
    b.set_item_passes([passes] * len(idx))
    prev = sysb.previous()
    b.position_cur[:] = torch.from_numpy(np.concatenate([sysb.position[p] for p in parts])).cuda()
    b.position_pre[:] = torch.from_numpy(np.concatenate([prev[p] for p in parts])).cuda()
    b.weight[:] = torch.from_numpy(np.concatenate([sysb.weight[p] for p in parts])).cuda()
    b.update(warmup)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    b.update(steps)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    b.close()
    return ms


def tune_levels(engine, sysb, sample: int = 16, steps: int = 3, warmup: int = 1, seed: int = 0):
    """Returns (num_levels per system, report per bucket)."""
    sizes = sysb.sizes()
    buckets = np.floor(np.log2(np.maximum(sizes, 1))).astype(int)
    levels = np.zeros(len(sizes), np.int32)
    report = {}
    rng = np.random.default_rng(seed)
    for bucket in sorted(set(buckets.tolist())):
        members = np.nonzero(buckets == bucket)[0]
        idx = np.sort(rng.choice(members, min(sample, len(members)), replace=False))
        cands = candidate_levels(int(np.median(sizes[members])))
        times = {lv: _time_batch(engine, sysb, idx, lv, steps, warmup) for lv in cands}
        best = min(times, key=times.get)
        levels[members] = best
        report[int(bucket)] = {"systems": int(len(members)), "candidates_ms": {int(k): v for k, v in times.items()},
                               "num_level": int(best)}
    return levels, report


def tune(engine, sysb, sample: int = 16, steps: int = 3, warmup: int = 1, seed: int = 0):
    """Depth and P2P tile per bucket. Returns (num_levels per system, item passes per system, report per bucket)."""
    sizes = sysb.sizes()
    buckets = np.floor(np.log2(np.maximum(sizes, 1))).astype(int)
    levels = np.zeros(len(sizes), np.int32)
    passes = np.full(len(sizes), 4, np.int32)
    report = {}
    rng = np.random.default_rng(seed)
    for bucket in sorted(set(buckets.tolist())):
        members = np.nonzero(buckets == bucket)[0]
        idx = np.sort(rng.choice(members, min(sample, len(members)), replace=False))
        cands = [(lv, p) for lv in candidate_levels(int(np.median(sizes[members]))) for p in ITEM_PASSES]
        times = {c: _time_batch(engine, sysb, idx, c[0], steps, warmup, c[1]) for c in cands}
        best = min(times, key=times.get)
        levels[members], passes[members] = best
        report[int(bucket)] = {"systems": int(len(members)),
                               "candidates_ms": {f"L{lv}/p{p}": v for (lv, p), v in times.items()},
                               "num_level": int(best[0]), "item_passes": int(best[1])}
    return levels, passes, report
