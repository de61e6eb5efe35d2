"""CPU: the multi-rank path of the bench (replicas, no data-path collective) with world_size 2 over gloo.

Each rank steps its own replica of a small seeded system with the oracle's Stars::update, times it, and the
ranks agree on the maximum time and the whole-job rate through nbfmm_gb300.replicas, as the bench does under
torchrun on GPUs. The replicas must come out identical to a single-process run: nothing is exchanged."""
import os
import socket

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def replica_state(steps=3):
    """A 2,000-star disk stepped `steps` times by the oracle; returns (cur, prev, w, n)."""
    import sys

    sys.path.insert(0, os.path.dirname(HERE))
    from oracle import oracle as O

    rng = np.random.default_rng(17)
    n = 2000
    r = np.sqrt(rng.uniform(0.01, 1.0, n))
    a = rng.uniform(0, 2 * np.pi, n)
    cur = np.stack([r * np.cos(a), r * np.sin(a)], 1).astype(np.float32)
    prev = (cur * np.float32(0.999)).astype(np.float32)
    w = np.full(n, 1.0 / n, np.float32)
    lim = (-1.5, -1.5, 1.5, 1.5)
    for _ in range(steps):
        k, cur[:n], prev[:n], w[:n], _ = O.stars_update(cur[:n], prev[:n], w[:n], 3, lim, 1e-3, 1e-3)
        n = k
    return cur, prev, w, n


def rank_main(rank, world, port, out_dir):
    import time

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    from nbfmm_gb300 import replicas

    r, wsz, local = replicas.rank_info()
    assert (r, wsz, local) == (rank, world, rank)
    dist = replicas.init(wsz, "gloo")
    replicas.barrier(dist)
    t0 = time.perf_counter()
    cur, prev, w, n = replica_state()
    time.sleep(0.05 * (rank + 1))  # ranks finish at different times
    elapsed_ms = (time.perf_counter() - t0) * 1e3
    replicas.barrier(dist)
    slowest = replicas.max_over_ranks(elapsed_ms, dist)
    rate = replicas.whole_job_rate(2000 * 3, wsz, slowest)
    np.savez(os.path.join(out_dir, f"rank{rank}.npz"), cur=cur, prev=prev, w=w, n=n, elapsed=elapsed_ms,
             slowest=slowest, rate=rate)
    replicas.finish(dist)


def test_two_gloo_ranks_run_independent_replicas(tmp_path, orc):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    # `orc` has built and loaded the oracle here, so the two ranks only load it.
    port = free_port()
    mp.start_processes(rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    r0 = np.load(tmp_path / "rank0.npz")
    r1 = np.load(tmp_path / "rank1.npz")
    cur, prev, w, n = replica_state()
    for r in (r0, r1):
        assert int(r["n"]) == n
        np.testing.assert_array_equal(r["cur"], cur)
        np.testing.assert_array_equal(r["prev"], prev)
        np.testing.assert_array_equal(r["w"], w)
        assert float(r["slowest"]) == max(float(r0["elapsed"]), float(r1["elapsed"]))
        assert float(r["rate"]) == pytest.approx(2000 * 3 * 2 / (float(r["slowest"]) / 1e3))
    # each rank timed its own work, its sleep included (the ranks' compute times vary with the shared cores)
    assert float(r0["elapsed"]) >= 50.0 and float(r1["elapsed"]) >= 100.0


def test_one_rank_needs_no_process_group(monkeypatch):
    from nbfmm_gb300 import replicas

    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert replicas.rank_info() == (0, 1, 0)
    assert replicas.init(1, "gloo") is None
    assert replicas.max_over_ranks(3.5, None) == 3.5
    assert replicas.whole_job_rate(1000, 1, 500.0) == 2000.0
