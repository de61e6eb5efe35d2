"""CPU: the bench's roofline mirrors p2p.cu's reciprocal-series rule (which work items take the series, and how
many transcendental-unit operations a pair then costs). Both are read from the kernel source so they cannot drift."""
import os
import re
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def kernel_constants():
    src = open(os.path.join(ROOT, "nbfmm_gb300", "csrc", "p2p.cu")).read()
    max_v = float(re.search(r"constexpr float kSeriesMaxV = ([0-9.]+)f;", src).group(1))
    series_mask = int(re.search(r"#define NBFMM_P2P_SERIES_MASK (0x[0-9A-Fa-f]+)", src).group(1), 16)
    newton_mask = int(re.search(r"#define NBFMM_P2P_NEWTON_MASK (0x[0-9A-Fa-f]+)", src).group(1), 16)
    return max_v, series_mask, newton_mask


def test_bench_mirrors_the_series_rule_and_masks():
    import bench

    max_v, series_mask, newton_mask = kernel_constants()
    assert bench.SERIES_MAX_V == max_v
    # the square root always, the hardware reciprocal on the sources whose bit is clear in the mask
    assert bench.P2P_MUFU_PER_PAIR == 1 + (16 - bin(newton_mask).count("1")) / 16
    assert bench.P2P_MUFU_PER_PAIR_SERIES[2] == 1 + (16 - bin(series_mask).count("1")) / 16


def test_series_degree_of_the_measured_workloads():
    import bench
    from nbfmm_gb300 import workloads

    # the 16.8M two-disk step (and its fine capture case) take the series; the coarser configs do not
    expect = {"two_disks_16m": 2, "two_disks_4m_fine": 2, "two_disks_4m": 0, "disk_1m": 0, "plain_16k": 0}
    for name, degree in expect.items():
        sysm = workloads.CONFIGS[name]()
        assert bench.series_degree(sysm, "fast") == degree, name
        assert bench.series_degree(sysm, "exact") == 0, name
