"""CPU: bench.py's reference arm (the reference's algorithm restated, timed on the host cores) prints the contract's
JSON line, including across prunes of its window sample, and the modes without a reference counterpart say so."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def bench(*args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                       timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_reference_arm_line(orc):
    d = bench("--impl", "reference", "--steps", "2", "--warmup", "2")
    assert d["impl"] == "reference" and d["metric"] == "particle-steps/s" and d["unit"] == "particle-steps/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 2 and d["warmup"] == 2
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_reference_arm_of_modes_without_a_counterpart():
    for config in ("batched_512", "adjoint_262k"):
        d = bench("--impl", "reference", "--config", config, "--steps", "1", "--warmup", "0")
        assert d["impl"] == "reference" and "unavailable" in d
