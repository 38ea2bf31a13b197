"""bench.py's reference arm on CPU: one bounded step of the host-core Au
solver, printed as the contract's JSON line."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       cwd=ROOT, capture_output=True, text=True, timeout=300, check=True)
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "solves/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["n_gpus"] == 1 and line["steps"] == 1
    assert line["e2e"] == {"value": line["value"], "unit": "solves/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    assert line["config"]["workload"].startswith("4096 tiles x 64 vectors of 128x128")


def test_fp32_roofline_arithmetic():
    """The FP32-pipe figure of the roofline: the bench's last measured launch
    (1.73e10 node updates in 24.26 ms at 2070 MHz) is ~12% of the FMA rate."""
    sys.path.insert(0, ROOT)
    import bench
    r = bench.fp32_roofline(1.7314545664e10, 24.26, 2070.0)
    assert r["unit"] == "TFLOP/s" and abs(r["peak"] - 256 * 152 * 2070e6 / 1e12) < 1e-9
    assert abs(r["achieved"] - 14 * 1.7314545664e10 / 24.26e-3 / 1e12) < 1e-9
    assert 0.11 < r["frac"] < 0.13


def test_mixed_batch_cpu_baseline_combines_sizes_by_tile_share():
    """The mixed-size batch's host-core rate: each size timed on its own
    sample, the batch rate the harmonic combination weighted by tile shares
    (time per tile of the batch = sum of share x time per tile of each size)."""
    sys.path.insert(0, ROOT)
    import bench
    shares = {8: 3, 16: 1}
    r = bench.cpu_mixed_baseline(seconds_per_size=0.05, sizes=(8, 16), tiles_by_size=shares)
    rates = {int(k): v for k, v in r["by_size"].items()}
    assert set(rates) == {8, 16} and all(v > 0 for v in rates.values())
    assert rates[8] > rates[16]
    expect = 4.0 / (3.0 / rates[8] + 1.0 / rates[16])
    assert abs(r["value"] - expect) <= 1e-12 * expect
    assert min(rates.values()) <= r["value"] <= max(rates.values())
    assert r["kind"] == "port" and r["cores"] >= 1 and r["sample"].startswith("stratified: ")


def test_side_figure_reports_its_error_in_place():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.side_figure(lambda: {"x": 1}) == {"x": 1}
    r = bench.side_figure(lambda: {}["missing"])
    assert r == {"error": "KeyError: 'missing'"}
    with pytest.raises(KeyboardInterrupt):
        bench.side_figure(lambda: (_ for _ in ()).throw(KeyboardInterrupt()))
