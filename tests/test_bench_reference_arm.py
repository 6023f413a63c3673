"""bench.py's reference arm on the CPU: the reference build's pair rate on a
small torus, printed as one JSON line with the metric, the lower-bound solve
time in seconds and the cpu_baseline / e2e records the driver reads (no GPU
needed; skipped where the reference build is absent)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def test_reference_arm_line():
    if not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libref_dirichlet.so")):
        pytest.skip("reference build absent")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--N", "64",
                        "--steps", "1", "--warmup", "1"], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
    assert line["impl"] == "reference" and line["unit"] == "s" and line["higher_is_better"] is False
    assert line["pair_rate_gpair_s"] > 0
    # the FP64 product count was measured on the 256^3 torus only: no
    # extrapolated solve time for another grid
    assert line["value"] is None
    import bench
    n = 581420
    expect = 67 * float(n) * n / (line["pair_rate_gpair_s"] * 1e9)
    assert abs(bench.cpu_solve_seconds(line["pair_rate_gpair_s"] * 1e9, n) - expect) <= 1e-9 * expect
    assert line["cpu_baseline"]["kind"] == "reference" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert bench.cpu_solve_seconds(1e9, n, 128, 20.0) is None
