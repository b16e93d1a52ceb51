"""bench.py pieces that run without a GPU: the reference arm's JSON line (the
oracle timed on the host cores, as `bench.py --impl reference` prints it) and
the reference-algorithm flop model behind the roofline."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1", "--cpu-cols", "8"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["unit"] == line["unit"]


def test_flop_model_worked_example():
    # one Fourier term at N = 8, L = 72, K = 16: about 3.35 MFLOP, plus the
    # single-scatter term L (2K + 60)
    f = bench.alg_flops(8, 72, 0, K=16) - 72 * (2 * 16 + 60)
    assert 3.3e6 < f < 3.45e6
    # each further term adds its own count; later terms have fewer moments
    f1 = bench.alg_flops(8, 72, 1, K=16) - bench.alg_flops(8, 72, 0, K=16)
    assert 0 < f1 < f
