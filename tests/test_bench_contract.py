"""bench.py's reporting contract, checked on the CPU.

The reference arm (`bench.py --impl reference`) times Owl's CPU algorithm for
the config-2 step -- the oracle, Owl's im2col + OpenBLAS strategy restated
in C -- on a bounded sample and prints one JSON line with the same metric,
unit and config as the GPU arm.  The step's FLOP count is the config's
arithmetic: 2*M*N*K per pass, three passes per layer."""

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_step_flops_follow_the_config_shapes():
    sys.path.insert(0, str(ROOT))
    import bench

    f = {name: bench.layer_flops(xs, ks, st, r, p) for name, xs, ks, st, r, p in bench.LAYERS}
    # L1: [64;56;56;128] * [3;3;128;128] SAME -> M = 64*56*56, N = 128, K = 1152
    assert f["L1"] == 2.0 * 64 * 56 * 56 * 128 * 1152
    # L2: [64;28;28;256] * [3;3;256;256] stride 2 VALID -> 13 x 13 outputs
    assert bench.out_shape(*bench.LAYERS[1][1:]) == (64, 13, 13, 256)
    assert f["L2"] == 2.0 * 64 * 13 * 13 * 256 * 2304
    # dilated L1 (rate 2, SAME) keeps the 56 x 56 output
    assert f["D"] == f["L1"]
    step = 3 * sum(f.values())
    assert abs(step / 1e9 - 393.417) < 0.01


def test_reference_arm_prints_one_json_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "3"],
                       capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "conv2d fwd+bwd TFLOP/s (config 2: L1+L2+dilated)"
    assert d["unit"] == "TFLOP/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] >= 3
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference")
    assert cb["cores"] >= 1 and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == "TFLOP/s"
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    assert "workload" in d["config"]
