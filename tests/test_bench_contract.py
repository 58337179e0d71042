"""The bench's CPU-side pieces: the reference arm's JSON line (the CPU FP64 restatement on the host cores,
a small sample here) and the training step's byte model."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--ref-cells", "2048",
                        "--steps", "2", "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["unit"] == "cells/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["config"]["cells_per_step"] == 2048 and line["steps"] == 2


def test_training_step_byte_model():
    sys.path.insert(0, ROOT)
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    B, W, H = 65536, 256, 4
    n_params = (64 * W + (H - 1) * W * W + W * 64) + H * W + 64
    total = bench.train_step_bytes(B, 64, W, H, 64, n_params)
    act = B * W * 2
    # at least every hidden activation written (silu and silu') and read back by two GEMMs
    assert total > H * 2 * act + H * 2 * act
    # and below a few times the activations' bytes (no quadratic terms)
    assert total < 12 * H * act
    # linear in the batch plus a batch-independent part (split-K partials, optimizer state) of at most a
    # fifth of the step's traffic at this batch
    fixed = 2 * total - bench.train_step_bytes(2 * B, 64, W, H, 64, n_params)
    assert 0 < fixed < 0.2 * total
