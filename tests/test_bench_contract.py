"""bench.py's output contract, checked without a GPU: the reference arm's JSON
line (the CPU restatement of the reference's path timed on the host) carries
every key the benchmark consumers read, and the GPU arm fails with an error
instead of falling back to the CPU when no GPU is usable."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SMALL = ["--width", "128", "--frames", "500"]


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def _run(args, timeout=300):
    return subprocess.run([sys.executable, str(ROOT / "bench.py")] + args, cwd=str(ROOT),
                          capture_output=True, text=True, timeout=timeout)


def test_reference_arm_json_line():
    r = _run(["--impl", "reference", "--steps", "1", "--warmup", "0"] + SMALL)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "multitau_frames_per_s" and d["unit"] == "frames/s"
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["higher_is_better"] is True and d["scaling"] == "weak"
    assert d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 0
    assert d["data"] == "synthetic" and "vs_baseline" in d
    assert d["config"]["workload"].startswith("128x128 detector, 500 sparse IMM frames")
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


@pytest.mark.skipif(_has_gpu(), reason="checks the behaviour without a usable GPU")
def test_gpu_arm_fails_loudly_without_a_gpu():
    r = _run(["--steps", "1", "--warmup", "0", "--width", "64", "--frames", "100"])
    assert r.returncode != 0
    assert not [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert "XpcsError" in r.stderr or "CUDA" in r.stderr
