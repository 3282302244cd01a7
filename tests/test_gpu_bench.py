"""bench.py's GPU arm on a small series: one JSON line with the keys the
benchmark consumers read (device-timed value, end-to-end value with its copy
bytes, roofline of the multi-tau kernel, clocks, kernel launch count, CPU
baseline)."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def test_gpu_arm_json_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--steps", "2", "--warmup", "3",
                        "--width", "128", "--frames", "1000",
                        "--no-batch", "--no-serving", "--no-twotime", "--no-dense", "--no-corr"],
                       cwd=str(ROOT), capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["metric"] == "multitau_frames_per_s" and d["unit"] == "frames/s"
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["n_gpus"] == 1
    assert d["steps"] == 2 and d["warmup"] == 3 and d["higher_is_better"] is True
    assert d["config"]["workload"].startswith("128x128 detector, 1000 sparse IMM frames")
    e2e = d["e2e"]
    assert e2e["value"] > 0 and e2e["unit"] == "frames/s"
    assert e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] > 0
    rf = d["roofline"]
    assert rf["bound"] == "hbm" and rf["unit"] == "GB/s"
    assert rf["achieved"] > 0 and rf["peak"] > 0
    assert abs(rf["frac"] - rf["achieved"] / rf["peak"]) < 1e-9
    assert "traffic" in rf
    assert d["clocks"]["sm_mhz"] > 0 and d["clocks"]["sm_max_mhz"] > 0
    assert isinstance(d["clocks"]["reasons"], list)
    assert d["gpu_launches"] > 0
    cb = d["cpu_baseline"]
    assert cb["value"] > 0 and cb["kind"] == "port" and cb["cores"] >= 1
    assert "whole 1000-frame" in cb["sample"]
    # the reference arm reports the identical config object for the same series
    ref = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "0", "--width", "128", "--frames", "1000"],
                         cwd=str(ROOT), capture_output=True, text=True, timeout=600)
    assert ref.returncode == 0, ref.stderr[-2000:]
    rd = json.loads([l for l in ref.stdout.splitlines() if l.startswith("{")][0])
    assert rd["config"] == d["config"]
