"""The integer evaluation of the filters' double-rounded expressions
(csrc/f64emu.cuh) against double arithmetic on the host."""
import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent
CSRC = HERE.parent / "xpcs-eigen_gb300" / "csrc"


def test_f64emu_matches_double_arithmetic(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "f64emu_check"
    subprocess.run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I", str(CSRC),
                    str(HERE / "f64emu_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    mism, fallb, dr, checked = (int(x) for x in out.stdout.split()[-4:])
    assert mism == 0, out.stdout
    # every operand drawn lies in the handled range
    assert fallb == 0, out.stdout
    # the constructed cases do reach results where double rounding decides
    assert dr > 1000, out.stdout
    assert checked > 80_000_000
