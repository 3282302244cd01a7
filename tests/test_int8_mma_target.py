"""Why the two-time Gram uses fp16 operands and not int8: the 5th-generation
tensor cores of GB300 (sm_103a) have no integer MMA.  ptxas refuses
`tcgen05.mma ... kind::i8` for sm_103a, while it accepts it for sm_100a (B200).
Compile-only, no GPU: the probe kernel (tests/probes/tcgen05_kind_i8.cu) is
never launched."""
import shutil
import subprocess
from pathlib import Path

import pytest

NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
PROBE = Path(__file__).resolve().parent / "probes" / "tcgen05_kind_i8.cu"


def _compile(arch, tmp_path):
    return subprocess.run([NVCC, "-gencode", f"arch=compute_{arch},code=sm_{arch}", "-c",
                           str(PROBE), "-o", str(tmp_path / f"probe_{arch}.o")],
                          capture_output=True, text=True, timeout=300)


@pytest.mark.skipif(not Path(NVCC).exists(), reason="nvcc not found")
def test_tcgen05_kind_i8_is_not_available_on_sm_103a(tmp_path):
    r = _compile("103a", tmp_path)
    assert r.returncode != 0
    assert "kind::i8" in r.stderr and "sm_103a" in r.stderr, r.stderr
    # the same source is valid on sm_100a: the refusal is the target's
    assert _compile("100a", tmp_path).returncode == 0
