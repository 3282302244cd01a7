"""CPU checks of the C ABI (no kernel launches): the library loads, exports
every function include/xpcs_gpu.h declares, and its host logic -- delay
schedule, partition-map validation, argument checks -- behaves."""
import re
from pathlib import Path

import numpy as np
import pytest

import oracle
import xpcs_gpu as xg

HEADER = Path(__file__).resolve().parent.parent / "include" / "xpcs_gpu.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(xpcs_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = xg.lib()
    names = declared_functions()
    assert names, "no declarations parsed"
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert sorted(xg.EXPORTS) == names


def test_abi_version():
    assert xg.lib().xpcs_abi_version() == 1


@pytest.mark.parametrize("frames", [1, 2, 3, 7, 8, 9, 15, 16, 17, 100, 257, 500, 1000, 4096,
                                    10000, 20000, 65535, 100000])
@pytest.mark.parametrize("dpl", [1, 2, 4, 8, 16])
def test_delay_schedule_matches_oracle(frames, dpl):
    lv, tau = xg.delay_schedule(frames, dpl)
    olv, otau = oracle.delays(frames, dpl)
    assert np.array_equal(lv, olv) and np.array_equal(tau, otau)


def test_delay_schedule_known_sizes():
    # D for the benchmark configurations
    assert xg.delay_schedule(1000, 4)[0].size == 34
    assert xg.delay_schedule(10000, 8)[0].size == 88
    assert xg.delay_schedule(20000, 8)[0].size == 96


def _desc_args(W=8, H=8):
    dq = np.ones((H, W), np.int32)
    sq = np.ones((H, W), np.int32)
    return W, H, dq, sq


def test_qmap_undercounted_static_partition_is_rejected():
    # Q5: static bin 2 only appears as the first pixel of dynamic bin 2, so the
    # reference's partition total stays 1 and it would index out of bounds
    W, H, dq, sq = _desc_args()
    dq[:] = 1
    sq[:] = 1
    dq[0, 0] = 2
    sq[0, 0] = 2
    with pytest.raises(xg.XpcsError) as e:
        xg.Series(W, H, 64, 4, dq, sq)
    assert e.value.code == 5
    assert oracle.QMap(dq, sq).error == 1


def test_qmap_noncontiguous_dynamic_bins_are_rejected():
    # Q7: g2 rows are sized by the number of q bins but indexed by q-1
    W, H, dq, sq = _desc_args()
    dq[:] = 3
    sq[:] = 1
    with pytest.raises(xg.XpcsError) as e:
        xg.Series(W, H, 64, 4, dq, sq)
    assert e.value.code == 5


def test_invalid_arguments():
    W, H, dq, sq = _desc_args()
    for kw in (dict(stride=0), dict(average=0)):
        with pytest.raises(xg.XpcsError) as e:
            xg.Series(W, H, 64, 4, dq, sq, **kw)
        assert e.value.code == 1
    with pytest.raises(xg.XpcsError):
        xg.Series(0, H, 64, 4, dq, sq)


def test_no_device_reported_cleanly():
    import shutil
    import subprocess
    smi = shutil.which("nvidia-smi")
    has_gpu = smi is not None and subprocess.run([smi, "-L"], capture_output=True).returncode == 0
    if has_gpu:
        pytest.skip("a GPU is present")
    W, H, dq, sq = _desc_args()
    with pytest.raises(xg.XpcsError) as e:
        xg.Series(W, H, 64, 4, dq, sq)
    assert e.value.code == 7
    assert "CUDA" in xg.lib().xpcs_last_error().decode()


def test_batch_rejects_bad_arguments():
    import ctypes as C
    h = C.c_void_p()
    rc = xg.lib().xpcs_batch_create(None, 0, C.byref(h))
    assert rc == 1 and h.value is None
    assert xg.lib().xpcs_batch_run(None, 0, 1) == 1
    xg.lib().xpcs_batch_destroy(None)


def test_server_needs_a_device():
    import ctypes as C
    import shutil
    if shutil.which("nvidia-smi"):
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    rc = xg.lib().xpcs_server_create(0, 1 << 30, C.byref(h))
    assert rc == 7 and h.value is None
    xg.lib().xpcs_server_destroy(None)
