"""GPU test of xpcs_multitau2_noalloc, the entry point for callers that cannot
allocate device memory (a framework-owned memory pool, a fixed GPU memory
budget, or a loop that must not call cudaMalloc/cudaFree).  Through the C ABI
it must give exactly what the allocating entry point xpcs_multitau2 gives,
on two calls in a row (the second reuses the fixed scratch the first left
behind).  Device buffers for the caller are made with torch here, as an
outside framework would provide them.  Collected last on purpose."""
import numpy as np
import pytest

import xpcs_gpu as xg
from fixtures import load, oracle_filter, same_bits

pytestmark = pytest.mark.gpu


def _rows(case):
    fx = load(case)
    _, rows, _ = oracle_filter(fx)
    return fx, rows


def _noalloc(torch, rows, frames, dpl, mode):
    dev = torch.device("cuda", 0)
    rp = torch.from_numpy(rows.row_ptr).to(dev)
    fr = torch.from_numpy(rows.frame).to(dev)
    va = torch.from_numpy(rows.value).to(dev)
    D = xg.delay_schedule(frames, dpl)[0].size
    out = torch.full((3, D, rows.pixels), float("nan"), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    xg.multitau2_noalloc(rp.data_ptr(), fr.data_ptr(), va.data_ptr(), rows.pixels,
                         int(rows.row_ptr[-1]), frames, dpl, mode, out[0].data_ptr(),
                         out[1].data_ptr(), out[2].data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize(dev)
    return out.cpu().numpy()


@pytest.mark.parametrize("mode", [xg.MODE_REFERENCE, xg.MODE_EXACT])
def test_noalloc_matches_allocating_entry_point_twice(mode):
    torch = pytest.importorskip("torch")
    torch.cuda.set_device(0)
    for case in ("sparse_quirk", "sparse_flat"):  # two calls in a row, different rows
        fx, rows = _rows(case)
        want = xg.multitau2(rows.row_ptr, rows.frame, rows.value, fx["F"], fx["dpl"], mode)
        got = _noalloc(torch, rows, fx["F"], fx["dpl"], mode)
        for k in range(3):
            assert same_bits(got[k], want[k]), (case, k)


def test_noalloc_rejects_more_events_than_its_scratch():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    rp = torch.zeros(2, dtype=torch.int64, device=dev)
    fr = torch.zeros(1, dtype=torch.int32, device=dev)
    out = torch.zeros(1, dtype=torch.float32, device=dev)
    with pytest.raises(xg.XpcsError) as e:
        xg.multitau2_noalloc(rp.data_ptr(), fr.data_ptr(), fr.data_ptr(), 1,
                             xg.NOALLOC_MAX_EVENTS + 1, 100, 4, 0, out.data_ptr(),
                             out.data_ptr(), out.data_ptr(), 0)
    assert e.value.code == 1
