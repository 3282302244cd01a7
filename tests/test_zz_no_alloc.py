"""GPU tests of xpcs_multitau2_noalloc, the entry point for callers that cannot
allocate device memory: code running inside another framework's memory pool,
a process whose GPU memory budget is fixed up front, or an acquisition loop
that must never call cudaMalloc/cudaFree because those synchronise the device.

The test plays such a caller: it owns its device buffers (allocated here
through the CUDA runtime's C API) and passes raw device pointers through the
C ABI.  The entry point must give exactly what the allocating entry point
xpcs_multitau2 gives and what the oracle gives, on calls in a row (each call
reuses the fixed scratch the previous one left behind).  Collected last on
purpose, so that a run stopping at the first failure has run the rest."""
import numpy as np
import pytest

import devmem
import oracle
import xpcs_gpu as xg
from fixtures import load, oracle_filter, same_bits

pytestmark = pytest.mark.gpu


def _rows(case):
    fx = load(case)
    _, rows, _ = oracle_filter(fx)
    return fx, rows


def _noalloc(row_ptr, frame, value, frames, dpl, mode, events=None, fill=np.nan, whole=False):
    """One call on caller-owned device buffers; returns (G2, IP, IF) [D][P]
    (whole=True: the whole output buffer, at least one row per array)."""
    devmem.set_device(0)
    P = row_ptr.size - 1
    D = xg.delay_schedule(frames, dpl)[0].size
    events = int(row_ptr[-1]) if events is None else events
    out0 = np.full((3, max(D, 1), P), fill, np.float32)
    bufs = [devmem.Buffer.from_array(np.ascontiguousarray(row_ptr, np.int64)),
            devmem.Buffer.from_array(np.ascontiguousarray(frame, np.int32)),
            devmem.Buffer.from_array(np.ascontiguousarray(value, np.float32)),
            devmem.Buffer.from_array(out0)]
    st = devmem.Stream()
    try:
        rp, fr, va, out = bufs
        plane = 4 * max(D, 1) * P
        xg.multitau2_noalloc(rp.ptr, fr.ptr, va.ptr, P, events, frames, dpl, mode, out.ptr,
                             out.ptr + plane, out.ptr + 2 * plane, st.handle)
        st.synchronize()
        got = out.download(np.float32, out0.shape)
    finally:
        st.close()
        for b in bufs:
            b.free()
    return got if whole else got[:, :D, :]


@pytest.mark.parametrize("mode", [xg.MODE_REFERENCE, xg.MODE_EXACT])
def test_noalloc_matches_allocating_entry_point_and_oracle_on_calls_in_a_row(mode):
    for case in ("sparse_quirk", "sparse_flat", "sparse_quirk"):  # calls in a row
        fx, rows = _rows(case)
        want = xg.multitau2(rows.row_ptr, rows.frame, rows.value, fx["F"], fx["dpl"], mode)
        orc = oracle.multitau2(rows, fx["F"], fx["dpl"], mode)
        got = _noalloc(rows.row_ptr, rows.frame, rows.value, fx["F"], fx["dpl"], mode)
        for k in range(3):
            assert same_bits(got[k], want[k]), (case, k)
            assert same_bits(got[k], orc[k]), (case, k)


def test_noalloc_empty_rows_and_fewer_frames_than_one_delay():
    # pixels 0 and 3 without events; pixel 1 with one event; pixel 2 a short row
    row_ptr = np.array([0, 0, 1, 6, 6], np.int64)
    frame = np.array([3, 0, 2, 3, 7, 9], np.int32)
    value = np.array([2, 1, 1, 3, 1, 2], np.float32)
    rows = oracle.Rows(row_ptr, frame, value)
    for mode in (xg.MODE_REFERENCE, xg.MODE_EXACT):
        got = _noalloc(row_ptr, frame, value, 12, 2, mode)
        want = oracle.multitau2(rows, 12, 2, mode)
        for k in range(3):
            assert same_bits(got[k], want[k]), k
        assert not got[:, :, 0].any() and not got[:, :, 3].any()
    # one frame: no delay at all, so nothing is written to the outputs
    assert xg.delay_schedule(1, 4)[0].size == 0
    untouched = _noalloc(row_ptr, frame, value, 1, 4, xg.MODE_REFERENCE, fill=7.0, whole=True)
    assert np.all(untouched == 7.0)


def test_noalloc_row_pointers_outside_the_events_give_input_error_and_zero_rows():
    fx, rows = _rows("sparse_quirk")
    rp = rows.row_ptr.copy()
    P = rp.size - 1
    E = int(rp[-1])
    # pixel 5: a descending pointer (negative length); pixel P-1: past the events
    bad = [5, P - 1]
    rp[6] = rp[5] - 1 if rp[5] > 0 else rp[5]
    rp[5] = rp[6] + 1
    rp[P] = E + 10
    want = xg.multitau2(rows.row_ptr, rows.frame, rows.value, fx["F"], fx["dpl"], 0)
    with pytest.raises(xg.XpcsError) as e:
        _noalloc(rp, rows.frame, rows.value, fx["F"], fx["dpl"], 0, events=E)
    assert e.value.code == 6 and "row_ptr" in str(e.value)
    # the outputs of the call: bad rows zero, the others unchanged
    devmem.set_device(0)
    D = want[0].shape[0]
    bufs = [devmem.Buffer.from_array(rp), devmem.Buffer.from_array(rows.frame),
            devmem.Buffer.from_array(rows.value),
            devmem.Buffer.from_array(np.full((3, D, P), np.nan, np.float32))]
    try:
        with pytest.raises(xg.XpcsError):
            plane = 4 * D * P
            xg.multitau2_noalloc(bufs[0].ptr, bufs[1].ptr, bufs[2].ptr, P, E, fx["F"],
                                 fx["dpl"], 0, bufs[3].ptr, bufs[3].ptr + plane,
                                 bufs[3].ptr + 2 * plane, 0)
        got = bufs[3].download(np.float32, (3, D, P))
    finally:
        for b in bufs:
            b.free()
    for p in bad:
        assert not got[:, :, p].any()
    # the descending entry also makes row 6 start inside row 4: rows that share
    # scratch words with another row give unspecified values; the rest are exact
    lo6, hi6 = rp[6], rp[7]
    good = [p for p in range(P) if p not in bad and p != 6
            and rp[p] == rows.row_ptr[p] and rp[p + 1] == rows.row_ptr[p + 1]
            and (rp[p + 1] <= lo6 or rp[p] >= hi6)]
    assert len(good) > P - 10
    for k in range(3):
        assert same_bits(got[k][:, good], want[k][:, good])


def test_noalloc_rejects_more_events_or_delays_than_its_scratch():
    rp = np.array([0, 0], np.int64)
    with pytest.raises(xg.XpcsError) as e:
        _noalloc(rp, np.zeros(1, np.int32), np.zeros(1, np.float32), 100, 4, 0,
                 events=xg.NOALLOC_MAX_EVENTS + 1)
    assert e.value.code == 1 and "XPCS_NOALLOC_MAX_EVENTS" in str(e.value)
    # 64 delays per level over a million frames: 953 delays
    assert xg.delay_schedule(1_000_000, 64)[0].size > xg.NOALLOC_MAX_DELAYS
    devmem.set_device(0)
    bufs = [devmem.Buffer.from_array(rp), devmem.Buffer(16)]
    try:
        with pytest.raises(xg.XpcsError) as e:
            xg.multitau2_noalloc(bufs[0].ptr, bufs[1].ptr, bufs[1].ptr, 1, 0, 1_000_000, 64, 0,
                                 bufs[1].ptr, bufs[1].ptr, bufs[1].ptr, 0)
        assert e.value.code == 1 and "XPCS_NOALLOC_MAX_DELAYS" in str(e.value)
    finally:
        for b in bufs:
            b.free()
