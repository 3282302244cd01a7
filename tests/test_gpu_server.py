"""Serving (xpcs_server_*): acquisitions streamed frame by frame, admitted by
device-memory budget, with their work overlapping on the GPU.  Each result
must be bit-identical to the same series run alone through the series API,
whether the frames arrive interleaved from one thread or from one thread per
acquisition, and whether the acquisition waited for admission or not."""
import threading

import numpy as np
import pytest

import xpcs_gpu as xg
import xpcs_synth as xs
from fixtures import same_bits, same_bits_nan

pytestmark = pytest.mark.gpu

ACQS = [(64, 300, 0.02, 4, (2, 50)), (96, 900, 0.004, 8, (5, 300)), (48, 2000, 0.01, 8, (10, 900)),
        (80, 500, 0.05, 4, (2, 20)), (40, 1200, 0.2, 4, (2, 10))]


def make(i, side, F, mean, dpl, tau):
    acq = xs.Acquisition(width=side, height=side, frames=F, n_static=12, n_dynamic=6, mean=mean,
                         tau_min=tau[0], tau_max=tau[1], seed=300 + i, dpl=dpl)
    dq, sq, _, _ = xs.maps(acq)
    return acq, dq, sq, xs.sparse_frames(acq)


def alone(acq, dq, sq, frames, mode=xg.MODE_REFERENCE):
    with xg.Series(acq.width, acq.height, acq.frames, acq.dpl, dq, sq) as s:
        s.ingest_sparse(*frames)
        s.multitau(mode)
        G2, IP, IF = s.g2ipif()
        g2, se, _, _ = s.normalize(f64=True, f32=False)
    return g2, se, G2, IP, IF


def frame_slices(frames):
    nnz, idx, val = frames
    off = np.concatenate([[0], np.cumsum(nnz.astype(np.int64))])
    for t in range(nnz.size):
        yield nnz[t:t + 1], idx[off[t]:off[t + 1]], val[off[t]:off[t + 1]]


def check(res, ref):
    g2, se, G2, IP, IF = res
    rg2, rse, rG2, rIP, rIF = ref
    assert same_bits(G2, rG2) and same_bits(IP, rIP) and same_bits(IF, rIF)
    assert same_bits_nan(g2, rg2) and same_bits_nan(se, rse)


def test_interleaved_acquisitions_under_a_memory_budget():
    data = [make(i, *a) for i, a in enumerate(ACQS)]
    refs = [alone(*d) for d in data]
    # room for about two of these acquisitions at a time
    with xg.Server(memory_budget=150 << 20) as srv:
        ids, states = [], []
        for acq, dq, sq, fr in data:
            ids.append(srv.submit(acq.width, acq.height, acq.frames, acq.dpl, dq, sq,
                                  expected_events=fr[1].size))
            states.append(srv.state(ids[-1]))
        assert states[0] == "active" and "pending" in states
        gens = [frame_slices(fr) for _, _, _, fr in data]
        live = list(range(len(data)))
        while live:  # one frame of every live acquisition in turn
            for k in list(live):
                f = next(gens[k], None)
                if f is None:
                    srv.finish(ids[k])
                    live.remove(k)
                else:
                    srv.push(ids[k], *f)
            # free finished acquisitions as they complete so that waiting ones get in
            for k in range(len(data)):
                if ids[k] is not None and k not in live and srv.state(ids[k]) == "done":
                    check(srv.result(ids[k], g2ipif=True), refs[k])
                    srv.release(ids[k])
                    ids[k] = None
        for k in range(len(data)):
            if ids[k] is not None:
                check(srv.result(ids[k], g2ipif=True), refs[k])
                srv.release(ids[k])
        st = srv.stats()
        assert st["frames_ingested"] == sum(a.frames for a, _, _, _ in data)
        assert st["series_finished"] == len(data)
        assert st["peak_active"] >= 2 and st["active"] == 0 and st["pending"] == 0
        assert 0 < st["ingest_p50_ms"] <= st["ingest_p99_ms"]


def test_one_thread_per_acquisition():
    data = [make(i, *a) for i, a in enumerate(ACQS[:4])]
    refs = [alone(*d) for d in data]
    results = [None] * len(data)
    errors = []
    with xg.Server(memory_budget=8 << 30) as srv:
        def run(k):
            try:
                acq, dq, sq, fr = data[k]
                i = srv.submit(acq.width, acq.height, acq.frames, acq.dpl, dq, sq,
                               expected_events=fr[1].size)
                for f in frame_slices(fr):
                    srv.push(i, *f)
                srv.finish(i)
                results[k] = srv.result(i, g2ipif=True)
                srv.release(i)
            except Exception as e:  # reported below
                errors.append(e)

        th = [threading.Thread(target=run, args=(k,)) for k in range(len(data))]
        for t in th:
            t.start()
        for t in th:
            t.join()
        assert not errors, errors
        assert srv.stats()["series_finished"] == len(data)
    for r, ref in zip(results, refs):
        check(r, ref)


def test_errors_and_edge_cases():
    """Misuse is refused with an error and leaves the server usable: unknown
    ids, frames after finish, finish twice, results before finish.  An
    acquisition finished without frames gives the series' empty result; one
    larger than the whole budget is admitted when nothing else is active; a
    bad pixel index fails that acquisition only."""
    acq, dq, sq, frames = make(0, *ACQS[0])
    with xg.Server(memory_budget=256 << 20) as srv:
        with pytest.raises(xg.XpcsError):
            srv.state(12345)
        with pytest.raises(xg.XpcsError):
            srv.push(12345, *next(frame_slices(frames)))
        # no frames at all
        a = srv.submit(acq.width, acq.height, acq.frames, acq.dpl, dq, sq, 0)
        with pytest.raises(xg.XpcsError):
            srv.result(a)  # finish not called
        srv.finish(a)
        with pytest.raises(xg.XpcsError):
            srv.finish(a)
        with pytest.raises(xg.XpcsError):
            srv.push(a, *next(frame_slices(frames)))
        empty = (np.zeros(0, np.uint32), np.zeros(0, np.int32), np.zeros(0, np.int16))
        check(srv.result(a, g2ipif=True), alone(acq, dq, sq, empty))
        srv.release(a)
        # larger than the budget: admitted while nothing else is active
        big, bdq, bsq, bframes = make(1, 256, 400, 0.05, 8, (2, 40))
        b = srv.submit(big.width, big.height, big.frames, big.dpl, bdq, bsq,
                       int(bframes[1].size))
        for part in frame_slices(bframes):
            srv.push(b, *part)
        srv.finish(b)
        check(srv.result(b, g2ipif=True), alone(big, bdq, bsq, bframes))
        srv.release(b)
        # a pixel index past the detector fails this acquisition only
        c = srv.submit(acq.width, acq.height, acq.frames, acq.dpl, dq, sq, 10)
        d = srv.submit(acq.width, acq.height, acq.frames, acq.dpl, dq, sq,
                       int(frames[1].size))
        srv.push(c, np.array([1], np.uint32), np.array([acq.width * acq.height + 5], np.int32),
                 np.array([1], np.int16))
        for part in frame_slices(frames):
            srv.push(d, *part)
        srv.finish(c)
        srv.finish(d)
        with pytest.raises(xg.XpcsError):
            srv.result(c)
        check(srv.result(d, g2ipif=True), alone(acq, dq, sq, frames))
        srv.release(c)
        srv.release(d)


def test_close_after_finish_without_result():
    """Closing the server while acquisitions are finishing (finish called,
    result never read) waits for their work and frees them instead of
    deadlocking on the completion callback."""
    data = [make(i, *a) for i, a in enumerate(ACQS[:3])]
    srv = xg.Server(memory_budget=8 << 30)
    for acq, dq, sq, fr in data:
        i = srv.submit(acq.width, acq.height, acq.frames, acq.dpl, dq, sq,
                       expected_events=fr[1].size)
        srv.push(i, *fr)
        srv.finish(i)
    srv.close()  # returns: nothing waits on a lock the callbacks need
    # and a new server on the same device still works
    acq, dq, sq, fr = data[0]
    with xg.Server(memory_budget=8 << 30) as srv2:
        i = srv2.submit(acq.width, acq.height, acq.frames, acq.dpl, dq, sq,
                        expected_events=fr[1].size)
        srv2.push(i, *fr)
        srv2.finish(i)
        check(srv2.result(i, g2ipif=True), alone(acq, dq, sq, fr))
