"""Batches (xpcs_batch_*): several series of uneven shapes run as one CUDA
graph.  Each member's G2/IP/IF and g2/stderr (float64 and float32) must be
bit-identical to the same series run alone, the graph replay must repeat
them, a member whose frames change must be recaptured, and golden members
must still match the reference's own outputs."""
import numpy as np
import pytest

import xpcs_gpu as xg
import xpcs_synth as xs
from fixtures import load, same_bits, same_bits_nan

pytestmark = pytest.mark.gpu

# uneven members: detector side, frames, mean photons/pixel/frame, delays per level, tau range
MIX = [(64, 300, 0.02, 4, (2, 50)), (96, 1500, 0.004, 8, (5, 300)), (48, 4000, 0.01, 8, (10, 900)),
       (128, 600, 0.05, 4, (2, 20)), (80, 2500, 0.03, 8, (20, 2000)), (40, 200, 0.2, 4, (2, 10))]


def synth_member(i, side, F, mean, dpl, tau, seed_shift=0):
    acq = xs.Acquisition(width=side, height=side, frames=F, n_static=12, n_dynamic=6, mean=mean,
                         tau_min=tau[0], tau_max=tau[1], seed=100 + i + seed_shift, dpl=dpl)
    dq, sq, _, _ = xs.maps(acq)
    nnz, idx, val = xs.sparse_frames(acq)
    return acq, dq, sq, (nnz, idx, val)


def open_member(acq, dq, sq, frames):
    s = xg.Series(acq.width, acq.height, acq.frames, acq.dpl, dq, sq)
    s.ingest_sparse(*frames)
    return s


def golden_member(name):
    fx = load(name)
    if fx["dense"]:
        nd = fx["ndark"]
        s = xg.Series(fx["W"], fx["H"], fx["F"], fx["dpl"], fx["dqmap"], fx["sqmap"],
                      flatfield=fx["flatfield"], static_window=fx["swin"], dense=True,
                      lld=float(fx["lld_sigma"][0]), sigma=float(fx["lld_sigma"][1]))
        s.set_dark(fx["raw"][:nd])
        s.ingest_dense(fx["raw"][nd:])
    else:
        s = xg.Series(fx["W"], fx["H"], fx["F"], fx["dpl"], fx["dqmap"], fx["sqmap"],
                      flatfield=fx["flatfield"], stride=fx["stride"], average=fx["avg"],
                      static_window=fx["swin"])
        s.ingest_sparse(fx["nnz"], fx["idx"], fx["val"])
    return fx, s


def results(s, f32=True):
    G2, IP, IF = s.g2ipif()
    g64, s64, g32, s32 = s.normalized(f64=True, f32=f32)
    return dict(G2=G2, IP=IP, IF=IF, g64=g64, s64=s64, g32=g32, s32=s32)


def alone(s, mode):
    s.multitau(mode)
    s.normalize()
    return results(s)


def assert_same(a, b):
    for k in ("G2", "IP", "IF"):
        assert same_bits(a[k], b[k]), k
    for k in ("g64", "s64", "g32", "s32"):
        if a[k] is not None and b[k] is not None:
            assert same_bits_nan(a[k], b[k]), k


@pytest.mark.parametrize("mode", [xg.MODE_REFERENCE, xg.MODE_EXACT])
def test_batch_equals_each_series_alone(mode):
    members = [open_member(*synth_member(i, *m)) for i, m in enumerate(MIX)]
    goldens = [golden_member(n) for n in ("sparse_quirk", "sparse_stride_avg", "dense_dark")]
    series = members + [s for _, s in goldens]
    try:
        solo = [alone(s, mode) for s in series]
        with xg.Batch(series) as b:
            b.run(mode, f64=True, f32=True)
            ms, kernels, _ = b.stats()
            assert ms > 0 and kernels >= 10 * len(series)
            for s, r in zip(series, solo):
                assert_same(results(s), r)
            b.run(mode, f64=True, f32=True)  # graph replay
            for s, r in zip(series, solo):
                assert_same(results(s), r)
        if mode == xg.MODE_REFERENCE:
            for fx, s in goldens:
                r = results(s)
                for k in ("G2", "IP", "IF"):
                    assert same_bits(r[k], fx["ref_" + k]), k
                assert same_bits_nan(r["g32"], fx["ref_norm_0_g2"])
                assert same_bits_nan(r["s32"], fx["ref_norm_0_stderr"])
    finally:
        for s in series:
            s.close()


def test_batch_recaptures_when_a_member_changes():
    built = [synth_member(i, *m) for i, m in enumerate(MIX[:3])]
    series = [open_member(a, d, q, f) for a, d, q, f in built]
    try:
        with xg.Batch(series) as b:
            b.run()
            first = [results(s, f32=False) for s in series]
            # new frames for member 1 (same maps): the batch must notice and capture again
            _, _, _, frames = synth_member(1, *MIX[1], seed_shift=50)
            acq, dq, sq, _ = built[1]
            series[1].reset()
            series[1].ingest_sparse(*frames)
            b.run()
            changed = results(series[1], f32=False)
            assert not same_bits(changed["G2"], first[1]["G2"])
            for k in (0, 2):
                assert_same(results(series[k], f32=False), first[k])
            with open_member(acq, dq, sq, frames) as ref:
                r = alone(ref, xg.MODE_REFERENCE)
            for k in ("G2", "IP", "IF", "g64", "s64"):
                assert same_bits_nan(changed[k], r[k]), k
            # float32 normalisation was not requested in this run
            with pytest.raises(xg.XpcsError):
                series[0].normalized(f64=False, f32=True)
    finally:
        for s in series:
            s.close()


def test_autotune_changes_time_not_results():
    series = [open_member(*synth_member(i, *m)) for i, m in enumerate(MIX[:4])]
    try:
        before = [alone(s, xg.MODE_REFERENCE) for s in series]
        caps = [s.autotune() for s in series]
        assert all(c in (32, 48, 64, 80, 112) for c in caps)
        for s, r in zip(series, before):
            assert_same(alone(s, xg.MODE_REFERENCE), r)
        fresh = [open_member(*synth_member(i, *m)) for i, m in enumerate(MIX[4:], start=4)]
        solo = [alone(s, xg.MODE_REFERENCE) for s in fresh]
        with xg.Batch(series + fresh) as b:
            b.run(autotune=True, f32=True)
            for s, r in zip(series + fresh, before + solo):
                assert_same(results(s), r)
        for s in fresh:
            s.close()
    finally:
        for s in series:
            s.close()


def test_framesum_series_cannot_join_a_batch():
    fx, s = golden_member("sparse_quirk")
    fs = xg.Series(fx["W"], fx["H"], fx["F"], fx["dpl"], fx["dqmap"], fx["sqmap"],
                   normalize_by_framesum=True)
    try:
        with pytest.raises(xg.XpcsError):
            xg.Batch([s, fs])
    finally:
        s.close()
        fs.close()


def test_batch_timeline_covers_every_member():
    data = [synth_member(i, *m) for i, m in enumerate(MIX)]
    series = [open_member(*d) for d in data]
    try:
        b = xg.Batch(series)
        with pytest.raises(xg.XpcsError):
            b.timeline()  # not run yet
        b.run(xg.MODE_REFERENCE, f64=True)
        start, end = b.timeline()
        ms = b.stats()[0]
        assert start.shape == (len(series),) and np.all(start >= 0) and np.all(end > start)
        # every member's work lies inside the graph's run (timer resolution slack)
        assert float(np.max(end)) <= ms + 0.05
        b.close()
    finally:
        for s in series:
            s.close()


@pytest.mark.parametrize("mode", [xg.MODE_REFERENCE, xg.MODE_EXACT])
def test_every_knob_setting_gives_the_same_bits(mode):
    """Row capacity (warps per pixel), scratch words (level-fold schedule) and
    transpose tile change the work, never the results; bad values are refused."""
    members = [synth_member(i, *m) for i, m in enumerate(MIX[:3])]
    for acq, dq, sq, frames in members:
        s = open_member(acq, dq, sq, frames)
        try:
            ref = alone(s, mode)
            for cap, extra, ipt in ((32, 0, 8), (48, 8, 16), (64, 8, 0), (112, 0, 16),
                                    (80, 8, 8)):
                s.set_tuning(cap, extra, ipt)
                assert s.tuning() == {"thread_cap": cap, "scratch_extra": extra,
                                      "radix_items_per_lane": ipt}
                assert_same(alone(s, mode), ref)
            s.autotune(mode)
            t = s.tuning()
            assert t["thread_cap"] in (32, 48, 64, 80, 112) and t["scratch_extra"] in (0, 8)
            assert t["radix_items_per_lane"] in (8, 16)
            assert_same(alone(s, mode), ref)
            for bad in ((40, 0, 0), (80, 4, 0), (80, 0, 12)):
                with pytest.raises(xg.XpcsError):
                    s.set_tuning(*bad)
        finally:
            s.close()


LONG_ROWS = [(48, 4000, 0.15, 8, (10, 300)), (24, 8000, 0.25, 8, (5, 800))]


@pytest.mark.parametrize("queue", [True, False])
def test_both_batch_forms_equal_each_series_alone(queue):
    """The work-queue form (multi-tau of every member as persistent launches
    pulling 32-pixel groups and rows from device counters) and the chains form
    give each member the bits it gets alone: rows of every kernel class, from
    short thread-per-pixel rows to 1,000-4,000-event warp-per-pixel rows and
    float rows (flatfield, dense)."""
    members = [open_member(*synth_member(i, *m)) for i, m in enumerate(MIX + LONG_ROWS)]
    goldens = [golden_member(n) for n in ("sparse_flat", "dense_dark")]
    series = members + [s for _, s in goldens]
    try:
        solo = [alone(s, xg.MODE_REFERENCE) for s in series]
        with xg.Batch(series) as b:
            b.set_form(queue)
            b.run(xg.MODE_REFERENCE, f64=True, f32=True)
            assert b.form() == (queue, len(series))
            for s, r in zip(series, solo):
                assert_same(results(s), r)
            b.run(xg.MODE_REFERENCE, f64=True, f32=True, autotune=True)
            assert b.form()[0] == queue  # autotuning keeps the chosen form
            for s, r in zip(series, solo):
                assert_same(results(s), r)
            start, end = b.timeline()
            assert np.all(end > start)
    finally:
        for s in series:
            s.close()
