"""GPU parity through the C ABI: libxpcs_gpu against the reference's own
outputs (golden fixtures) and against the oracle.

Bars: G2/IP/IF and the float32 g2/stderr bit-identical to the reference
(NaN positions compared as NaN); float64 g2/stderr within 1e-12 relative of
the float64 oracle evaluated on the same G2/IP/IF."""
import numpy as np
import pytest

import oracle
import xpcs_gpu as xg
import xpcs_synth as xs
from fixtures import (SPARSE_CASES, frames_of, load, max_rel_err, oracle_run, same_bits,
                      same_bits_nan)

pytestmark = pytest.mark.gpu

F64_TOL = 1e-12


def series_for(fx):
    return xg.Series(fx["W"], fx["H"], fx["F"], fx["dpl"], fx["dqmap"], fx["sqmap"],
                     flatfield=fx["flatfield"], stride=fx["stride"], average=fx["avg"],
                     static_window=fx["swin"], normalize_by_framesum=fx["framesum"])


def run_gpu(fx, mode=xg.MODE_REFERENCE, chunks=1):
    with series_for(fx) as s:
        for nnz, idx, val in frames_of(fx, chunks):
            s.ingest_sparse(nnz, idx, val)
        s.multitau(mode)
        G2, IP, IF = s.g2ipif()
        g64, s64, g32, s32 = s.normalize()
        info = s.info()
    return dict(G2=G2, IP=IP, IF=IF, g64=g64, s64=s64, g32=g32, s32=s32, info=info)


@pytest.mark.parametrize("case", SPARSE_CASES)
def test_g2ipif_bit_exact_vs_reference(case):
    fx = load(case)
    r = run_gpu(fx)
    for k in ("G2", "IP", "IF"):
        assert same_bits(r[k], fx["ref_" + k]), k


@pytest.mark.parametrize("case", SPARSE_CASES)
def test_normalize_f32_bit_exact_vs_reference(case):
    fx = load(case)
    r = run_gpu(fx)
    assert same_bits_nan(r["g32"], fx["ref_norm_0_g2"])
    assert same_bits_nan(r["s32"], fx["ref_norm_0_stderr"])


@pytest.mark.parametrize("case", SPARSE_CASES)
def test_normalize_f64_vs_oracle(case):
    fx = load(case)
    r = run_gpu(fx)
    qm = oracle.QMap(fx["dqmap"], fx["sqmap"])
    g64, s64 = oracle.normalize_f64(qm, fx["ref_G2"], fx["ref_IP"], fx["ref_IF"])
    assert max_rel_err(r["g64"], g64) <= F64_TOL
    assert max_rel_err(r["s64"], s64) <= F64_TOL


def test_exact_mode_vs_oracle():
    fx = load("sparse_quirk")
    r = run_gpu(fx, mode=xg.MODE_EXACT)
    o = oracle_run(fx, mode=1)
    for k in ("G2", "IP", "IF"):
        assert same_bits(r[k], o[k]), k
    assert (r["G2"] != fx["ref_G2"]).sum() > 0  # quirk Q1 is exercised


@pytest.mark.parametrize("case", SPARSE_CASES)
@pytest.mark.parametrize("mode", [xg.MODE_REFERENCE, xg.MODE_EXACT])
def test_multitau2_on_caller_rows(case, mode):
    fx = load(case)
    _, rows, _ = __import__("fixtures").oracle_filter(fx)
    G2, IP, IF = xg.multitau2(rows.row_ptr, rows.frame, rows.value, fx["F"], fx["dpl"], mode)
    oG2, oIP, oIF = oracle.multitau2(rows, fx["F"], fx["dpl"], mode)
    assert same_bits(G2, oG2) and same_bits(IP, oIP) and same_bits(IF, oIF)


def test_chunked_ingest_and_reset_are_identical():
    fx = load("sparse_stride_avg")
    a = run_gpu(fx, chunks=1)
    b = run_gpu(fx, chunks=7)
    for k in ("G2", "IP", "IF", "g32", "s32"):
        assert same_bits(a[k], b[k]), k
    with series_for(fx) as s:
        for _ in range(2):
            s.reset()
            for nnz, idx, val in frames_of(fx, 3):
                s.ingest_sparse(nnz, idx, val)
            s.multitau()
            G2, IP, IF = s.g2ipif()
            assert same_bits(G2, a["G2"]) and same_bits(IF, a["IF"])


@pytest.mark.parametrize("case", SPARSE_CASES)
def test_event_counts_match_oracle(case):
    fx = load(case)
    r = run_gpu(fx)
    _, rows, _ = __import__("fixtures").oracle_filter(fx)
    n = np.diff(rows.row_ptr)
    assert r["info"].events == int(n.sum())
    assert r["info"].valid_pixels == int((n > 0).sum())


def test_float_path_is_used_for_hot_and_flatfield_pixels():
    assert run_gpu(load("sparse_hot"))["info"].float_path_pixels >= 3
    assert run_gpu(load("sparse_flat"))["info"].float_path_pixels > 0
    assert run_gpu(load("sparse_basic"))["info"].float_path_pixels == 0


def test_pixel_index_out_of_range_is_an_input_error():
    fx = load("sparse_basic")
    with series_for(fx) as s:
        idx = fx["idx"].copy()
        idx[5] = fx["W"] * fx["H"] + 3
        s.ingest_sparse(fx["nnz"], idx, fx["val"])
        s.multitau()
        with pytest.raises(xg.XpcsError) as e:
            s.g2ipif()
        assert e.value.code == 6


def test_no_frames_gives_zero_correlations():
    fx = load("sparse_basic")
    with series_for(fx) as s:
        s.multitau()
        G2, IP, IF = s.g2ipif()
        g64, s64, g32, s32 = s.normalize()
    assert not G2.any() and not IP.any() and not IF.any()
    qm = oracle.QMap(fx["dqmap"], fx["sqmap"])
    og, os_ = oracle.normalize_f32(qm, G2, IP, IF)
    assert same_bits_nan(g32, og) and same_bits_nan(s32, os_)


def test_config0_full_size_vs_oracle():
    """512x512, 1000 frames, dpl 4 (the reference's CPU-runnable case)."""
    acq = xs.preset("c0")
    dq, sq, _, _ = xs.maps(acq)
    nnz, idx, val = xs.sparse_frames(acq)
    with xg.Series(acq.width, acq.height, acq.frames, acq.dpl, dq, sq) as s:
        s.ingest_sparse(nnz, idx, val)
        s.multitau()
        G2, IP, IF = s.g2ipif()
        g64, s64, g32, s32 = s.normalize()
    qm = oracle.QMap(dq, sq)
    rows, _ = oracle.sparse_filter(qm, nnz, idx, val, acq.frames)
    oG2, oIP, oIF = oracle.multitau2(rows, acq.frames, acq.dpl, 0)
    assert same_bits(G2, oG2) and same_bits(IP, oIP) and same_bits(IF, oIF)
    og, os_ = oracle.normalize_f32(qm, oG2, oIP, oIF)
    assert same_bits_nan(g32, og) and same_bits_nan(s32, os_)
    o64, s64o = oracle.normalize_f64(qm, oG2, oIP, oIF)
    assert max_rel_err(g64, o64) <= F64_TOL and max_rel_err(s64, s64o) <= F64_TOL


# ------------------------------------------------------------------ dense frames

def run_gpu_dense(fx, mode=xg.MODE_REFERENCE, chunks=1):
    nd = fx["ndark"]
    raw = fx["raw"]
    with xg.Series(fx["W"], fx["H"], fx["F"], fx["dpl"], fx["dqmap"], fx["sqmap"],
                   flatfield=fx["flatfield"], stride=fx["stride"], average=fx["avg"],
                   static_window=fx["swin"], dense=True, lld=float(fx["lld_sigma"][0]),
                   sigma=float(fx["lld_sigma"][1])) as s:
        if nd:
            s.set_dark(raw[:nd])
        data = raw[nd:]
        for part in np.array_split(data, chunks):
            s.ingest_dense(part)
        s.multitau(mode)
        G2, IP, IF = s.g2ipif()
        g64, s64, g32, s32 = s.normalize()
        avg, std = s.dark() if nd else (None, None)
        info = s.info()
    return dict(G2=G2, IP=IP, IF=IF, g64=g64, s64=s64, g32=g32, s32=s32, avg=avg, std=std,
                info=info)


def test_dense_bit_exact_vs_reference():
    fx = load("dense_dark")
    r = run_gpu_dense(fx)
    for k in ("G2", "IP", "IF"):
        assert same_bits(r[k], fx["ref_" + k]), k
    assert same_bits_nan(r["g32"], fx["ref_norm_0_g2"])
    assert same_bits_nan(r["s32"], fx["ref_norm_0_stderr"])
    assert r["info"].float_path_pixels > 0


def test_dense_dark_image_and_chunked_ingest():
    fx = load("dense_dark")
    nd = fx["ndark"]
    flat = fx["flatfield"].ravel() if fx["flatfield"] is not None else np.ones(fx["W"] * fx["H"])
    avg, std = oracle.dark_image(fx["raw"][:nd], flat)
    r = run_gpu_dense(fx, chunks=5)
    assert same_bits(r["avg"], avg) and same_bits(r["std"], std)
    one = run_gpu_dense(fx, chunks=1)
    for k in ("G2", "IP", "IF"):
        assert same_bits(r[k], one[k]), k


def test_dense_medium_vs_oracle():
    acq = xs.Acquisition(width=96, height=80, frames=700, n_static=12, n_dynamic=6, mean=0.05,
                         tau_min=5, tau_max=80, seed=31, dpl=8, dense=True, dark_frames=40,
                         gain_min=0.9, gain_max=1.1)
    dq, sq, flat, _ = xs.maps(acq)
    ds = xs.DenseStream(acq)
    raw = ds.next(acq.dark_frames + acq.frames)
    ds.close()
    lld, sigma = 0.0, 3.0
    with xg.Series(acq.width, acq.height, acq.frames, acq.dpl, dq, sq, flatfield=flat,
                   dense=True, lld=lld, sigma=sigma) as s:
        s.set_dark(raw[:acq.dark_frames])
        s.ingest_dense(raw[acq.dark_frames:])
        s.multitau()
        G2, IP, IF = s.g2ipif()
        g64, s64, g32, s32 = s.normalize()
    qm = oracle.QMap(dq, sq)
    da, dsd = oracle.dark_image(raw[:acq.dark_frames], flat.ravel())
    rows, _ = oracle.dense_filter(qm, raw[acq.dark_frames:], acq.frames, da, dsd, lld, sigma,
                                  flat=flat.ravel())
    oG2, oIP, oIF = oracle.multitau2(rows, acq.frames, acq.dpl, 0)
    assert same_bits(G2, oG2) and same_bits(IP, oIP) and same_bits(IF, oIF)
    og, os_ = oracle.normalize_f32(qm, oG2, oIP, oIF)
    assert same_bits_nan(g32, og) and same_bits_nan(s32, os_)


@pytest.mark.parametrize("mode,dpl", [(xg.MODE_REFERENCE, 8), (xg.MODE_EXACT, 8),
                                      (xg.MODE_REFERENCE, 4), (xg.MODE_REFERENCE, 16)])
def test_dense_long_float_rows_vs_oracle(mode, dpl):
    """Dark-subtracted, flat-fielded CCD rows of hundreds to thousands of float
    events (gain below 1 lifts the dark residual over the threshold): the
    warp-per-pixel float kernel on long, densely occupied rows."""
    acq = xs.Acquisition(width=40, height=36, frames=5000, n_static=12, n_dynamic=6, mean=0.03,
                         tau_min=3, tau_max=400, seed=41 + dpl, dpl=dpl, dense=True,
                         dark_frames=30, gain_min=0.85, gain_max=1.1)
    dq, sq, flat, _ = xs.maps(acq)
    ds = xs.DenseStream(acq)
    raw = ds.next(acq.dark_frames + acq.frames)
    ds.close()
    lld, sigma = 0.0, 3.0
    with xg.Series(acq.width, acq.height, acq.frames, acq.dpl, dq, sq, flatfield=flat,
                   dense=True, lld=lld, sigma=sigma) as s:
        s.set_dark(raw[:acq.dark_frames])
        s.ingest_dense(raw[acq.dark_frames:])
        s.multitau(mode)
        G2, IP, IF = s.g2ipif()
        info = s.info()
    qm = oracle.QMap(dq, sq)
    da, dsd = oracle.dark_image(raw[:acq.dark_frames], flat.ravel())
    rows, _ = oracle.dense_filter(qm, raw[acq.dark_frames:], acq.frames, da, dsd, lld, sigma,
                                  flat=flat.ravel())
    lens = np.diff(rows.row_ptr)
    assert info.float_path_pixels > 0 and lens.max() > 1500
    oG2, oIP, oIF = oracle.multitau2(rows, acq.frames, acq.dpl, mode)
    assert same_bits(G2, oG2) and same_bits(IP, oIP) and same_bits(IF, oIF)


def test_dense_stride_average_ragged_chunks_vs_oracle():
    """Dense frames with stride 2 and averaging over 3, a detector width whose
    rows are not a multiple of 8 pixels (no 16-byte loads), ingested in three
    uneven parts."""
    stride, avg, F = 2, 3, 150
    acq = xs.Acquisition(width=37, height=29, frames=F * stride * avg, n_static=8, n_dynamic=4,
                         mean=0.05, tau_min=3, tau_max=60, seed=19, dpl=4, dense=True,
                         dark_frames=20, gain_min=0.9, gain_max=1.1)
    dq, sq, flat, _ = xs.maps(acq)
    ds = xs.DenseStream(acq)
    raw = ds.next(acq.dark_frames + acq.frames)
    ds.close()
    data = raw[acq.dark_frames:]
    lld, sigma = 1.0, 2.5
    with xg.Series(acq.width, acq.height, F, acq.dpl, dq, sq, flatfield=flat, stride=stride,
                   average=avg, dense=True, lld=lld, sigma=sigma) as s:
        s.set_dark(raw[:acq.dark_frames])
        for a, b in ((0, 250), (250, 650), (650, data.shape[0])):
            s.ingest_dense(data[a:b])
        s.multitau()
        G2, IP, IF = s.g2ipif()
    qm = oracle.QMap(dq, sq)
    da, dsd = oracle.dark_image(raw[:acq.dark_frames], flat.ravel())
    rows, _ = oracle.dense_filter(qm, data, F, da, dsd, lld, sigma, stride=stride, average=avg,
                                  flat=flat.ravel())
    oG2, oIP, oIF = oracle.multitau2(rows, F, acq.dpl, 0)
    assert same_bits(G2, oG2) and same_bits(IP, oIP) and same_bits(IF, oIF)


@pytest.mark.parametrize("mode", [xg.MODE_REFERENCE, xg.MODE_EXACT])
def test_sparse_float_rows_with_stale_tail_misses_vs_oracle(mode):
    """Sparse counts times a flatfield are float rows; on these the reference's
    lower_bound over the out-of-order buffer misses some partners (the
    REFERENCE and EXACT results differ), which the float kernel reproduces."""
    acq = xs.Acquisition(width=64, height=64, frames=10000, n_static=12, n_dynamic=6,
                         mean=0.005, tau_min=5, tau_max=500, seed=5, dpl=8, gain_min=0.9,
                         gain_max=1.1)
    dq, sq, flat, _ = xs.maps(acq)
    nnz, idx, val = xs.sparse_frames(acq)
    with xg.Series(acq.width, acq.height, acq.frames, acq.dpl, dq, sq, flatfield=flat) as s:
        s.ingest_sparse(nnz, idx, val)
        s.multitau(mode)
        G2, IP, IF = s.g2ipif()
        info = s.info()
    qm = oracle.QMap(dq, sq)
    rows, _ = oracle.sparse_filter(qm, nnz, idx, val, acq.frames, flat=flat.ravel())
    assert info.float_path_pixels > 1000
    oG2, oIP, oIF = oracle.multitau2(rows, acq.frames, acq.dpl, mode)
    assert same_bits(G2, oG2) and same_bits(IP, oIP) and same_bits(IF, oIF)
    other = oracle.multitau2(rows, acq.frames, acq.dpl, 1 - mode)[0]
    assert np.count_nonzero(other != oG2) > 10  # the stale-tail searches matter here


# ------------------------------------------------------------- side statistics

def _side_gpu(fx):
    if fx["dense"]:
        nd = fx["ndark"]
        s = xg.Series(fx["W"], fx["H"], fx["F"], fx["dpl"], fx["dqmap"], fx["sqmap"],
                      flatfield=fx["flatfield"], stride=fx["stride"], average=fx["avg"],
                      static_window=fx["swin"], dense=True, lld=float(fx["lld_sigma"][0]),
                      sigma=float(fx["lld_sigma"][1]))
        if nd:
            s.set_dark(fx["raw"][:nd])
        s.ingest_dense(fx["raw"][nd:])
    else:
        s = series_for(fx)
        s.ingest_sparse(fx["nnz"], fx["idx"], fx["val"])
    with s:
        s.multitau()
        return s.side_stats(fx["swin"])


@pytest.mark.parametrize("case", [c for c in __import__("fixtures").CASES])
def test_side_statistics_bit_exact_vs_reference(case):
    fx = load(case)
    ps, fs, tot, part = _side_gpu(fx)
    assert same_bits_nan(ps, fx["ref_pixelSum"])
    assert same_bits_nan(fs, fx["ref_frameSum"])
    assert same_bits_nan(tot, fx["ref_partition_mean_total"])
    assert same_bits_nan(part, fx["ref_partition_mean_partial"])


@pytest.mark.parametrize("mode", [xg.MODE_REFERENCE, xg.MODE_EXACT])
def test_long_rows_take_the_integer_path_and_match_the_oracle(mode):
    """Rows of 300-2000 events (beyond the 256-event warp rows) are integer
    rows with sum |v| < 4096: the long-row warp kernel, not the float replay."""
    acq = xs.Acquisition(width=40, height=36, frames=20000, n_static=12, n_dynamic=6, mean=0.06,
                         tau_min=3, tau_max=3000, seed=77, dpl=8)
    dq, sq, _, _ = xs.maps(acq)
    nnz, idx, val = xs.sparse_frames(acq)
    with xg.Series(acq.width, acq.height, acq.frames, acq.dpl, dq, sq) as s:
        s.ingest_sparse(nnz, idx, val)
        s.multitau(mode)
        G2, IP, IF = s.g2ipif()
        info = s.info()
    qm = oracle.QMap(dq, sq)
    rows, _ = oracle.sparse_filter(qm, nnz, idx, val, acq.frames)
    lens = np.diff(rows.row_ptr)
    assert lens.max() > 256 and info.float_path_pixels == 0
    oG2, oIP, oIF = oracle.multitau2(rows, acq.frames, acq.dpl, mode)
    assert same_bits(G2, oG2) and same_bits(IP, oIP) and same_bits(IF, oIF)
