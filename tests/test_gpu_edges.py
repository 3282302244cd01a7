"""Edge shapes through the C ABI against the oracle, bit for bit, in both modes:
a two-pixel detector, detectors whose pixel count is not a multiple of a warp
or a tile, fewer frames than delays per level, pixels with an event in every
frame (rows past the 4096-event warp rows go to the float-row kernel), more
than 65,536 frames (no packed integer rows), a fully masked detector and
frames without events.  A one-pixel detector is refused: BuildQMap raises the
static-partition total only from a bin's second pixel (quirk Q5), so the
reference would index past its partition arrays."""
import numpy as np
import pytest

import oracle
import xpcs_gpu as xg
from fixtures import same_bits, same_bits_nan

pytestmark = pytest.mark.gpu


def make(W, H, F, mean, seed, hot=(), mask_all=False, maxc=3, empty_every=0):
    """Sparse frames with one static/dynamic bin over the detector: per frame
    the pixels drawn with probability `mean` plus the `hot` pixels, counts in
    [1, maxc]; every `empty_every`-th frame has no events."""
    rng = np.random.default_rng(seed)
    P = W * H
    dq = np.full(P, 0 if mask_all else 1, np.int32)
    sq = dq.copy()
    nnz = np.zeros(F, np.uint32)
    idx, val = [], []
    for f in range(F):
        sel = np.flatnonzero(rng.random(P) < mean)
        sel = np.union1d(sel, np.asarray(hot, np.int64)).astype(np.int32)
        if empty_every and f % empty_every == 0:
            sel = sel[:0]
        nnz[f] = sel.size
        idx.append(sel)
        val.append(rng.integers(1, maxc + 1, sel.size).astype(np.int16))
    return (dq.reshape(H, W), sq.reshape(H, W), nnz, np.concatenate(idx).astype(np.int32),
            np.concatenate(val).astype(np.int16))


CASES = {
    "two_pixels": dict(W=2, H=1, F=50, mean=0.5, seed=1),
    "21_pixels_5_frames": dict(W=3, H=7, F=5, mean=0.3, seed=2),
    "561_pixels_2_frames": dict(W=33, H=17, F=2, mean=0.2, seed=3),
    "hot_rows_300": dict(W=40, H=40, F=300, mean=0.01, seed=4, hot=(5, 77, 1599)),
    "hot_row_9000": dict(W=16, H=16, F=9000, mean=0.001, seed=5, hot=(100,)),
    "70000_frames": dict(W=4, H=4, F=70000, mean=0.01, seed=6),
    "empty_frames": dict(W=8, H=8, F=100, mean=0.1, seed=7, empty_every=3),
    "masked": dict(W=8, H=8, F=60, mean=0.2, seed=8, mask_all=True),
}


@pytest.mark.parametrize("mode", [xg.MODE_REFERENCE, xg.MODE_EXACT])
@pytest.mark.parametrize("name", sorted(CASES))
def test_edge_shapes_vs_oracle(name, mode):
    c = dict(CASES[name])
    W, H, F = c.pop("W"), c.pop("H"), c.pop("F")
    dq, sq, nnz, idx, val = make(W, H, F, **c)
    dpl = 4
    with xg.Series(W, H, F, dpl, dq, sq) as s:
        s.ingest_sparse(nnz, idx, val)
        s.multitau(mode)
        G2, IP, IF = s.g2ipif()
        g64, s64, g32, s32 = s.normalize()
    qm = oracle.QMap(dq, sq)
    rows, _ = oracle.sparse_filter(qm, nnz, idx, val, F)
    oG2, oIP, oIF = oracle.multitau2(rows, F, dpl, mode)
    assert same_bits(G2, oG2) and same_bits(IP, oIP) and same_bits(IF, oIF)
    og, ose = oracle.normalize_f32(qm, oG2, oIP, oIF)
    assert same_bits_nan(g32, og) and same_bits_nan(s32, ose)


def test_one_pixel_detector_is_refused():
    dq, sq, _, _, _ = make(1, 1, 10, 0.5, 9)
    with pytest.raises(xg.XpcsError):
        xg.Series(1, 1, 10, 4, dq, sq)


# ------------------------------------------------------------------ dense frames

DENSE_CASES = {
    # detector 5 x 3: rows are not a multiple of 8 pixels (no 16-byte loads)
    "tiny_with_darks": dict(W=5, H=3, F=40, darks=6, lld=0.0, sigma=2.0, gain=(0.9, 1.1)),
    "one_frame": dict(W=16, H=8, F=1, darks=4, lld=0.0, sigma=1.0, gain=(1.0, 1.0)),
    "two_frames_no_darks_flat": dict(W=24, H=24, F=2, darks=0, lld=0.0, sigma=0.0,
                                     gain=(0.8, 1.2)),
    "no_darks_no_flat": dict(W=32, H=16, F=30, darks=0, lld=0.0, sigma=0.0, gain=(1.0, 1.0)),
    # a threshold above every value: no pixel is kept
    "nothing_kept": dict(W=16, H=16, F=20, darks=5, lld=30000.0, sigma=0.0, gain=(1.0, 1.0)),
}


@pytest.mark.parametrize("name", sorted(DENSE_CASES))
def test_dense_edge_shapes_vs_oracle(name):
    import xpcs_synth as xs

    c = DENSE_CASES[name]
    W, H, F, nd = c["W"], c["H"], c["F"], c["darks"]
    acq = xs.Acquisition(width=W, height=H, frames=F, n_static=4, n_dynamic=2, mean=0.2,
                         tau_min=3, tau_max=30, seed=60 + W + F, dpl=4, dense=True,
                         dark_frames=nd, gain_min=c["gain"][0], gain_max=c["gain"][1])
    dq, sq, flat, _ = xs.maps(acq)
    use_flat = c["gain"] != (1.0, 1.0)
    ds = xs.DenseStream(acq)
    raw = ds.next(nd + F)
    ds.close()
    with xg.Series(W, H, F, 4, dq, sq, flatfield=flat if use_flat else None, dense=True,
                   lld=c["lld"], sigma=c["sigma"]) as s:
        if nd:
            s.set_dark(raw[:nd])
        s.ingest_dense(raw[nd:])
        s.multitau()
        G2, IP, IF = s.g2ipif()
        info = s.info()
    qm = oracle.QMap(dq, sq)
    ones = np.ones(W * H)
    da, dsd = (oracle.dark_image(raw[:nd], flat.ravel() if use_flat else ones) if nd
               else (None, None))
    rows, _ = oracle.dense_filter(qm, raw[nd:], F, da, dsd, c["lld"], c["sigma"],
                                  flat=flat.ravel() if use_flat else None)
    oG2, oIP, oIF = oracle.multitau2(rows, F, 4, 0)
    assert same_bits(G2, oG2) and same_bits(IP, oIP) and same_bits(IF, oIF)
    if name == "nothing_kept":
        assert info.events == 0


def test_series_call_order_and_kind_errors():
    """Calls out of order, or for the other kind of frames, are refused with
    an error and leave the handle usable: the results that follow match the
    oracle."""
    import xpcs_synth as xs

    W, H, F = 12, 10, 200
    dq, sq, nnz, idx, val = make(W, H, F, 0.05, 70)
    with xg.Series(W, H, F, 4, dq, sq) as s:
        for call in (s.g2ipif, s.normalize, lambda: s.side_stats(20),
                     lambda: s.normalized(f64=True),
                     lambda: xg.check(xg.lib().xpcs_get_twotime(s._h, *[None] * 5))):
            with pytest.raises(xg.XpcsError):
                call()
        with pytest.raises(xg.XpcsError):
            s.set_dark(np.zeros((2, W * H), np.int16))  # darks are for dense series
        with pytest.raises(xg.XpcsError):
            s.ingest_dense(np.zeros((3, W * H), np.int16))
        s.ingest_sparse(nnz, idx, val)
        s.multitau()
        with pytest.raises(xg.XpcsError):
            s.normalized(f64=True)  # no normalisation has run yet
        G2, IP, IF = s.g2ipif()
        g64, s64, g32, s32 = s.normalize()
        n64, e64, _, _ = s.normalized(f64=True)
        assert same_bits_nan(n64, g64) and same_bits_nan(e64, s64)
    qm = oracle.QMap(dq, sq)
    rows, _ = oracle.sparse_filter(qm, nnz, idx, val, F)
    oG2, oIP, oIF = oracle.multitau2(rows, F, 4, xg.MODE_REFERENCE)
    assert same_bits(G2, oG2) and same_bits(IP, oIP) and same_bits(IF, oIF)

    acq = xs.Acquisition(width=8, height=8, frames=20, n_static=4, n_dynamic=2, mean=0.2,
                         tau_min=3, tau_max=30, seed=71, dpl=4, dense=True, dark_frames=2)
    dq, sq, _, _ = xs.maps(acq)
    ds = xs.DenseStream(acq)
    raw = ds.next(22)
    ds.close()
    with xg.Series(8, 8, 20, 4, dq, sq, dense=True, sigma=1.0) as s:
        with pytest.raises(xg.XpcsError):
            s.ingest_sparse(np.array([1], np.uint32), np.array([0], np.int32),
                            np.array([1], np.int16))
        s.set_dark(raw[:2])
        s.ingest_dense(raw[2:])
        with pytest.raises(xg.XpcsError):
            s.set_dark(raw[:2])  # darks come before the frames
        s.multitau()
        G2, IP, IF = s.g2ipif()
    qm = oracle.QMap(dq, sq)
    da, dsd = oracle.dark_image(raw[:2], np.ones(64))
    rows, _ = oracle.dense_filter(qm, raw[2:], 20, da, dsd, 0.0, 1.0, flat=None)
    oG2, oIP, oIF = oracle.multitau2(rows, 20, 4, 0)
    assert same_bits(G2, oG2) and same_bits(IP, oIP) and same_bits(IF, oIF)


@pytest.mark.parametrize("mode", [xg.MODE_REFERENCE, xg.MODE_EXACT])
@pytest.mark.parametrize("dpl", [1, 2, 3, 16])
def test_delays_per_level_vs_oracle(dpl, mode):
    """The delays per level decide which levels of the thread-per-pixel kernel
    take the bitmask pair search (at most 16 delays and 32 bins per scratch
    word) and which take the sparse search: dpl 1-3 give few scratch words,
    dpl 16 gives 32 delays at level 0.  Hot pixels put rows on the warp
    kernels too."""
    F = 3000
    dq, sq, nnz, idx, val = make(24, 20, F, 0.01, 80 + dpl, hot=(7, 300), maxc=3)
    with xg.Series(24, 20, F, dpl, dq, sq) as s:
        s.ingest_sparse(nnz, idx, val)
        s.multitau(mode)
        G2, IP, IF = s.g2ipif()
    qm = oracle.QMap(dq, sq)
    rows, _ = oracle.sparse_filter(qm, nnz, idx, val, F)
    oG2, oIP, oIF = oracle.multitau2(rows, F, dpl, mode)
    assert same_bits(G2, oG2) and same_bits(IP, oIP) and same_bits(IF, oIF)


def _signed_frames(F, P, mean, seed, big_pixel=None):
    """Sparse frames whose values are signed int16 (quirk Q3: counts above
    32767 read back negative); `big_pixel` gets values near the int16 limits."""
    rng = np.random.default_rng(seed)
    nnz = np.zeros(F, np.uint32)
    idx, val = [], []
    for f in range(F):
        sel = np.flatnonzero(rng.random(P) < mean).astype(np.int32)
        v = rng.choice(np.array([-3, -2, -1, 1, 2, 3], np.int16), sel.size)
        if big_pixel is not None and rng.random() < 0.01:
            sel = np.union1d(sel, [big_pixel]).astype(np.int32)
            v = rng.choice(np.array([-3, -2, -1, 1, 2, 3], np.int16), sel.size)
            v[np.searchsorted(sel, big_pixel)] = rng.choice(np.array([-32768, -30000, 32767],
                                                                     np.int16))
        nnz[f] = sel.size
        idx.append(sel)
        val.append(v.astype(np.int16))
    return nnz, np.concatenate(idx).astype(np.int32), np.concatenate(val).astype(np.int16)


@pytest.mark.parametrize("flat", [False, True])
def test_65536_frames_signed_values_vs_oracle(flat):
    """65,536 frames is the longest series whose radix items are packed
    (frame 65535 in the high half, the signed raw value in the low half); the
    flatfield is then applied as the events are written out."""
    F, W, H = 65536, 4, 4
    P = W * H
    nnz, idx, val = _signed_frames(F - 1, P, 0.0008, 90 + flat, big_pixel=5)
    # the last frame (65535) holds an event of every pixel
    extra_idx = np.arange(P, dtype=np.int32)
    extra_val = np.full(P, 2, np.int16)
    nnz = np.append(nnz, np.uint32(P))
    idx = np.concatenate([idx, extra_idx])
    val = np.concatenate([val, extra_val])
    dq = np.ones((H, W), np.int32)
    sq = dq.copy()
    g = np.random.default_rng(7).uniform(0.9, 1.1, (H, W)) if flat else None
    with xg.Series(W, H, F, 4, dq, sq, flatfield=g) as s:
        s.ingest_sparse(nnz, idx, val)
        s.multitau(xg.MODE_REFERENCE)
        G2, IP, IF = s.g2ipif()
    qm = oracle.QMap(dq, sq)
    rows, _ = oracle.sparse_filter(qm, nnz, idx, val, F,
                                   flat=g.ravel() if flat else None)
    oG2, oIP, oIF = oracle.multitau2(rows, F, 4, 0)
    assert same_bits(G2, oG2) and same_bits(IP, oIP) and same_bits(IF, oIF)


def test_stride_past_65536_raw_frames_vs_oracle():
    """Stride 2 over 40,000 filter frames reads 80,000 raw frames: the packed
    radix items carry the filter frame, which stays below 65,536."""
    F, W, H, stride = 40000, 6, 5, 2
    P = W * H
    nnz, idx, val = _signed_frames(F * stride, P, 0.002, 95)
    dq = np.ones((H, W), np.int32)
    sq = dq.copy()
    with xg.Series(W, H, F, 4, dq, sq, stride=stride) as s:
        s.ingest_sparse(nnz, idx, val)
        s.multitau(xg.MODE_REFERENCE)
        G2, IP, IF = s.g2ipif()
    qm = oracle.QMap(dq, sq)
    rows, _ = oracle.sparse_filter(qm, nnz, idx, val, F, stride=stride)
    oG2, oIP, oIF = oracle.multitau2(rows, F, 4, 0)
    assert same_bits(G2, oG2) and same_bits(IP, oIP) and same_bits(IF, oIF)


@pytest.mark.parametrize("odd_only", [True, False])
def test_stride_drops_events_vs_oracle(odd_only):
    """Stride 2 reads every other raw frame.  With events only in the skipped
    frames every event sorts last and the rows come out empty; otherwise the
    kept events interleave with dropped ones."""
    F, W, H, stride = 50, 6, 4, 2
    rng = np.random.default_rng(97)
    P = W * H
    nnz = np.zeros(F * stride, np.uint32)
    idx, val = [], []
    for r in range(F * stride):
        if odd_only and r % 2 == 0:
            continue
        sel = np.flatnonzero(rng.random(P) < 0.3).astype(np.int32)
        nnz[r] = sel.size
        idx.append(sel)
        val.append(rng.integers(1, 4, sel.size).astype(np.int16))
    idx = np.concatenate(idx).astype(np.int32)
    val = np.concatenate(val).astype(np.int16)
    dq = np.ones((H, W), np.int32)
    sq = dq.copy()
    with xg.Series(W, H, F, 4, dq, sq, stride=stride) as s:
        s.ingest_sparse(nnz, idx, val)
        s.multitau(xg.MODE_REFERENCE)
        G2, IP, IF = s.g2ipif()
        info = s.info()
    qm = oracle.QMap(dq, sq)
    rows, _ = oracle.sparse_filter(qm, nnz, idx, val, F, stride=stride)
    oG2, oIP, oIF = oracle.multitau2(rows, F, 4, 0)
    assert same_bits(G2, oG2) and same_bits(IP, oIP) and same_bits(IF, oIF)
    if odd_only:
        assert info.events == 0 and not G2.any() and not IP.any()
