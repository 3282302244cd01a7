"""Parity at the benchmark configurations themselves, through the C ABI.

* 1024x1024 detector, 10,000 sparse frames (Poisson speckle, mean 0.005
  photons/pixel/frame, tau_c log-uniform [5, 500] per ring, 36/18 rings,
  8 delays per level; D = 88, ~52 M events): every one of the 88 x 1 Mi
  G2/IP/IF cells bit for bit against the oracle's Corr::multiTau2
  (src/xpcs/corr.cpp:315-431), in both search modes; the float32 g2/stderr
  bit for bit and the float64 g2/stderr within 1e-12 (relative) of the
  oracle's Corr::normalizeG2s (:927-1091).
* 960x960 dense CCD frames, 100 darks + 20,000 frames (dark N(100, 8^2), read
  noise 4 ADU, 35 ADU/photon at 0.02 photons/pixel/frame, gain U[0.9, 1.1],
  3-sigma threshold, 8 delays per level; ~1.35 G kept events, D = 96): the
  dark image (DarkImage::Compute, dark_image.cpp:81-106) bit for bit at every
  pixel, and G2/IP/IF bit for bit on a seeded 1-in-64 sample of pixels whose
  oracle rows come from DenseFilter::Apply restated (dense_filter.cpp:
  121-210) on exactly the frames the GPU read.

The frames are drawn on the GPU by the seeded generator and copied back, so
the oracle sees the very input the library processed.  Each case takes about
a minute, most of it the oracle on the host cores."""
import numpy as np
import pytest

import oracle
import xpcs_gpu as xg
import xpcs_synth as xs
from fixtures import max_rel_err, same_bits, same_bits_nan

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c1():
    acq = xs.preset("c1")
    dq, sq, _, _ = xs.maps(acq)
    d = xs.DeviceFrames(acq)
    nnz, idx, val = d.to_host()
    d.close()
    qm = oracle.QMap(dq, sq)
    rows, _ = oracle.sparse_filter(qm, nnz, idx, val, acq.frames, finish=False)
    return dict(acq=acq, dq=dq, sq=sq, nnz=nnz, idx=idx, val=val, qm=qm, rows=rows)


def _gpu_c1(c, mode):
    acq = c["acq"]
    with xg.Series(acq.width, acq.height, acq.frames, acq.dpl, c["dq"], c["sq"], device=0) as s:
        s.ingest_sparse(c["nnz"], c["idx"], c["val"])
        s.multitau(mode)
        G2, IP, IF = s.g2ipif()
        g64, s64, g32, s32 = s.normalize(f64=True, f32=True)
        info = s.info()
    return G2, IP, IF, g64, s64, g32, s32, info


def test_c1_headline_series_bit_exact(c1):
    acq = c1["acq"]
    G2, IP, IF, g64, s64, g32, s32, info = _gpu_c1(c1, xg.MODE_REFERENCE)
    assert G2.shape == (88, 1024 * 1024)
    assert info.events == c1["rows"].row_ptr[-1] and info.float_path_pixels == 0
    oG2, oIP, oIF = oracle.multitau2(c1["rows"], acq.frames, acq.dpl, 0)
    for name, got, want in (("G2", G2, oG2), ("IP", IP, oIP), ("IF", IF, oIF)):
        assert same_bits(got, want), (name, int(np.count_nonzero(got != want)))
    o32g, o32s = oracle.normalize_f32(c1["qm"], oG2, oIP, oIF)
    assert same_bits_nan(g32, o32g) and same_bits_nan(s32, o32s)
    o64g, o64s = oracle.normalize_f64(c1["qm"], oG2, oIP, oIF)
    assert max_rel_err(g64, o64g) <= 1e-12
    assert max_rel_err(s64, o64s) <= 1e-12


def test_c1_headline_series_exact_mode(c1):
    acq = c1["acq"]
    G2, IP, IF, *_ = _gpu_c1(c1, xg.MODE_EXACT)
    oG2, oIP, oIF = oracle.multitau2(c1["rows"], acq.frames, acq.dpl, 1)
    for name, got, want in (("G2", G2, oG2), ("IP", IP, oIP), ("IF", IF, oIF)):
        assert same_bits(got, want), (name, int(np.count_nonzero(got != want)))


def test_c2_dense_series_dark_and_sampled_pixels_bit_exact():
    acq = xs.preset("c2")
    dq, sq, flat, _ = xs.maps(acq)
    F, P, nd = acq.frames, acq.width * acq.height, acq.dark_frames
    flat = np.ascontiguousarray(flat.ravel(), np.float64)
    frames = xs.DeviceDenseFrames(acq)
    try:
        darks = frames.to_host(0, nd)
        with xg.Series(acq.width, acq.height, F, acq.dpl, dq, sq, flatfield=flat, device=0,
                       dense=True, lld=acq.lld, sigma=acq.sigma) as s:
            s.set_dark(darks)
            s.ingest_dense_device(frames.frame_ptr(nd), F)
            s.multitau(xg.MODE_REFERENCE)
            G2, IP, IF = s.g2ipif()
            dark_avg, dark_std = s.dark()
            info = s.info()
        # the sampled pixels' raw values over every data frame, from the device copy
        rng = np.random.default_rng(64)
        sample = np.sort(rng.choice(P, size=P // 64, replace=False))
        raw = np.empty((F, sample.size), np.int16)
        step = 1000
        for f0 in range(0, F, step):
            n = min(step, F - f0)
            raw[f0:f0 + n] = frames.to_host(nd + f0, n)[:, sample]
    finally:
        frames.close()
    assert info.float_path_pixels > 100_000 and info.events > (1 << 27)  # 16-item tiles
    oda, ods = oracle.dark_image(darks, flat)
    assert same_bits(dark_avg, oda) and same_bits(dark_std, ods)
    # a sub-detector of the sampled pixels: the filter and multi-tau are per pixel
    ok = ((dq.ravel()[sample] >= 1) & (sq.ravel()[sample] >= 1)).astype(np.int32)
    qm = oracle.QMap(ok, ok)
    rows, _ = oracle.dense_filter(qm, raw, F, oda[sample], ods[sample], acq.lld, acq.sigma,
                                  flat=flat[sample], finish=False)
    oG2, oIP, oIF = oracle.multitau2(rows, F, acq.dpl, 0)
    for name, got, want in (("G2", G2, oG2), ("IP", IP, oIP), ("IF", IF, oIF)):
        sub = np.ascontiguousarray(got[:, sample])
        assert same_bits(sub, want), (name, int(np.count_nonzero(sub != want)))
