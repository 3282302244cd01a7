"""Dense series without stride or frame averaging are filtered straight into
pixel-major blocks (k_dense.cu: per-pixel counts per slice, a prefix over the
slices and a scan over the pixels, a write pass that stages each pixel's
events in shared memory and stores whole 32-byte sectors, then one warp per
pixel gathering its blocks).  Ingests of every size must give the oracle's
DenseFilter::Apply + Corr::multiTau2 (dense_filter.cpp:121-210,
corr.cpp:315-431) bit for bit: single frames that wait in the pending buffer,
runs that go straight to blocks, a mix of both, host and device frames, and
detectors whose pixel count is or is not a multiple of the 8-pixel lane group.
Small detectors split a block's frames into many slices, so rows are cut
inside sectors at every slice boundary."""
import numpy as np
import pytest

import oracle
import xpcs_gpu as xg
import xpcs_synth as xs
from fixtures import same_bits

pytestmark = pytest.mark.gpu

LLD, SIGMA = 0.0, 3.0

# call sizes: short runs wait for a block's worth (256 frames here), long runs
# go straight to blocks, None = the rest
SPLITS = {
    "one call": [None],
    "mixed": [1, 3, 250, 7, 300, 1, None],
    "single frames": "ones",
}


def _acq(w, h, frames, seed):
    return xs.Acquisition(width=w, height=h, frames=frames, n_static=12, n_dynamic=6, mean=0.05,
                          tau_min=3, tau_max=300, seed=seed, dpl=8, dense=True, dark_frames=20,
                          gain_min=0.85, gain_max=1.1)


def _calls(split, n):
    if split == "ones":
        return [(a, a + 1) for a in range(n)]
    out, a = [], 0
    for k in split:
        b = n if k is None else min(n, a + k)
        out.append((a, b))
        a = b
    return out


def _oracle(acq, raw, flat, dq, sq):
    nd = acq.dark_frames
    qm = oracle.QMap(dq, sq)
    da, dsd = oracle.dark_image(raw[:nd], flat.ravel())
    rows, _ = oracle.dense_filter(qm, raw[nd:], acq.frames, da, dsd, LLD, SIGMA,
                                  flat=flat.ravel())
    return rows, oracle.multitau2(rows, acq.frames, acq.dpl, xg.MODE_REFERENCE)


def _series(acq, dq, sq, flat):
    return xg.Series(acq.width, acq.height, acq.frames, acq.dpl, dq, sq, flatfield=flat,
                     dense=True, lld=LLD, sigma=SIGMA)


@pytest.mark.parametrize("w,h", [(48, 40), (37, 29)])
@pytest.mark.parametrize("split", list(SPLITS))
def test_dense_pixel_major_ingest_vs_oracle(w, h, split):
    acq = _acq(w, h, 1300, seed=7 + w + len(split))
    dq, sq, flat, _ = xs.maps(acq)
    ds = xs.DenseStream(acq)
    raw = ds.next(acq.dark_frames + acq.frames)
    ds.close()
    nd = acq.dark_frames
    rows, (oG2, oIP, oIF) = _oracle(acq, raw, flat, dq, sq)
    with _series(acq, dq, sq, flat) as s:
        s.set_dark(raw[:nd])
        for a, b in _calls(SPLITS[split], acq.frames):
            s.ingest_dense(raw[nd + a:nd + b])
        s.multitau(xg.MODE_REFERENCE)
        G2, IP, IF = s.g2ipif()
        info = s.info()
        assert info.raw_frames == acq.frames
        assert info.raw_events == rows.row_ptr[-1] and info.events == rows.row_ptr[-1]
        for name, got, want in (("G2", G2, oG2), ("IP", IP, oIP), ("IF", IF, oIF)):
            assert same_bits(got, want), (name, int(np.count_nonzero(got != want)))
        # a reset empties the pending buffer and the blocks: the same frames again
        s.reset()
        for a, b in _calls([5, None], acq.frames):
            s.ingest_dense(raw[nd + a:nd + b])
        s.multitau(xg.MODE_REFERENCE)
        G2b, _, _ = s.g2ipif()
        assert same_bits(G2b, oG2)


def test_dense_pixel_major_device_frames_vs_oracle():
    acq = _acq(64, 48, 1500, seed=91)
    dq, sq, flat, _ = xs.maps(acq)
    nd = acq.dark_frames
    frames = xs.DeviceDenseFrames(acq)
    try:
        raw = frames.to_host(0, nd + acq.frames)
        rows, (oG2, oIP, oIF) = _oracle(acq, raw, flat, dq, sq)
        with _series(acq, dq, sq, flat) as s:
            s.set_dark(raw[:nd])
            for a, b in _calls([2, 600, 9, 250, None], acq.frames):
                s.ingest_dense_device(frames.frame_ptr(nd + a), b - a)
            s.multitau(xg.MODE_REFERENCE)
            G2, IP, IF = s.g2ipif()
            info = s.info()
    finally:
        frames.close()
    assert info.raw_events == rows.row_ptr[-1]
    for name, got, want in (("G2", G2, oG2), ("IP", IP, oIP), ("IF", IF, oIF)):
        assert same_bits(got, want), (name, int(np.count_nonzero(got != want)))


def test_dense_pixel_major_framesum_and_side_statistics_vs_oracle():
    """normalize_by_framesum on a pixel-major dense series (the finishing
    gather forces the float rows; the float kernel scales by the frame sums)
    and the side statistics' pixel and frame sums, formed from the rows."""
    acq = _acq(40, 32, 900, seed=5)
    dq, sq, flat, _ = xs.maps(acq)
    ds = xs.DenseStream(acq)
    raw = ds.next(acq.dark_frames + acq.frames)
    ds.close()
    nd, F = acq.dark_frames, acq.frames
    qm = oracle.QMap(dq, sq)
    da, dsd = oracle.dark_image(raw[:nd], flat.ravel())
    rows, side = oracle.dense_filter(qm, raw[nd:], F, da, dsd, LLD, SIGMA, flat=flat.ravel())
    scaled = oracle.framesum_normalize(rows, side["frames_sum"], F)
    oG2, oIP, oIF = oracle.multitau2(scaled, F, acq.dpl, xg.MODE_REFERENCE)
    with xg.Series(acq.width, acq.height, F, acq.dpl, dq, sq, flatfield=flat, dense=True,
                   lld=LLD, sigma=SIGMA, normalize_by_framesum=True) as s:
        s.set_dark(raw[:nd])
        for a, b in _calls([3, 400, None], F):
            s.ingest_dense(raw[nd + a:nd + b])
        s.multitau(xg.MODE_REFERENCE)
        G2, IP, IF = s.g2ipif()
        ps, fs, _, _ = s.side_stats(max(F // 10, 1))
    for name, got, want in (("G2", G2, oG2), ("IP", IP, oIP), ("IF", IF, oIF)):
        assert same_bits(got, want), (name, int(np.count_nonzero(got != want)))
    # the oracle's side outputs are already the reference's pixelSum / frameSum
    assert same_bits(ps, side["pixels_sum"].astype(np.float32).reshape(ps.shape))
    assert same_bits(fs, side["frames_sum"].astype(np.float32).reshape(fs.shape))
