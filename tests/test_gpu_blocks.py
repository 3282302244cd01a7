"""Incremental transposes (xpcs_series_set_block_frames): frames transposed in
blocks as they are ingested, the blocks' rows joined at xpcs_multitau.  Every
result must be bit-identical to the reference's outputs (golden fixtures) and
to one transpose of all frames, for any block size and any way of splitting
the frames into ingest calls -- including blocks of one frame, blocks longer
than the series, stride/average grouping (a filter frame's raw frames never
straddle two blocks), repeated pixel indices inside a frame, flat-fielded and
dense frames."""
import numpy as np
import pytest

import xpcs_gpu as xg
import xpcs_synth as xs
from fixtures import SPARSE_CASES, load, same_bits, same_bits_nan

pytestmark = pytest.mark.gpu


def _chunks(fx, sizes):
    """The fixture's raw frames in ingest calls of the given frame counts (cycled)."""
    nnz = fx["nnz"]
    off = np.concatenate([[0], np.cumsum(nnz.astype(np.int64))])
    a, k = 0, 0
    while a < nnz.size:
        b = min(nnz.size, a + sizes[k % len(sizes)])
        yield nnz[a:b], fx["idx"][off[a]:off[b]], fx["val"][off[a]:off[b]]
        a, k = b, k + 1


def _run(fx, block, sizes=(1 << 30,), mode=xg.MODE_REFERENCE):
    with xg.Series(fx["W"], fx["H"], fx["F"], fx["dpl"], fx["dqmap"], fx["sqmap"],
                   flatfield=fx["flatfield"], stride=fx["stride"], average=fx["avg"],
                   static_window=fx["swin"], normalize_by_framesum=fx["framesum"]) as s:
        s.set_block_frames(block)
        for part in _chunks(fx, sizes):
            s.ingest_sparse(*part)
        s.multitau(mode)
        G2, IP, IF = s.g2ipif()
        g64, s64, g32, s32 = s.normalize()
        side = s.side_stats(fx["swin"])
        info = s.info()
    return dict(G2=G2, IP=IP, IF=IF, g64=g64, s64=s64, g32=g32, s32=s32, side=side, info=info)


@pytest.mark.parametrize("case", SPARSE_CASES)
@pytest.mark.parametrize("block,sizes", [(1, (1,)), (3, (2, 5)), (7, (1 << 30,)),
                                         (10_000, (4,))])
def test_blocks_bit_exact_vs_reference(case, block, sizes):
    fx = load(case)
    r = _run(fx, block, sizes)
    for k in ("G2", "IP", "IF"):
        assert same_bits(r[k], fx["ref_" + k]), k
    assert same_bits_nan(r["g32"], fx["ref_norm_0_g2"])
    assert same_bits_nan(r["s32"], fx["ref_norm_0_stderr"])
    ps, fs, tot, part = r["side"]
    assert same_bits_nan(ps, fx["ref_pixelSum"])
    assert same_bits_nan(fs, fx["ref_frameSum"])
    assert same_bits_nan(tot, fx["ref_partition_mean_total"])
    assert same_bits_nan(part, fx["ref_partition_mean_partial"])
    one = _run(fx, 0)
    assert same_bits(r["g64"], one["g64"]) and same_bits(r["s64"], one["s64"])
    assert r["info"].events == one["info"].events


def test_blocks_on_a_larger_series_equal_one_transpose():
    acq = xs.Acquisition(width=256, height=256, frames=3000, n_static=12, n_dynamic=6,
                         mean=0.02, tau_min=5.0, tau_max=300.0, seed=77, dpl=8)
    dq, sq, _, _ = xs.maps(acq)
    nnz, idx, val = xs.sparse_frames(acq)
    fx = dict(W=256, H=256, F=3000, dpl=8, dqmap=dq, sqmap=sq, flatfield=None, stride=1, avg=1,
              swin=300, framesum=0, nnz=nnz, idx=idx, val=val)
    one = _run(fx, 0)
    for block, sizes in ((256, (200,)), (1000, (1, 999, 37))):
        for mode in (xg.MODE_REFERENCE, xg.MODE_EXACT):
            r = _run(fx, block, sizes, mode)
            ref = one if mode == xg.MODE_REFERENCE else _run(fx, 0, mode=mode)
            for k in ("G2", "IP", "IF", "g64", "s64"):
                assert same_bits(r[k], ref[k]), (block, mode, k)


def test_dense_blocks_bit_exact_vs_reference():
    fx = load("dense_dark")
    nd = fx["ndark"]
    raw = fx["raw"]
    for block, step in ((1, 1), (4, 3), (100_000, 5)):
        with xg.Series(fx["W"], fx["H"], fx["F"], fx["dpl"], fx["dqmap"], fx["sqmap"],
                       flatfield=fx["flatfield"], stride=fx["stride"], average=fx["avg"],
                       static_window=fx["swin"], dense=True, lld=float(fx["lld_sigma"][0]),
                       sigma=float(fx["lld_sigma"][1])) as s:
            s.set_block_frames(block)
            s.set_dark(raw[:nd])
            data = raw[nd:]
            for a in range(0, data.shape[0], step):
                s.ingest_dense(data[a:a + step])
            s.multitau(xg.MODE_REFERENCE)
            G2, IP, IF = s.g2ipif()
        for k, got in (("G2", G2), ("IP", IP), ("IF", IF)):
            assert same_bits(got, fx["ref_" + k]), (block, k)


def test_block_size_is_set_before_frames_and_refused_in_a_batch():
    fx = load("sparse_basic")
    with xg.Series(fx["W"], fx["H"], fx["F"], fx["dpl"], fx["dqmap"], fx["sqmap"]) as s:
        s.ingest_sparse(fx["nnz"][:2], fx["idx"][:int(fx["nnz"][:2].sum())],
                        fx["val"][:int(fx["nnz"][:2].sum())])
        with pytest.raises(xg.XpcsError) as e:
            s.set_block_frames(4)
        assert e.value.code == 4
        s.reset()
        s.set_block_frames(4)
        with pytest.raises(xg.XpcsError) as e:
            xg.Batch([s])
        assert e.value.code == 1


def test_bad_pixel_index_in_an_early_block_is_reported():
    fx = load("sparse_basic")
    idx = fx["idx"].copy()
    idx[int(fx["nnz"][0])] = fx["W"] * fx["H"] + 1  # first event of frame 1
    with xg.Series(fx["W"], fx["H"], fx["F"], fx["dpl"], fx["dqmap"], fx["sqmap"]) as s:
        s.set_block_frames(2)
        s.ingest_sparse(fx["nnz"], idx, fx["val"])
        s.multitau(xg.MODE_REFERENCE)
        with pytest.raises(xg.XpcsError) as e:
            s.synchronize()
        assert e.value.code == 6
