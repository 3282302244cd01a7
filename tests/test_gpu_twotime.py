"""Two-time on the GPU (xpcs_twotime, REFERENCE mode) against the reference's
own C2T outputs (tests/golden/twotime_*.npz): sg, every C2T_all/g2_<q>,
g2full and g2partials bit for bit; and against the two-time oracle on a
larger synthetic case."""
import numpy as np
import pytest

import oracle
import xpcs_gpu as xg
import xpcs_synth as xs
from fixtures import TWOTIME_CASES, load_twotime, same_bits_nan

pytestmark = pytest.mark.gpu


def gpu_twotime(fx):
    with xg.Series(fx["W"], fx["H"], fx["F"], 4, fx["dqmap"], fx["sqmap"]) as s:
        s.ingest_sparse(fx["nnz"], fx["idx"], fx["val"])
        return s.twotime(fx["qlist"], static_map=fx["static_map"], average=fx["average"],
                         window=fx["wsize"], frame_threading=fx["frame_threading"])


@pytest.mark.parametrize("case", TWOTIME_CASES)
def test_twotime_bit_exact_vs_reference(case):
    fx = load_twotime(case)
    r = gpu_twotime(fx)
    assert same_bits_nan(r["sg"], fx["ref_sg"])
    assert sorted(r["c2t"]) == sorted(int(k[7:]) for k in fx if k.startswith("ref_g2_"))
    for q, C in r["c2t"].items():
        assert same_bits_nan(C, fx[f"ref_g2_{q:05d}"]), q
    assert same_bits_nan(r["g2full"], fx["ref_g2full"])
    assert same_bits_nan(r["g2partials"], fx["ref_g2partials"])


@pytest.mark.parametrize("static_map,average,threading", [(True, True, False), (False, False, True)])
def test_twotime_vs_oracle(static_map, average, threading):
    acq = xs.Acquisition(width=72, height=64, frames=700, n_static=16, n_dynamic=8, mean=0.04,
                         tau_min=3, tau_max=200, seed=91, dpl=4)
    dq, sq, _, _ = xs.maps(acq)
    nnz, idx, val = xs.sparse_frames(acq)
    qlist = [1, 2, 5, 8]
    with xg.Series(acq.width, acq.height, acq.frames, 4, dq, sq) as s:
        s.ingest_sparse(nnz, idx, val)
        r = s.twotime(qlist, static_map=static_map, average=average, window=7,
                      frame_threading=threading)
    qm = oracle.QMap(dq, sq)
    rows, _ = oracle.sparse_filter(qm, nnz, idx, val, acq.frames)
    o = oracle.twotime(qm, rows, acq.frames, qlist, static_map, average, 7, sort_pixels=threading)
    assert same_bits_nan(r["sg"], o["sg"])
    for q, C in o["c2t"].items():
        assert same_bits_nan(r["c2t"][q], C), q
    assert same_bits_nan(r["g2full"], o["g2full"])
    assert same_bits_nan(r["g2partials"], o["g2partials"])


def _max_rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.max(np.abs(b)) if b.size else 0.0
    return float(np.max(np.abs(a - b)) / scale) if scale > 0 else float(np.max(np.abs(a - b)))


@pytest.mark.parametrize("case", TWOTIME_CASES)
def test_exact_twotime_tensor_cores_equal_integer_cuda_cores(case):
    """The tensor-core Gram of the counts is exact: every output equals the one
    from the int64 CUDA-core Gram bit for bit; both agree with the reference's
    float32 outputs to float32 rounding."""
    fx = load_twotime(case)
    out = {}
    for mode in (xg.MODE_EXACT, xg.TWOTIME_EXACT_CUDA_CORES):
        with xg.Series(fx["W"], fx["H"], fx["F"], 4, fx["dqmap"], fx["sqmap"]) as s:
            s.ingest_sparse(fx["nnz"], fx["idx"], fx["val"])
            out[mode] = s.twotime(fx["qlist"], static_map=fx["static_map"], average=fx["average"],
                                  window=fx["wsize"], frame_threading=fx["frame_threading"],
                                  mode=mode)
    t, c = out[xg.MODE_EXACT], out[xg.TWOTIME_EXACT_CUDA_CORES]
    assert same_bits_nan(t["sg"], c["sg"])
    for q in t["c2t"]:
        assert same_bits_nan(t["c2t"][q], c["c2t"][q]), q
    assert same_bits_nan(t["g2full"], c["g2full"]) and same_bits_nan(t["g2partials"], c["g2partials"])
    # the reference accumulates sg and C2T in float32 (relative rounding ~ terms x 2^-24)
    assert _max_rel(t["sg"], fx["ref_sg"]) < 1e-5
    for q, C in t["c2t"].items():
        assert _max_rel(C, fx[f"ref_g2_{q:05d}"]) < 1e-4, q
    assert _max_rel(t["g2full"], fx["ref_g2full"]) < 1e-4


def test_exact_twotime_large_tiles():
    """F not a multiple of the 128-frame tile, a few thousand pixels per group,
    several k tiles per Gram: tensor cores equal the int64 CUDA-core Gram."""
    acq = xs.Acquisition(width=96, height=96, frames=700, n_static=8, n_dynamic=4, mean=0.03,
                         tau_min=3, tau_max=300, seed=93, dpl=4)
    dq, sq, _, _ = xs.maps(acq)
    nnz, idx, val = xs.sparse_frames(acq)
    out = {}
    for mode in (xg.MODE_EXACT, xg.TWOTIME_EXACT_CUDA_CORES):
        with xg.Series(acq.width, acq.height, acq.frames, 4, dq, sq) as s:
            s.ingest_sparse(nnz, idx, val)
            out[mode] = s.twotime([1, 2, 3, 4], static_map=True, average=False, window=9,
                                  mode=mode)
        for q in out[mode]["c2t"]:
            assert np.count_nonzero(out[mode]["c2t"][q]) > 0
    t, c = out[xg.MODE_EXACT], out[xg.TWOTIME_EXACT_CUDA_CORES]
    for q in t["c2t"]:
        assert same_bits_nan(t["c2t"][q], c["c2t"][q]), q
    assert same_bits_nan(t["g2full"], c["g2full"])


@pytest.mark.parametrize("frames", [5, 127, 128, 257])
@pytest.mark.parametrize("static_map", [False, True])
def test_twotime_frame_counts_around_the_tiles(frames, static_map):
    """Frame counts below, at and just past the 128/256-frame Gram tiles
    (padding rows and columns): REFERENCE mode against the oracle bit for bit,
    EXACT mode on the tensor cores equal to the CUDA-core Gram, and within
    float32 rounding of REFERENCE."""
    acq = xs.Acquisition(width=24, height=20, frames=frames, n_static=8, n_dynamic=4, mean=0.1,
                         tau_min=2, tau_max=50, seed=frames + (7 if static_map else 0), dpl=4)
    dq, sq, _, _ = xs.maps(acq)
    nnz, idx, val = xs.sparse_frames(acq)
    qlist = [1, 3, 4]
    window = min(4, frames)
    res = {}
    for mode in (xg.MODE_REFERENCE, xg.MODE_EXACT, xg.TWOTIME_EXACT_CUDA_CORES):
        with xg.Series(acq.width, acq.height, frames, 4, dq, sq) as s:
            s.ingest_sparse(nnz, idx, val)
            res[mode] = s.twotime(qlist, static_map=static_map, average=False, window=window,
                                  mode=mode)
    qm = oracle.QMap(dq, sq)
    rows, _ = oracle.sparse_filter(qm, nnz, idx, val, frames)
    o = oracle.twotime(qm, rows, frames, qlist, static_map, False, window)
    r, t, c = res[xg.MODE_REFERENCE], res[xg.MODE_EXACT], res[xg.TWOTIME_EXACT_CUDA_CORES]
    assert same_bits_nan(r["sg"], o["sg"])
    for q, C in o["c2t"].items():
        assert same_bits_nan(r["c2t"][q], C), q
        assert same_bits_nan(t["c2t"][q], c["c2t"][q]), q
        assert _max_rel(t["c2t"][q], C) <= 1e-4, q
    assert same_bits_nan(r["g2full"], o["g2full"])
    assert same_bits_nan(r["g2partials"], o["g2partials"])
    assert same_bits_nan(t["g2full"], c["g2full"])
