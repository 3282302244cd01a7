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
