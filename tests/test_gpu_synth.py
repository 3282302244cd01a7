"""The GPU draws of the synthetic sparse and dense frames (benchmark inputs)
give the frames of the host generator for the same parameters."""
import numpy as np
import pytest

import xpcs_synth as xs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("side,frames,mean,tau", [(64, 700, 0.02, (2, 50)),
                                                  (200, 300, 0.005, (5, 500)),
                                                  (33, 1500, 0.3, (10, 10))])
def test_device_frames_equal_host_frames(side, frames, mean, tau):
    acq = xs.Acquisition(width=side, height=side, frames=frames, n_static=12, n_dynamic=6,
                         mean=mean, tau_min=tau[0], tau_max=tau[1], seed=7 + side)
    nnz, idx, val = xs.sparse_frames(acq)
    d = xs.DeviceFrames(acq)
    try:
        dn, di, dv = d.to_host()
    finally:
        d.close()
    assert d.events == idx.size
    assert np.array_equal(dn, nnz) and np.array_equal(di, idx) and np.array_equal(dv, val)


@pytest.mark.parametrize("side,frames,darks", [(48, 120, 10), (96, 40, 0)])
def test_device_dense_frames_match_host_frames(side, frames, darks):
    """Dense CCD frames: the same per-pixel streams as xs_dense_next.  The host
    build may contract dark + noise * n into one FMA, which moves a value that
    sits on a rounding midpoint by one ADU; nothing else may differ."""
    acq = xs.preset("c2", width=side, height=side, frames=frames, dark_frames=darks,
                    n_static=12, n_dynamic=6, seed=11 + side)
    host = xs.DenseStream(acq).next(darks + frames)
    d = xs.DeviceDenseFrames(acq)
    try:
        dev = d.to_host(0, darks + frames)
    finally:
        d.close()
    diff = np.abs(dev.view(np.uint16).astype(np.int32) - host.view(np.uint16).astype(np.int32))
    assert diff.max() <= 1
    assert np.count_nonzero(diff) <= max(2, diff.size // 10000)
    # the photon signal is there: data frames carry counts of 35 ADU on a dark level near 100
    assert host[darks:].view(np.uint16).max() > 150
