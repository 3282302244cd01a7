"""The GPU draw of the synthetic sparse frames (benchmark inputs) gives the
frames of the host generator for the same parameters."""
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
