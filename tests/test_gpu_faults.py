"""Failures injected on the host, checked on the GPU without faulting it: an
allocation refused by the library's device-memory limit must come back as
XPCS_ERR_OUT_OF_MEMORY, leave the handle usable, and leak nothing; a sparse
frame with a pixel index outside the detector must come back as
XPCS_ERR_INPUT (the reference would write out of bounds,
sparse_filter.cpp:168-187)."""
import numpy as np
import pytest

import xpcs_gpu as xg
from fixtures import load, same_bits

pytestmark = pytest.mark.gpu


def _series(fx):
    return xg.Series(fx["W"], fx["H"], fx["F"], fx["dpl"], fx["dqmap"], fx["sqmap"],
                     static_window=fx["swin"], device=0)


def test_device_memory_limit_refuses_cleanly_and_the_handle_recovers():
    fx = load("sparse_basic")
    used0, _ = xg.device_memory(0)
    try:
        with _series(fx) as s:
            s.ingest_sparse(fx["nnz"], fx["idx"], fx["val"])
            s.synchronize()
            used1, _ = xg.device_memory(0)
            assert used1 > used0
            # room for a few bytes more than the series holds: the transpose needs more
            xg.set_device_memory_limit(0, used1 + 64)
            with pytest.raises(xg.XpcsError) as e:
                s.multitau(xg.MODE_REFERENCE)
            assert e.value.code == 3 and "limit" in str(e.value)
            assert xg.device_memory(0)[0] <= used1 + 64
            xg.set_device_memory_limit(0, 0)
            s.multitau(xg.MODE_REFERENCE)
            G2, IP, IF = s.g2ipif()
        for name, got in (("G2", G2), ("IP", IP), ("IF", IF)):
            assert same_bits(got, fx["ref_" + name]), name
    finally:
        xg.set_device_memory_limit(0, 0)
    assert xg.device_memory(0)[0] == used0  # everything the series held was returned


def test_series_creation_over_the_limit_is_refused():
    fx = load("sparse_basic")
    used0, _ = xg.device_memory(0)
    try:
        xg.set_device_memory_limit(0, used0 + 16)
        with pytest.raises(xg.XpcsError) as e:
            _series(fx)
        assert e.value.code == 3
    finally:
        xg.set_device_memory_limit(0, 0)
    assert xg.device_memory(0)[0] == used0


def test_pixel_index_outside_the_detector_is_an_input_error():
    fx = load("sparse_basic")
    idx = fx["idx"].copy()
    idx[len(idx) // 2] = fx["W"] * fx["H"] + 7
    with _series(fx) as s:
        s.ingest_sparse(fx["nnz"], idx, fx["val"])
        s.multitau(xg.MODE_REFERENCE)
        with pytest.raises(xg.XpcsError) as e:
            s.synchronize()
        assert e.value.code == 6
        # the same handle, reset and given good frames, gives the reference's result
        s.reset()
        s.ingest_sparse(fx["nnz"], fx["idx"], fx["val"])
        s.multitau(xg.MODE_REFERENCE)
        G2 = s.g2ipif()[0]
    assert same_bits(G2, fx["ref_G2"])
    assert np.all(np.isfinite(G2))


def test_device_properties_and_bad_ordinal():
    assert xg.device_sm_count(0) >= 1
    with pytest.raises(xg.XpcsError) as e:
        xg.device_sm_count(1 << 20)
    assert e.value.code == 1
