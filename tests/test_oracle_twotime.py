"""The two-time oracle against the reference's own C2T outputs
(tests/golden/twotime_*.npz): sg, every C2T_all/g2_<q> matrix, g2full and
g2partials bit for bit, for the static-map and symmetric smoothings, with and
without the average filter, and for the frame-threading pixel order."""
import numpy as np
import pytest

from fixtures import TWOTIME_CASES, load_twotime, oracle_twotime, same_bits


@pytest.mark.parametrize("case", TWOTIME_CASES)
def test_twotime_bit_exact(case):
    fx = load_twotime(case)
    r, _ = oracle_twotime(fx)
    assert same_bits(r["sg"], fx["ref_sg"])
    for q, C in r["c2t"].items():
        assert same_bits(C, fx[f"ref_g2_{q:05d}"]), q
    assert same_bits(r["g2full"], fx["ref_g2full"])
    assert same_bits(r["g2partials"], fx["ref_g2partials"])
