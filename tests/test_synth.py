"""CPU tests of the seeded generator (include/fastcc_synth.h)."""
import numpy as np

import fastcc_gpu as F


def test_deterministic_and_distinct():
    c1, v1 = F.synth_coo(5, [40, 30, 20], [1.2, 0, 1.1], 5000, lognormal=True)
    c2, v2 = F.synth_coo(5, [40, 30, 20], [1.2, 0, 1.1], 5000, lognormal=True)
    assert np.array_equal(c1, c2) and np.array_equal(v1, v2)
    assert c1.shape == (5000, 3)
    lin = (c1[:, 0].astype(np.int64) * 30 + c1[:, 1]) * 20 + c1[:, 2]
    assert np.unique(lin).size == 5000
    assert (c1 >= 0).all() and (c1 < np.array([40, 30, 20])).all()
    c3, _ = F.synth_coo(6, [40, 30, 20], [1.2, 0, 1.1], 5000, lognormal=True)
    assert not np.array_equal(c1, c3)


def test_zipf_skew_and_value_ranges():
    c, v = F.synth_coo(9, [1000, 1000], [1.2, 0.0], 20000)
    assert (v >= -1).all() and (v < 1).all()
    h0 = np.bincount(c[:, 0], minlength=1000)
    h1 = np.bincount(c[:, 1], minlength=1000)
    assert h0[0] > 5 * h0[500:].mean()      # Zipf head
    assert h1.max() < 3 * h1.mean()         # uniform mode
    _, lv = F.synth_coo(9, [1000, 1000], [0, 0], 20000, lognormal=True)
    assert (lv < 0).any() and (lv > 0).any()
    ll = np.log(np.abs(lv))
    assert abs(np.median(ll)) < 0.05 and 0.95 < ll.std() < 1.05  # lognormal(0, 1)


def test_support_exhaustion_returns_fewer():
    c, v = F.synth_coo(1, [3, 3], [0, 0], 20)
    assert c.shape[0] == 9 and v.shape[0] == 9
