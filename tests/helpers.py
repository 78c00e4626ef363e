"""Comparison helpers for the parity tests.

Parity bar: the output coordinate set is bit-exact with the oracle, and every
value satisfies |x - y| <= 1e-12 * S, where y is the oracle's value and S the
oracle's sum of |a*b| over that output's products. S bounds the rounding error
of any summation order, so the test accepts a reordered sum even where
cancellation makes the plain relative error 1e-12*|y| unattainable. Values
that miss the plain relative bound are counted and reported as cancellation
cases, never hidden.
"""
import os

import numpy as np

RTOL = 1e-12
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sort_rows(coords, *cols):
    coords = np.asarray(coords)
    if coords.shape[0] == 0 or coords.ndim < 2 or coords.shape[1] == 0:
        return (coords,) + cols
    idx = np.lexsort(coords.T[::-1])
    return (coords[idx],) + tuple(np.asarray(c)[idx] for c in cols)


def check_parity(got_coords, got_vals, want_coords, want_vals, want_abs, rtol=RTOL):
    """Asserts the parity bar; returns (n, max plain relative error, cancellation cases)."""
    gc, gv = sort_rows(np.asarray(got_coords, np.int64), got_vals)
    wc, wv, wa = sort_rows(np.asarray(want_coords, np.int64), want_vals, want_abs)
    assert gc.shape == wc.shape, f"output count {gc.shape} != oracle {wc.shape}"
    assert np.array_equal(gc, wc), "output coordinate sets differ"
    if gc.shape[0] > 1 and gc.shape[1] > 0:
        assert not np.any(np.all(gc[1:] == gc[:-1], axis=1)), "duplicate output coordinates"
    err = np.abs(np.asarray(gv) - np.asarray(wv))
    bound = rtol * np.maximum(np.abs(wv), wa)
    bad = err > bound
    assert not bad.any(), (f"{int(bad.sum())} values exceed 1e-12*S; worst err {err[bad].max():.3e} "
                           f"at S {wa[bad][np.argmax(err[bad])]:.3e}")
    rel = err / np.maximum(np.abs(wv), 1e-300)
    canc = int(np.sum(err > rtol * np.abs(wv)))
    return gc.shape[0], float(rel.max()) if rel.size else 0.0, canc


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def golden_names():
    """Fixtures of the reference's fastcc_multiply."""
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz") and not f.startswith("modes_"))


def mode_golden_names():
    """Fixtures of the reference's Tensor::multiply with batch modes."""
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz") and f.startswith("modes_"))
