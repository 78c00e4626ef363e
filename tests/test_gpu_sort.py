"""The device radix sort (index build of every contraction, tile plan,
expand-sort-reduce) against numpy's stable sort: keys bit-exact and payloads
in the same stable order, over tile-boundary sizes, key widths, heavy
duplicates and both payload widths."""
import numpy as np
import pytest

import fastcc_gpu as F

pytestmark = pytest.mark.gpu

TILE = 4096  # keys per scatter tile


def _keys(rng, n, nbits, dist):
    hi = (1 << nbits) if nbits < 64 else None
    if dist == "uniform":
        if hi is None:
            return rng.integers(0, np.iinfo(np.uint64).max, n, dtype=np.uint64, endpoint=True)
        return rng.integers(0, hi, n, dtype=np.uint64)
    if dist == "few":  # long runs of equal keys: stability decides the payload order
        pool = rng.integers(0, hi if hi else 1 << 63, 7, dtype=np.uint64)
        return pool[rng.integers(0, 7, n)]
    if dist == "sorted":
        return np.sort(rng.integers(0, hi if hi else 1 << 63, n, dtype=np.uint64))
    if dist == "reversed":
        return np.sort(rng.integers(0, hi if hi else 1 << 63, n, dtype=np.uint64))[::-1].copy()
    raise ValueError(dist)


def _check(keys, vals, nbits):
    ko, vo, ms = F.radix_sort(keys, vals, nbits)
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(ko, keys[order])
    np.testing.assert_array_equal(vo, vals[order])
    assert ms >= 0


@pytest.mark.parametrize("n", [1, 2, 31, TILE - 1, TILE, TILE + 1, 3 * TILE + 17, 100_003])
@pytest.mark.parametrize("nbits", [1, 8, 15, 34, 64])
def test_sizes_and_widths(n, nbits):
    rng = np.random.Generator(np.random.PCG64(n * 131 + nbits))
    keys = _keys(rng, n, nbits, "uniform")
    _check(keys, np.arange(n, dtype=np.uint32), nbits)


@pytest.mark.parametrize("dist", ["few", "sorted", "reversed"])
@pytest.mark.parametrize("vdt", [np.uint32, np.uint64])
def test_duplicates_and_presorted(dist, vdt):
    rng = np.random.Generator(np.random.PCG64(9))
    n = 5 * TILE + 123
    keys = _keys(rng, n, 40, dist)
    vals = rng.integers(0, np.iinfo(vdt).max, n, dtype=vdt, endpoint=True)
    _check(keys, vals, 40)


@pytest.mark.parametrize("n", [1, TILE - 1, TILE, 7 * TILE + 5, 300_001])
@pytest.mark.parametrize("nbits", [5, 24, 31, 32])
def test_32bit_keys_64bit_payloads(n, nbits):
    rng = np.random.Generator(np.random.PCG64(n + 17 * nbits))
    keys = rng.integers(0, 1 << nbits, n, dtype=np.uint64).astype(np.uint32)
    keys[::5] = keys[0]
    vals = rng.integers(0, np.iinfo(np.uint64).max, n, dtype=np.uint64, endpoint=True)
    _check(keys, vals, nbits)


def test_large_64bit_payloads():
    rng = np.random.Generator(np.random.PCG64(5))
    n = 2_000_000
    keys = _keys(rng, n, 45, "uniform")
    keys[::3] = keys[0]  # one digit value in every pass for a third of the keys
    vals = rng.integers(0, np.iinfo(np.uint64).max, n, dtype=np.uint64, endpoint=True)
    _check(keys, vals, 45)


def test_zero_bits_and_empty():
    keys = np.array([5, 3, 9], np.uint64)
    ko, vo, _ = F.radix_sort(keys, np.arange(3, dtype=np.uint32), 0)
    np.testing.assert_array_equal(ko, keys)
    np.testing.assert_array_equal(vo, [0, 1, 2])
    ko, vo, _ = F.radix_sort(np.empty(0, np.uint64), np.empty(0, np.uint32), 10)
    assert ko.size == 0 and vo.size == 0
