"""CPU tests of the oracle (the restatement in oracle/fastcc_oracle.cpp).

The oracle is pinned to the reference's own fastcc_multiply through the golden
fixtures in tests/golden (made by tests/golden/make_golden.py from the
reference compiled from its sources) and, where the reference sources are
present, by running the compiled reference live.
"""
import numpy as np
import pytest

import oracle
from helpers import golden_names, load_golden, mode_golden_names, sort_rows


@pytest.mark.parametrize("name", golden_names())
def test_oracle_reproduces_reference_golden(name):
    g = load_golden(name)
    o = oracle.fastcc_multiply(g["a_coords"], g["a_vals"], g["a_max"], g["b_coords"], g["b_vals"],
                               g["b_max"], g["ctr_a"], g["ctr_b"], tile_size=int(g["tile"]))
    idx = np.lexsort((o["right"], o["left"]))
    assert o["order"] == int(g["out_order"])
    assert np.array_equal(o["left"][idx], g["left"])
    assert np.array_equal(o["right"][idx], g["right"])
    # same summation order as the reference: values are bit-identical
    assert np.array_equal(o["values"][idx], g["values"])
    # The shipped TileAccumulator path loses entries after an empty per-thread
    # list (ListTensor::concatenate, index_tensors.hpp:115-125); when it
    # returned everything, its values are the same multiset.
    assert int(g["shipped_count"]) <= len(g["values"])
    if int(g["shipped_count"]) == len(g["values"]):
        assert np.array_equal(np.sort(o["values"]), g["shipped_sorted_values"])


def _rand_case(rng, order_a, order_b, k, max_dim=9, nnz_a=200, nnz_b=150):
    ext_a = list(rng.integers(2, max_dim, size=order_a))
    ext_b = list(rng.integers(2, max_dim, size=order_b))
    ca = list(rng.permutation(order_a)[:k])
    cb = list(rng.permutation(order_b)[:k])
    for x, y in zip(ca, cb):
        ext_b[y] = ext_a[x]
    def gen(ext, n):
        space = int(np.prod(ext))
        n = min(n, space)
        lin = rng.choice(space, size=n, replace=False)
        c = np.stack(np.unravel_index(lin, ext), axis=1).astype(np.int32)
        return c, rng.uniform(-1, 1, n)
    ac, av = gen(ext_a, nnz_a)
    bc, bv = gen(ext_b, nnz_b)
    return ac, av, np.array(ext_a, np.int32) - 1, bc, bv, np.array(ext_b, np.int32) - 1, ca, cb


@pytest.mark.parametrize("seed", range(12))
def test_oracle_matches_bruteforce(seed):
    rng = np.random.Generator(np.random.PCG64(100 + seed))
    oa, ob = int(rng.integers(1, 5)), int(rng.integers(1, 5))
    k = int(rng.integers(0, min(oa, ob) + 1))
    case = _rand_case(rng, oa, ob, k)
    tile = int(rng.choice([0, 1, 3, 16, 100, 1000]))
    o = oracle.fastcc_multiply(*case, tile_size=tile, want_abs=True)
    b = oracle.bruteforce(*case)
    oc, ov, oabs = sort_rows(o["coords"], o["values"], o["abs_sum"])
    assert o["products"] == b["products"]
    assert np.array_equal(oc, b["coords"])
    assert np.all(np.abs(ov - b["values"]) <= 1e-12 * b["abs_sum"] + 1e-300)
    assert np.allclose(oabs, b["abs_sum"], rtol=1e-12, atol=0)
    assert oracle.count_products(*case) == b["products"]


@pytest.mark.skipif(not oracle.ref_available(), reason="reference sources not compiled here")
@pytest.mark.parametrize("seed", range(6))
def test_oracle_bit_identical_to_live_reference(seed):
    rng = np.random.Generator(np.random.PCG64(900 + seed))
    oa, ob = int(rng.integers(2, 5)), int(rng.integers(2, 5))
    k = int(rng.integers(1, min(oa, ob) + 1))
    case = _rand_case(rng, oa, ob, k, max_dim=12, nnz_a=800, nnz_b=500)
    tile = int(rng.choice([1, 8, 100, 128]))
    o = oracle.fastcc_multiply(*case, tile_size=tile)
    r = oracle.reference_multiply(*case, tile_size=tile)
    io = np.lexsort((o["right"], o["left"]))
    ir = np.lexsort((r["right"], r["left"]))
    assert np.array_equal(o["left"][io], r["left"][ir])
    assert np.array_equal(o["right"][io], r["right"][ir])
    assert np.array_equal(o["values"][io], r["values"][ir])


def test_infer_shape_is_per_mode_max():
    c = np.array([[3, 0, 5], [1, 7, 2]], np.int32)
    assert list(oracle.infer_shape(c)) == [3, 7, 5]


def test_oracle_rejects_bad_arguments():
    c = np.zeros((1, 2), np.int32)
    v = np.ones(1)
    m = np.zeros(2, np.int32)
    with pytest.raises(ValueError):
        oracle.fastcc_multiply(c, v, m, c, v, m, [0, 0], [0, 1])  # repeated mode
    with pytest.raises(ValueError):
        oracle.fastcc_multiply(c, v, m, c, v, m, [2], [0])  # out of range


def test_batch_mode_restatement_reduces_to_fastcc_and_to_batched_slices():
    """oracle.multiply_batch_modes (Tensor::multiply, contract.hpp:284-367):
    without batch modes it equals fastcc_multiply; with one it equals the
    per-batch-index fastcc_multiply of the slices, batch index prepended."""
    import oracle
    rng = np.random.Generator(np.random.PCG64(55))
    ea, eb = [5, 4, 6], [6, 4, 3]  # A(b, i, k), B(k, b, j)
    la = rng.choice(np.prod(ea), 60, replace=False)
    lb = rng.choice(np.prod(eb), 40, replace=False)
    ac = np.stack(np.unravel_index(la, ea), 1).astype(np.int32)
    bc = np.stack(np.unravel_index(lb, eb), 1).astype(np.int32)
    av, bv = rng.uniform(-1, 1, 60), rng.uniform(-1, 1, 40)
    c0, v0, _ = oracle.multiply_batch_modes(ac, av, bc, bv, [2], [0], [], [])
    o = oracle.fastcc_multiply(ac, av, np.array(ea) - 1, bc, bv, np.array(eb) - 1, [2], [0])
    idx = np.lexsort(o["coords"].T[::-1])
    assert np.array_equal(c0, o["coords"][idx].astype(np.int64))
    assert np.allclose(v0, o["values"][idx], rtol=1e-12, atol=1e-15)
    c1, v1, _ = oracle.multiply_batch_modes(ac, av, bc, bv, [2], [0], [0], [1])
    rows = []
    for bidx in range(ea[0]):
        sa, sb = ac[ac[:, 0] == bidx], bc[bc[:, 1] == bidx]
        if len(sa) == 0 or len(sb) == 0:
            continue
        va, vb = av[ac[:, 0] == bidx], bv[bc[:, 1] == bidx]
        c, v, _ = oracle.multiply_batch_modes(sa[:, 1:], va, sb[:, [0, 2]], vb, [1], [0], [], [])
        for k in range(len(v)):
            rows.append(((bidx,) + tuple(c[k]), v[k]))
    rows.sort()
    assert np.array_equal(c1, np.array([r[0] for r in rows], np.int64).reshape(len(rows), 3))
    assert np.allclose(v1, [r[1] for r in rows], rtol=1e-12)


def _mode_args(g):
    return (g["a_coords"], g["a_vals"], g["b_coords"], g["b_vals"], g["ctr_a"], g["ctr_b"], g["batch_a"],
            g["batch_b"])


@pytest.mark.parametrize("name", mode_golden_names())
def test_batch_mode_restatement_matches_reference_fixture(name):
    """oracle.multiply_batch_modes against the reference's own Tensor::multiply
    (contract.hpp:286-367) recorded in tests/golden/modes_*.npz: the same
    output coordinates, values within 1e-12 * S (the two sum in different
    orders: the reference in its hash maps' iteration order)."""
    g = load_golden(name)
    c, v, s = oracle.multiply_batch_modes(*_mode_args(g))
    assert np.array_equal(c, g["coords"].astype(np.int64))
    assert np.all(np.abs(v - g["values"]) <= 1e-12 * np.maximum(np.abs(g["values"]), s))


@pytest.mark.skipif(not oracle.ref_available(), reason="reference sources not compiled here")
@pytest.mark.parametrize("name", mode_golden_names())
def test_batch_mode_fixture_reproduces_from_the_reference(name):
    g = load_golden(name)
    c, v = oracle.reference_multiply_modes(g["a_coords"], g["a_vals"], g["a_max"], g["b_coords"], g["b_vals"],
                                           g["b_max"], g["ctr_a"], g["ctr_b"], g["batch_a"], g["batch_b"])
    c, v = sort_rows(c, v)
    assert np.array_equal(c, g["coords"]) and np.array_equal(v, g["values"])
