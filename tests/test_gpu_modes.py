"""GPU parity of the contraction with batch modes (fcc_contract_modes)
against the reference's own Tensor::multiply (contract.hpp:286-367) recorded
in tests/golden/modes_*.npz, and against a dictionary restatement of it
(oracle.multiply_batch_modes, pinned to those fixtures on the CPU), under the
bar of tests/helpers.py."""
import numpy as np
import pytest

import fastcc_gpu as F
import oracle
from helpers import check_parity, load_golden, mode_golden_names

pytestmark = pytest.mark.gpu


def _tensor(rng, ext, n):
    space = int(np.prod(ext))
    n = min(n, space)
    lin = rng.choice(space, size=n, replace=False)
    c = np.stack(np.unravel_index(lin, ext), axis=1).astype(np.int32).reshape(n, len(ext))
    return c, rng.uniform(-1, 1, n)


CASES = [
    # (A extents, B extents, ctr_a, ctr_b, batch_a, batch_b): C(b,i,j) = sum_k A(b,i,k) B(b,k,j) and friends
    ([6, 7, 5], [6, 5, 8], [2], [1], [0], [0]),
    ([4, 9, 3, 5], [5, 3, 4, 7], [1, 2], [2, 1], [3], [0]),
    ([5, 6], [6, 5], [1], [0], [0], [1]),             # batch only with contraction, no externals on A
    ([3, 4, 5], [5, 4, 3], [], [], [0, 1], [2, 1]),   # no contracted mode: batched outer product
    ([8, 6, 4], [4, 6, 9], [1], [1], [2], [0]),
]


@pytest.mark.parametrize("i", range(len(CASES)))
@pytest.mark.parametrize("opts", [{}, {"accumulator": F.ACC_HASH}, {"products_per_item": 5}])
def test_batch_modes_match_the_reference_semantics(ctx, i, opts):
    ea, eb, ca, cb, ba, bb = CASES[i]
    rng = np.random.Generator(np.random.PCG64(700 + i))
    for x, y in list(zip(ca, cb)) + list(zip(ba, bb)):
        eb[y] = ea[x]
    ac, av = _tensor(rng, ea, 150)
    bc, bv = _tensor(rng, eb, 120)
    A = F.Tensor(ac, av, np.array(ea, np.int32) - 1)
    B = F.Tensor(bc, bv, np.array(eb, np.int32) - 1)
    want_c, want_v, want_s = oracle.multiply_batch_modes(ac, av, bc, bv, ca, cb, ba, bb)
    r = ctx.contract_modes(A, B, ca, cb, ba, bb, F.Options(**opts))
    try:
        c, v = r.to_numpy()
    finally:
        r.free()
    check_parity(c, v, want_c, want_v, want_s)


def test_batch_modes_equal_fastcc_without_batch(ctx):
    rng = np.random.Generator(np.random.PCG64(711))
    ac, av = _tensor(rng, [7, 6, 5], 120)
    bc, bv = _tensor(rng, [5, 9], 40)
    A = F.Tensor(ac, av, np.array([6, 5, 4], np.int32))
    B = F.Tensor(bc, bv, np.array([4, 8], np.int32))
    r1 = ctx.contract_modes(A, B, [2], [0], [], [])
    r2 = ctx.contract(A, B, [2], [0])
    try:
        (c1, v1), (c2, v2) = r1.to_numpy(), r2.to_numpy()
    finally:
        r1.free()
        r2.free()
    o = oracle.fastcc_multiply(ac, av, A.max_index, bc, bv, B.max_index, [2], [0], want_abs=True)
    check_parity(c1, v1, o["coords"], o["values"], o["abs_sum"])
    check_parity(c2, v2, o["coords"], o["values"], o["abs_sum"])


def test_batch_modes_errors(ctx):
    rng = np.random.Generator(np.random.PCG64(712))
    ac, av = _tensor(rng, [3, 4, 5], 20)
    A = F.Tensor(ac, av, np.array([2, 3, 4], np.int32))
    with pytest.raises(F.FccError):
        ctx.contract_modes(A, A, [0], [0], [0], [0])  # a mode both contracted and batch
    with pytest.raises(F.FccError):
        ctx.contract_modes(A, A, [], [], [3], [0])    # batch mode out of range
    big = F.Tensor(np.zeros((1, 7), np.int32), np.ones(1), np.zeros(7, np.int32))
    with pytest.raises(F.FccError):
        ctx.contract_modes(big, big, [], [], [0, 1], [0, 1])  # 7 + 2 modes > 8


@pytest.mark.parametrize("name", mode_golden_names())
@pytest.mark.parametrize("opts", [{}, {"accumulator": F.ACC_HASH}, {"products_per_item": 5}])
def test_batch_modes_match_reference_fixtures(ctx, name, opts):
    g = load_golden(name)
    A = F.Tensor(g["a_coords"], g["a_vals"], g["a_max"])
    B = F.Tensor(g["b_coords"], g["b_vals"], g["b_max"])
    _, _, want_s = oracle.multiply_batch_modes(g["a_coords"], g["a_vals"], g["b_coords"], g["b_vals"], g["ctr_a"],
                                               g["ctr_b"], g["batch_a"], g["batch_b"])
    r = ctx.contract_modes(A, B, g["ctr_a"], g["ctr_b"], g["batch_a"], g["batch_b"], F.Options(**opts))
    try:
        c, v = r.to_numpy()
    finally:
        r.free()
    check_parity(c, v, g["coords"], g["values"], want_s)
