"""GPU parity of the batched contraction (fcc_contract_batch): every instance
of a batch against the oracle's result for that instance alone, under the
same bar as the single-contraction tests (tests/helpers.py). The batch's
mode 0 is the instance; the rest are the instance's own output coordinates.
"""
import numpy as np
import pytest

import fastcc_gpu as F
import oracle
import workloads
from helpers import check_parity

pytestmark = pytest.mark.gpu


def _instances(rng, n, order_a, order_b, ca, cb, max_dim, nnz_max, empty_every=0):
    out = []
    for t in range(n):
        ext_a = [int(x) for x in rng.integers(1, max_dim, size=order_a)]
        ext_b = [int(x) for x in rng.integers(1, max_dim, size=order_b)]
        for x, y in zip(ca, cb):
            ext_b[y] = ext_a[x]

        def gen(ext, cap):
            space = int(np.prod(ext))
            m = min(int(rng.integers(0, cap + 1)), space)
            if empty_every and t % empty_every == empty_every - 1:
                m = 0
            lin = rng.choice(space, size=m, replace=False)
            c = np.stack(np.unravel_index(lin, ext), axis=1).astype(np.int32).reshape(m, len(ext))
            return F.Tensor(c, rng.uniform(-1, 1, m), np.array(ext, np.int32) - 1)

        out.append((gen(ext_a, nnz_max), gen(ext_b, nnz_max)))
    return out


def _check_batch(ctx, pairs, ca, cb, opts=None, device=False):
    As = [p[0] for p in pairs]
    Bs = [p[1] for p in pairs]
    if device:
        import torch
        dev = lambda t: F.Tensor(torch.from_numpy(t.coords).cuda(), torch.from_numpy(t.values).cuda(),
                                 t.max_index)
        As, Bs = [dev(a) for a in As], [dev(b) for b in Bs]
    r, counts = ctx.contract_batch(As, Bs, ca, cb, opts)
    try:
        coords, vals = r.to_numpy()
    finally:
        r.free()
    total_products = 0
    for t, (a, b) in enumerate(pairs):
        o = oracle.fastcc_multiply(a.coords, a.values, a.max_index, b.coords, b.values, b.max_index, ca, cb,
                                   want_abs=True)
        sel = coords[:, 0] == t
        assert counts[t] == int(sel.sum()), f"instance {t}: count {counts[t]} != {int(sel.sum())}"
        check_parity(coords[sel, 1:], vals[sel], o["coords"], o["values"], o["abs_sum"])
        total_products += o["products"]
    assert r.products == total_products
    assert coords.shape[0] == counts.sum()
    return coords, vals, counts


@pytest.mark.parametrize("seed", range(12))
def test_batch_random_parity(ctx, seed):
    rng = np.random.Generator(np.random.PCG64(9100 + seed))
    oa, ob = int(rng.integers(1, 5)), int(rng.integers(1, 5))
    k = int(rng.integers(0, min(oa, ob) + 1))
    ca = [int(x) for x in rng.permutation(oa)[:k]]
    cb = [int(x) for x in rng.permutation(ob)[:k]]
    n = int(rng.integers(1, 24))
    pairs = _instances(rng, n, oa, ob, ca, cb, max_dim=int(rng.integers(2, 12)),
                       nnz_max=int(rng.integers(1, 1500)), empty_every=5 if seed % 3 == 0 else 0)
    opts = [None, F.Options(accumulator=F.ACC_HASH), F.Options(products_per_item=7),
            F.Options(capacity_hint=3)][seed % 4]
    _check_batch(ctx, pairs, ca, cb, opts)


def test_batch_readme_pattern(ctx):
    # the batched benchmark's pattern (a(i,c0,j,c1) x b(k,c0,c1)) at small sizes
    inst = workloads.batched(seed=3, count=24, nnz_lo=50, nnz_hi=3e4, dim_lo=8, dim_hi=64)
    pairs = [(w["a"], w["b"]) for w in inst]
    for opts in (None, F.Options(accumulator=F.ACC_HASH), F.Options(dense_mode=F.DENSE_SENTINEL)):
        _check_batch(ctx, pairs, [1, 3], [1, 2], opts)


def test_batch_device_inputs(ctx):
    rng = np.random.Generator(np.random.PCG64(9201))
    pairs = _instances(rng, 9, 3, 3, [1], [0], max_dim=10, nnz_max=600)
    _check_batch(ctx, pairs, [1], [0], device=True)


def test_batch_single_instance_matches_plain(ctx):
    w = workloads.readme(seed=5, scale=0.03)
    coords, vals, counts = _check_batch(ctx, [(w["a"], w["b"])], w["ctr_a"], w["ctr_b"])
    r = ctx.contract(w["a"], w["b"], w["ctr_a"], w["ctr_b"])
    try:
        c1, v1 = r.to_numpy()
    finally:
        r.free()
    assert counts[0] == c1.shape[0]
    assert np.all(coords[:, 0] == 0)


def test_batch_full_contraction_and_empty(ctx):
    rng = np.random.Generator(np.random.PCG64(9202))
    # every mode contracted: each instance yields at most one (empty-coordinate) entry
    pairs = _instances(rng, 7, 2, 2, [0, 1], [1, 0], max_dim=6, nnz_max=30, empty_every=3)
    coords, vals, counts = _check_batch(ctx, pairs, [0, 1], [1, 0])
    assert coords.shape[1] == 1 and np.all(counts <= 1)
    # all instances empty
    empty = [(F.Tensor(np.zeros((0, 2), np.int32), np.zeros(0), np.array([3, 3], np.int32)),
              F.Tensor(np.zeros((0, 2), np.int32), np.zeros(0), np.array([3, 3], np.int32)))] * 4
    r, counts = ctx.contract_batch([p[0] for p in empty], [p[1] for p in empty], [0], [0])
    assert r.nnz == 0 and not counts.any()
    r.free()


def test_batch_errors(ctx):
    rng = np.random.Generator(np.random.PCG64(9203))
    pairs = _instances(rng, 3, 3, 3, [1], [0], max_dim=6, nnz_max=50)
    As, Bs = [p[0] for p in pairs], [p[1] for p in pairs]
    # an instance of another order
    bad = F.Tensor(np.zeros((1, 2), np.int32), np.ones(1), np.array([1, 1], np.int32))
    with pytest.raises(F.FccError) as e:
        ctx.contract_batch(As[:2] + [bad], Bs, [1], [0])
    assert e.value.status == 1
    # a coordinate beyond its own instance's max_index
    c = np.array([[0, 5, 0]], np.int32)
    over = F.Tensor(c, np.ones(1), np.array([4, 4, 4], np.int32))
    with pytest.raises(F.FccError) as e:
        ctx.contract_batch(As[:2] + [over], Bs, [1], [0])
    assert e.value.status == 1
    # order(A) + 2 above the mode limit
    big = F.Tensor(np.zeros((1, 7), np.int32), np.ones(1), np.zeros(7, np.int32))
    with pytest.raises(F.FccError):
        ctx.contract_batch([big], [Bs[0]], [0], [0])
    # the context still works
    _check_batch(ctx, pairs, [1], [0])
