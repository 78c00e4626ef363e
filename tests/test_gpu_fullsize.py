"""GPU parity at the benchmark sizes, against the oracle in full.

The workloads are the ones bench.py times, with the same seeds:
  * zipf3: A 20,000 x 20,000 x 500,000, 10M nonzeros, A x A over {1,2}
    (4.36e9 multiply-adds, 3.9e8 outputs);
  * twomode: A 5,000 x 5,000 x 2,000 x 50, 5M nonzeros, A x A over {0,2}
    (4.2e8 multiply-adds, 2.0e8 outputs);
  * batched: the 256-instance batch of the readme pattern, one
    fcc_contract_batch call, every instance against the oracle alone.

Each output is identified by its linearised (A external, B external) pair,
the oracle's (left, right) (contract.hpp:876-909 with the drain decode fixed).
Both sides are sorted by that key on the device and compared whole: equal
output counts, equal key arrays (the coordinate sets bit for bit) and every
value within 1e-12 * S, S the oracle's sum of |a*b| for that output
(tests/helpers.py states the bar).
"""
import numpy as np
import pytest

import fastcc_gpu as F
import oracle
import workloads

pytestmark = pytest.mark.gpu

RTOL = 1e-12


class _Dev:
    """Wraps a device pointer for torch.as_tensor (CUDA array interface)."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False),
                                         "version": 3, "strides": None}


def _radices(t, ctr):
    return [int(t.max_index[m]) + 1 for m in range(t.order) if m not in ctr]


def _device_columns(r):
    import torch
    cptr, stride, vptr = r.device_pointers()
    n = r.nnz
    vals = torch.as_tensor(_Dev(vptr, n, "<f8"), device="cuda")
    cols = [torch.as_tensor(_Dev(cptr + 4 * m * stride, n, "<i4"), device="cuda") for m in range(r.order)]
    return cols, vals


def _horner(cols, radices):
    import torch
    out = torch.zeros(cols[0].numel() if cols else 0, dtype=torch.int64, device="cuda")
    for c, rad in zip(cols, radices):
        out = out * rad + c.long()
    return out


def _compare(key_g, val_g, o, LB):
    """Sorted-key comparison of a device result (key_g, val_g) with an oracle
    result o (left, right, values, abs_sum). Returns (outputs, cancellation
    cases)."""
    import torch
    left = torch.from_numpy(o["left"].view(np.int64)).cuda()
    right = torch.from_numpy(o["right"].view(np.int64)).cuda()
    key_o = left * LB + right
    del left, right
    assert key_g.numel() == key_o.numel(), f"output count {key_g.numel()} != oracle {key_o.numel()}"
    kg, ig = torch.sort(key_g)
    ko, io = torch.sort(key_o)
    del key_o
    assert torch.equal(kg, ko), "output coordinate sets differ"
    if kg.numel() > 1:
        assert bool((kg[1:] != kg[:-1]).all()), "duplicate output coordinates"
    del kg, ko
    vg = val_g[ig]
    vo = torch.from_numpy(o["values"]).cuda()[io]
    so = torch.from_numpy(o["abs_sum"]).cuda()[io]
    err = (vg - vo).abs()
    bad = err > RTOL * torch.maximum(vo.abs(), so)
    nbad = int(bad.sum())
    assert nbad == 0, f"{nbad} values exceed 1e-12*S; worst {float(err[bad].max()):.3e}"
    canc = int((err > RTOL * vo.abs()).sum())
    return int(vg.numel()), canc


def _oracle(w):
    a, b = w["a"], w["b"]
    return oracle.fastcc_multiply(a.coords, a.values, a.max_index, b.coords, b.values, b.max_index,
                                  w["ctr_a"], w["ctr_b"], tile_size=128, want_abs=True)


def _device_tensor(t):
    import torch
    return F.Tensor(torch.from_numpy(t.coords).cuda(), torch.from_numpy(t.values).cuda(), t.max_index)


_ORACLE = {}


def _check_single(ctx, w, opts=None):
    import torch
    a, b = w["a"], w["b"]
    A = _device_tensor(a)
    B = A if b is a else _device_tensor(b)
    r = ctx.contract(A, B, w["ctr_a"], w["ctr_b"], opts)
    try:
        ra, rb = _radices(a, w["ctr_a"]), _radices(b, w["ctr_b"])
        cols, vals = _device_columns(r)
        LB = int(np.prod(rb))
        key = _horner(cols[:len(ra)], ra) * LB + _horner(cols[len(ra):], rb)
        vals = vals.clone()
        products = r.products
    finally:
        r.free()
    del A, B
    torch.cuda.synchronize()
    if w["name"] not in _ORACLE:  # one oracle run per workload, shared by the kernel variants
        _ORACLE.clear()
        _ORACLE[w["name"]] = _oracle(w)
    o = _ORACLE[w["name"]]
    assert products == o["products"]
    n, canc = _compare(key, vals, o, LB)
    return n, products, canc


@pytest.mark.parametrize("dense_kernel", [0, 2])
def test_zipf3_full_size_matches_oracle(ctx, dense_kernel):
    n, p, canc = _check_single(ctx, workloads.zipf3(seed=1), F.Options(dense_kernel=dense_kernel))
    assert p == 4_362_229_740 and n == 393_466_340
    print(f"zipf3: {n} outputs, {p} multiply-adds, {canc} cancellation cases")


def test_twomode_full_size_matches_oracle(ctx):
    n, p, canc = _check_single(ctx, workloads.twomode(seed=1))
    assert p == 415_279_252 and n == 199_932_409
    print(f"twomode: {n} outputs, {p} multiply-adds, {canc} cancellation cases")


def test_batched_benchmark_batch_matches_oracle(ctx):
    """The 256-instance batch that bench.py times, in one fcc_contract_batch
    call, every instance against the oracle run on that instance alone."""
    import torch
    inst = workloads.batched(seed=1, count=256)
    As = [_device_tensor(x["a"]) for x in inst]
    Bs = [_device_tensor(x["b"]) for x in inst]
    ctr_a, ctr_b = inst[0]["ctr_a"], inst[0]["ctr_b"]
    r, counts = ctx.contract_batch(As, Bs, ctr_a, ctr_b)
    total_out = total_prod = 0
    try:
        cols, vals = _device_columns(r)
        inst_col = cols[0]
        assert int(counts.sum()) == r.nnz
        for t, x in enumerate(inst):
            ra, rb = _radices(x["a"], ctr_a), _radices(x["b"], ctr_b)
            LB = int(np.prod(rb))
            sel = (inst_col == t).nonzero().flatten()
            assert sel.numel() == int(counts[t]), f"instance {t}: count {int(counts[t])} != {sel.numel()}"
            sub = [c[sel] for c in cols[1:]]
            key = _horner(sub[:len(ra)], ra) * LB + _horner(sub[len(ra):], rb)
            o = _oracle(x)
            n, _ = _compare(key, vals[sel], o, LB)
            total_out += n
            total_prod += o["products"]
            del sub, key, sel, o
        assert r.products == total_prod
        assert total_out == r.nnz
    finally:
        r.free()
    del As, Bs
    torch.cuda.synchronize()
    print(f"batched: 256 instances, {total_out} outputs, {total_prod} multiply-adds")
