"""fcc_contract_noalloc against fcc_contract, through the C ABI.

fcc_contract_noalloc serves callers that cannot allocate device memory: hosts
that reserve the whole device heap for their own pool, real-time loops that
must not stall on cudaMalloc's device-wide synchronisation, plugins that must
leave their host's device heap alone. It takes the caller's input and output
buffers and keeps every temporary in one static device array inside the
library. Here it runs twice in a row on the same inputs; each result must
match fcc_contract's on the same inputs: the same output coordinate set and
values within 1e-12 * S (S = the oracle's sum of |a*b| per output), the
tolerance of the other parity tests. Further checks: calls on different
contractions in turn (the array keeps the previous call's contents), host
and device operands, free device memory unchanged across calls once each
kernel has run once, and the capacity errors (too many nonzeros, temporaries
larger than the array, an output buffer too small).
"""
import ctypes

import numpy as np
import pytest

import fastcc_gpu as F
import oracle
import workloads
from helpers import check_parity, sort_rows

pytestmark = pytest.mark.gpu

MAX_NNZ = 131072


def _entry():
    fn = F.lib().fcc_contract_noalloc
    vp, i32, i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
    fn.argtypes = [ctypes.POINTER(F._CTensor), ctypes.POINTER(F._CTensor), vp, vp, i32,
                   ctypes.POINTER(F.Options), vp, vp, i64, vp, i64, ctypes.POINTER(i64),
                   ctypes.POINTER(i64)]
    fn.restype = ctypes.c_int
    return fn


def _call(ta, tb, ca, cb, out_c, out_v, cap):
    n, p = ctypes.c_int64(), ctypes.c_int64()
    sa, sb = ta._struct(), tb._struct()
    rc = _entry()(ctypes.byref(sa), ctypes.byref(sb), ca.ctypes.data, cb.ctypes.data, len(ca), None,
                  None, out_c.data_ptr(), out_c.stride(0), out_v.data_ptr(), cap, ctypes.byref(n),
                  ctypes.byref(p))
    return rc, n.value, p.value


def test_noalloc_matches_fcc_contract_twice():
    import torch
    w = workloads.readme(seed=21, scale=0.4)
    a, b = w["a"], w["b"]
    assert a.nnz + b.nnz <= MAX_NNZ
    ca = np.asarray(w["ctr_a"], np.int32)
    cb = np.asarray(w["ctr_b"], np.int32)
    # the existing entry point (host operands) and the oracle's |a*b| sums
    with F.Context(0) as ctx:
        r = ctx.contract(a, b, ca, cb)
        ref_c, ref_v = r.to_numpy()
        order, n_ref, prod_ref = r.order, r.nnz, r.products
        r.free()
    o = oracle.fastcc_multiply(a.coords, a.values, a.max_index, b.coords, b.values, b.max_index,
                               ca, cb, want_abs=True)
    check_parity(ref_c, ref_v, o["coords"], o["values"], o["abs_sum"])
    ref_c, ref_v = sort_rows(ref_c, ref_v)
    oc, oabs = sort_rows(o["coords"], o["abs_sum"])
    assert np.array_equal(ref_c, oc)

    # device operands and caller-owned output buffers
    ta = F.Tensor(torch.from_numpy(a.coords).cuda(), torch.from_numpy(a.values).cuda(), a.max_index)
    tb = F.Tensor(torch.from_numpy(b.coords).cuda(), torch.from_numpy(b.values).cuda(), b.max_index)
    cap = n_ref + 1000
    out_c = torch.empty((order, cap), dtype=torch.int32, device="cuda")
    out_v = torch.empty(cap, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for call in range(2):
        out_v.fill_(float("nan"))
        out_c.fill_(-1)
        torch.cuda.synchronize()
        rc, n, p = _call(ta, tb, ca, cb, out_c, out_v, cap)
        assert rc == 0, (call, rc, F.lib().fcc_last_error(None))
        assert n == n_ref and p == prod_ref
        got_c = out_c[:, :n].t().cpu().numpy()
        got_v = out_v[:n].cpu().numpy()
        check_parity(got_c, got_v, ref_c, ref_v, oabs)


def test_noalloc_reports_capacity():
    import torch
    w = workloads.readme(seed=22, scale=0.1)
    a, b = w["a"], w["b"]
    ca = np.asarray(w["ctr_a"], np.int32)
    cb = np.asarray(w["ctr_b"], np.int32)
    out_c = torch.empty((3, 16), dtype=torch.int32, device="cuda")
    out_v = torch.empty(16, dtype=torch.float64, device="cuda")
    rc, n, _ = _call(a, b, ca, cb, out_c, out_v, 16)
    assert rc == 8 and n > 16  # FCC_ERR_CAPACITY, with the count needed
    big = workloads.readme(seed=23, scale=0.7)  # 210,000 nonzeros in all
    rc, _, _ = _call(big["a"], big["b"], ca, cb, out_c, out_v, 16)
    assert rc == 8


def _pair(w):
    a, b = w["a"], w["b"]
    return (a, b, np.asarray(w["ctr_a"], np.int32), np.asarray(w["ctr_b"], np.int32))


def _device(t):
    import torch
    return F.Tensor(torch.from_numpy(t.coords).cuda(), torch.from_numpy(t.values).cuda(), t.max_index)


def test_noalloc_alternating_contractions_allocate_nothing():
    """readme, a small two-mode self-contraction (hash tiles), readme again,
    twice round: each call against the oracle; after the first round (module
    loading and the one-time set-up), device free memory stays the same."""
    import torch
    cases = [_pair(workloads.readme(seed=31, scale=0.3)),
             _pair(workloads.twomode(seed=32, nnz=40_000, dims=(300, 300, 100, 20))),
             _pair(workloads.readme(seed=33, scale=0.2))]
    want = []
    for a, b, ca, cb in cases:
        assert a.nnz + (0 if b is a else b.nnz) <= MAX_NNZ
        o = oracle.fastcc_multiply(a.coords, a.values, a.max_index, b.coords, b.values, b.max_index, ca, cb,
                                   want_abs=True)
        want.append(o)
    cap = max(len(o["values"]) for o in want) + 64
    order = max(o["order"] for o in want)
    out_c = torch.empty((order, cap), dtype=torch.int32, device="cuda")
    out_v = torch.empty(cap, dtype=torch.float64, device="cuda")
    dev = [(_device(a), b, ca, cb) for a, b, ca, cb in cases]  # A on the device, B from the host
    torch.cuda.synchronize()
    free = []
    for rnd in range(2):
        for (ta, tb, ca, cb), o in zip(dev, want):
            out_v.fill_(float("nan"))
            torch.cuda.synchronize()
            f0 = torch.cuda.mem_get_info()[0]
            rc, n, p = _call(ta, tb, ca, cb, out_c, out_v, cap)
            torch.cuda.synchronize()
            f1 = torch.cuda.mem_get_info()[0]
            assert rc == 0, (rnd, rc, F.lib().fcc_last_error(None))
            assert n == len(o["values"]) and p == o["products"]
            got_c = out_c[:o["order"], :n].t().cpu().numpy()
            check_parity(got_c, out_v[:n].cpu().numpy(), o["coords"], o["values"], o["abs_sum"])
            if rnd == 1:
                free.append(f1 - f0)
    assert free == [0] * len(cases), free


def test_noalloc_reports_scratch_exhausted_below_the_nnz_limit():
    """63,000 nonzeros in all, but 300 output rows of 20,000 columns, each
    split into many work items (products_per_item = 1024): the split rows'
    partial tiles need ~48 MB, more than the static array holds."""
    import torch
    rng = np.random.Generator(np.random.PCG64(41))
    ia, ca_ = np.meshgrid(np.arange(300), np.arange(10), indexing="ij")
    a = F.Tensor(np.stack([ia.ravel(), ca_.ravel()], 1).astype(np.int32), rng.uniform(-1, 1, 3000),
                 np.array([299, 9], np.int32))
    lin = rng.choice(20_000 * 10, size=60_000, replace=False)
    b = F.Tensor(np.stack(np.unravel_index(lin, (20_000, 10)), 1).astype(np.int32), rng.uniform(-1, 1, 60_000),
                 np.array([19_999, 9], np.int32))
    ca, cb = np.array([1], np.int32), np.array([1], np.int32)
    out_c = torch.empty((2, 300 * 20_000), dtype=torch.int32, device="cuda")
    out_v = torch.empty(300 * 20_000, dtype=torch.float64, device="cuda")
    n, p = ctypes.c_int64(), ctypes.c_int64()
    sa, sb = a._struct(), b._struct()
    opts = F.Options(products_per_item=1024)
    rc = _entry()(ctypes.byref(sa), ctypes.byref(sb), ca.ctypes.data, cb.ctypes.data, 1, ctypes.byref(opts), None,
                  out_c.data_ptr(), out_c.stride(0), out_v.data_ptr(), out_v.shape[0], ctypes.byref(n),
                  ctypes.byref(p))
    assert rc == 8, (rc, F.lib().fcc_last_error(None))  # FCC_ERR_CAPACITY
    # the next call still works (the failed one left no work running)
    w = workloads.readme(seed=42, scale=0.1)
    ta, tb, ca2, cb2 = _pair(w)
    rc, n2, _ = _call(ta, tb, ca2, cb2, out_c, out_v, out_v.shape[0])
    assert rc == 0 and n2 > 0
