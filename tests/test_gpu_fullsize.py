"""GPU checks at the benchmark sizes, through size-independent properties.

The oracle cannot contract these workloads in seconds, so each full-size
result is checked by properties that O(nnz) host arithmetic can verify:
  * linearity: sum over outputs of v*w[row]*u[col] equals
    sum_c (sum_{a in c} va*w[row_a]) * (sum_{b in c} vb*u[col_b]) for random
    weights w, u (a Freivalds-style checksum of the whole product);
  * row sums: sum_col C[row, col] = sum_{a in row} va * sB(key_a);
  * exact rows: a handful of rows, the heaviest included, recomputed exactly
    on the host and compared coordinate by coordinate (1e-12 * S);
  * structure: coordinates inside the extents and no duplicate outputs.
"""
import numpy as np
import pytest

import fastcc_gpu as F
import workloads
from helpers import check_parity

pytestmark = pytest.mark.gpu


class _Dev:
    """Wraps a device pointer for torch.as_tensor (CUDA array interface)."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False),
                                         "version": 3, "strides": None}


def _lin(coords, modes, radix):
    out = np.zeros(coords.shape[0], np.int64)
    for m in modes:
        out = out * np.int64(radix[m]) + coords[:, m].astype(np.int64)
    return out


def _host_model(w):
    a, b = w["a"], w["b"]
    ra, rb = a.max_index.astype(np.int64) + 1, b.max_index.astype(np.int64) + 1
    ea = [m for m in range(a.order) if m not in w["ctr_a"]]
    eb = [m for m in range(b.order) if m not in w["ctr_b"]]
    rowA = _lin(a.coords, ea, ra)
    keyA = _lin(a.coords, w["ctr_a"], ra)
    colB = _lin(b.coords, eb, rb)
    keyB = _lin(b.coords, w["ctr_b"], rb)
    LA = int(np.prod(ra[ea])) if ea else 1
    LB = int(np.prod(rb[eb])) if eb else 1
    return dict(rowA=rowA, keyA=keyA, colB=colB, keyB=keyB, LA=LA, LB=LB, ea=ea, eb=eb, ra=ra, rb=rb)


def _key_sums(keys, vals, ukeys):
    idx = np.searchsorted(ukeys, keys)
    ok = (idx < ukeys.size) & (ukeys[np.minimum(idx, ukeys.size - 1)] == keys)
    s = np.zeros(ukeys.size)
    np.add.at(s, idx[ok], vals[ok])
    return s


def _check_workload(ctx, w, sample_rows):
    import torch
    a, b = w["a"], w["b"]
    h = _host_model(w)
    r = ctx.contract(a, b, w["ctr_a"], w["ctr_b"])
    try:
        n, order = r.nnz, r.order
        cptr, stride, vptr = r.device_pointers()
        vals = torch.as_tensor(_Dev(vptr, n, "<f8"), device="cuda")
        cols = [torch.as_tensor(_Dev(cptr + 4 * m * stride, n, "<i4"), device="cuda").long()
                for m in range(order)]
        na = len(h["ea"])
        ext_r = [int(h["ra"][m]) for m in h["ea"]] + [int(h["rb"][m]) for m in h["eb"]]
        for m in range(order):
            assert int(cols[m].min()) >= 0 and int(cols[m].max()) < ext_r[m]
        row = torch.zeros(n, dtype=torch.long, device="cuda")
        for m in range(na):
            row = row * ext_r[m] + cols[m]
        col = torch.zeros(n, dtype=torch.long, device="cuda")
        for m in range(na, order):
            col = col * ext_r[m] + cols[m]
        # structure: no duplicate (row, col)
        lin = row * h["LB"] + col
        assert torch.unique(lin).numel() == n
        del lin
        # linearity checksum with random weights
        rng = np.random.Generator(np.random.PCG64(2024))
        wr = rng.uniform(-1, 1, h["LA"])
        uc = rng.uniform(-1, 1, h["LB"])
        ukeys = np.unique(np.concatenate([h["keyA"], h["keyB"]]))
        sa = _key_sums(h["keyA"], a.values * wr[h["rowA"]], ukeys)
        sb = _key_sums(h["keyB"], b.values * uc[h["colB"]], ukeys)
        want = float(np.dot(sa, sb))
        sa_abs = _key_sums(h["keyA"], np.abs(a.values * wr[h["rowA"]]), ukeys)
        sb_abs = _key_sums(h["keyB"], np.abs(b.values * uc[h["colB"]]), ukeys)
        scale = float(np.dot(sa_abs, sb_abs))
        wr_t = torch.from_numpy(wr).cuda()
        uc_t = torch.from_numpy(uc).cuda()
        got = float((vals * wr_t[row] * uc_t[col]).sum())
        assert abs(got - want) <= 1e-10 * scale, (got, want, scale)
        # row sums
        sB = _key_sums(h["keyB"], b.values, ukeys)
        sB_abs = _key_sums(h["keyB"], np.abs(b.values), ukeys)
        kidx = np.searchsorted(ukeys, h["keyA"])
        rs_want = np.zeros(h["LA"])
        rs_abs = np.zeros(h["LA"])
        np.add.at(rs_want, h["rowA"], a.values * sB[kidx])
        np.add.at(rs_abs, h["rowA"], np.abs(a.values) * sB_abs[kidx])
        rs_got = torch.zeros(h["LA"], dtype=torch.float64, device="cuda").index_add_(0, row, vals).cpu().numpy()
        assert np.all(np.abs(rs_got - rs_want) <= 1e-11 * rs_abs + 1e-300)
        # exact rows
        orderB = np.argsort(h["keyB"], kind="stable")
        kB = h["keyB"][orderB]
        for rr in sample_rows:
            sel = np.nonzero(h["rowA"] == rr)[0]
            if sel.size == 0:
                continue
            lo = np.searchsorted(kB, h["keyA"][sel], side="left")
            hi = np.searchsorted(kB, h["keyA"][sel], side="right")
            cnt = hi - lo
            tot = int(cnt.sum())
            rep = np.repeat(np.arange(sel.size), cnt)
            offs = np.arange(tot) - np.repeat(np.cumsum(cnt) - cnt, cnt)
            bidx = orderB[np.repeat(lo, cnt) + offs]
            prods = a.values[sel][rep] * b.values[bidx]
            ucol, inv = np.unique(h["colB"][bidx], return_inverse=True)
            wv = np.zeros(ucol.size)
            ws = np.zeros(ucol.size)
            np.add.at(wv, inv, prods)
            np.add.at(ws, inv, np.abs(prods))
            m = (row == rr).nonzero().flatten()
            gc = col[m].cpu().numpy()
            gv = vals[m].cpu().numpy()
            check_parity(gc[:, None], gv, ucol[:, None], wv, ws)
        return n, r.products
    finally:
        r.free()


def test_zipf3_full_size(ctx):
    w = workloads.zipf3(seed=1)
    n, p = _check_workload(ctx, w, sample_rows=[0, 1, 2, 17, 1000, 19999])
    assert p > 4e9 and n > 1e8


def test_twomode_full_size(ctx):
    w = workloads.twomode(seed=1)
    n, p = _check_workload(ctx, w, sample_rows=[0, 1, 50, 4999 * 50 + 49, 123456])
    assert p > 1e8
