"""fcc_contract_into: the contraction written into caller buffers (device
memory or pinned host memory), checked against the oracle."""
import numpy as np
import pytest

import fastcc_gpu as F
import oracle
import workloads
from helpers import check_parity

pytestmark = pytest.mark.gpu


def _case():
    w = workloads.readme(seed=17, scale=0.04)
    a, b = w["a"], w["b"]
    o = oracle.fastcc_multiply(a.coords, a.values, a.max_index, b.coords, b.values, b.max_index, w["ctr_a"],
                               w["ctr_b"], want_abs=True)
    return w, o


@pytest.mark.parametrize("where", ["device", "pinned"])
def test_into_caller_buffers(ctx, where):
    import torch
    w, o = _case()
    n = len(o["values"])
    order = o["coords"].shape[1]
    if where == "device":
        oc = torch.empty((order, n + 7), dtype=torch.int32, device="cuda")
        ov = torch.empty(n + 7, dtype=torch.float64, device="cuda")
    else:
        oc = torch.empty((order, n + 7), dtype=torch.int32).pin_memory().numpy()
        ov = torch.empty(n + 7, dtype=torch.float64).pin_memory().numpy()
    got, prods = ctx.contract_into(w["a"], w["b"], w["ctr_a"], w["ctr_b"], oc, ov)
    assert got == n and prods == o["products"]
    if where == "device":
        oc, ov = oc.cpu().numpy(), ov.cpu().numpy()
    check_parity(oc[:, :n].T, ov[:n], o["coords"], o["values"], o["abs_sum"])


@pytest.mark.parametrize("opts", [{"out_waves": 2}, {"out_waves": 5, "products_per_item": 40},
                                  {"out_waves": 16, "accumulator": F.ACC_HASH, "products_per_item": 30},
                                  {"out_waves": 3, "accumulator": F.ACC_HASH, "hash_slots": 64, "hash_esc": -1}])
def test_into_pinned_in_waves(ctx, opts):
    # pinned host output: produced on the device in waves of tiles, each
    # wave's range copied out while the next runs; split tiles and expanded
    # tiles come after the last wave
    import torch
    w, o = _case()
    n = len(o["values"])
    order = o["coords"].shape[1]
    oc = torch.full((order, n + 100), -1, dtype=torch.int32).pin_memory().numpy()
    ov = torch.full((n + 100,), np.nan, dtype=torch.float64).pin_memory().numpy()
    got, prods = ctx.contract_into(w["a"], w["b"], w["ctr_a"], w["ctr_b"], oc, ov, F.Options(**opts))
    assert got == n and prods == o["products"]
    check_parity(oc[:, :n].T, ov[:n], o["coords"], o["values"], o["abs_sum"])
    assert (oc[:, n:] == -1).all() and np.isnan(ov[n:]).all()  # nothing written past the output


def test_into_too_small_reports_the_size(ctx):
    import torch
    w, o = _case()
    n = len(o["values"])
    order = o["coords"].shape[1]
    small_c = torch.empty((order, n // 3), dtype=torch.int32).pin_memory().numpy()
    small_v = torch.empty(n // 3, dtype=torch.float64).pin_memory().numpy()
    with pytest.raises(F.FccError) as e:
        ctx.contract_into(w["a"], w["b"], w["ctr_a"], w["ctr_b"], small_c, small_v)
    assert e.value.status == 8 and e.value.needed == n
    with pytest.raises(F.FccError) as e:  # a size query
        ctx.contract_into(w["a"], w["b"], w["ctr_a"], w["ctr_b"], np.zeros((order, 0), np.int32), np.zeros(0))
    assert e.value.status == 8 and e.value.needed == n
    c = torch.empty((order, n), dtype=torch.int32).pin_memory().numpy()
    v = torch.empty(n, dtype=torch.float64).pin_memory().numpy()
    got, _ = ctx.contract_into(w["a"], w["b"], w["ctr_a"], w["ctr_b"], c, v)
    assert got == n
    check_parity(c.T, v, o["coords"], o["values"], o["abs_sum"])
    # the context still serves ordinary calls
    r = ctx.contract(w["a"], w["b"], w["ctr_a"], w["ctr_b"])
    assert r.nnz == n
    r.free()


def test_into_rejects_missing_coordinates(ctx):
    import ctypes
    w, o = _case()
    ta, tb = w["a"]._struct(), w["b"]._struct()
    ca = np.array(w["ctr_a"], np.int32)
    cb = np.array(w["ctr_b"], np.int32)
    v = np.zeros(len(o["values"]))
    n, p = ctypes.c_int64(), ctypes.c_int64()
    rc = F.lib().fcc_contract_into(ctx._h, ctypes.byref(ta), ctypes.byref(tb), ca.ctypes.data, cb.ctypes.data,
                                   2, ctypes.byref(F.Options()), None, v.shape[0], v.ctypes.data, v.shape[0],
                                   ctypes.byref(n), ctypes.byref(p))
    assert rc == 1
