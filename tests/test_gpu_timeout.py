"""Bounded device waits: a wait that runs out ends the call with
FCC_ERR_TIMEOUT, and the context stays usable.

The dense tiles stage long B segments in shared memory through a ring of
bulk copies whose waits poll an mbarrier a bounded number of times
(fcc_options.wait_polls). With fcc_options.fault_wait the consumer warps
first wait on an mbarrier that nothing completes, so that wait always runs
out: no GPU fault, no hang, only the status. The same context then
contracts the same operands correctly (oracle parity).
"""
import numpy as np
import pytest

import fastcc_gpu as F
import oracle
import workloads
from helpers import check_parity

pytestmark = pytest.mark.gpu


def _staged_case():
    # Zipf(1.2) self-contraction: hub contraction keys have B segments of
    # thousands of entries, so dense items run phase 1 through the ring (one
    # row per tile leaves room for the ring beside the 5,000-column tile).
    return workloads.zipf3(seed=3, nnz=400_000, dims=(5_000, 2_000, 5_000))


STAGED = {"rows_per_tile": 1, "dense_kernel": 1}


def _check(ctx, w, opts=None):
    a, b = w["a"], w["b"]
    r = ctx.contract(a, b, w["ctr_a"], w["ctr_b"], opts)
    try:
        coords, vals = r.to_numpy()
    finally:
        r.free()
    o = oracle.fastcc_multiply(a.coords, a.values, a.max_index, b.coords, b.values, b.max_index,
                               w["ctr_a"], w["ctr_b"], want_abs=True)
    check_parity(coords, vals, o["coords"], o["values"], o["abs_sum"])


def test_injected_wait_times_out_and_context_recovers():
    w = _staged_case()
    a, b = w["a"], w["b"]
    with F.Context(0) as ctx:
        for polls in (1, 64):
            with pytest.raises(F.FccError) as e:
                ctx.contract(a, b, w["ctr_a"], w["ctr_b"], F.Options(fault_wait=1, wait_polls=polls, **STAGED))
            assert e.value.status == 4, e.value  # FCC_ERR_TIMEOUT
            assert "bounded device wait" in str(e.value)
            _check(ctx, w, F.Options(**STAGED))  # the same context, right after the timeout
            _check(ctx, w)


def test_default_and_short_poll_limits_without_injection_are_exact(ctx):
    # without the injected wait, a limit of 2^16 polls is ample for the ring
    w = _staged_case()
    _check(ctx, w, F.Options(wait_polls=1 << 16, **STAGED))


def test_wait_options_are_validated(ctx):
    w = workloads.readme(seed=1, scale=0.01)
    for bad in (F.Options(wait_polls=-1), F.Options(fault_wait=2)):
        with pytest.raises(F.FccError) as e:
            ctx.contract(w["a"], w["b"], w["ctr_a"], w["ctr_b"], bad)
        assert e.value.status == 1
