"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Bar (tests/helpers.py): bit-exact output coordinate set; |x - y| <= 1e-12 * S
per value, S = the oracle's sum of |a*b| over the output's products.
"""
import numpy as np
import pytest

import fastcc_gpu as F
import oracle
import workloads
from helpers import check_parity, golden_names, load_golden

pytestmark = pytest.mark.gpu


def run_gpu(ctx, ac, av, am, bc, bv, bm, ca, cb, **opts):
    r = ctx.contract(F.Tensor(ac, av, am), F.Tensor(bc, bv, bm), ca, cb, F.Options(**opts))
    try:
        c, v = r.to_numpy()
        return c, v, r.products
    finally:
        r.free()


def run_oracle(ac, av, am, bc, bv, bm, ca, cb, tile=100):
    return oracle.fastcc_multiply(ac, av, am, bc, bv, bm, ca, cb, tile_size=tile, want_abs=True)


VARIANTS = [
    {},
    {"accumulator": F.ACC_HASH},
    {"products_per_item": 7},                               # forces split tiles
    {"accumulator": F.ACC_HASH, "products_per_item": 5},    # expand-sort-reduce (default)
    {"accumulator": F.ACC_HASH, "products_per_item": 5, "hash_esc": -1},   # global hash merge
    {"accumulator": F.ACC_HASH, "hash_slots": 64, "hash_esc": -1},
    {"schedule": F.SCHED_FORCE + F.CLASS_HASH_S, "products_per_item": 40, "hash_esc": -1},
    {"rows_per_tile": 1},
    {"dense_cap": 2048, "products_per_item": 300},
    {"capacity_hint": 3},                                   # overflow -> exact-count retry
    {"hash_slots": 64},
    {"dense_mode": F.DENSE_SENTINEL},
    {"dense_mode": F.DENSE_SENTINEL, "products_per_item": 9},
    {"dense_mode": F.DENSE_BITMASK, "products_per_item": 11},
    {"hot_columns": 32, "rows_per_tile": 1},
    {"hot_columns": 32, "rows_per_tile": 1, "dense_mode": F.DENSE_BITMASK, "products_per_item": 13},
    {"hot_columns": 64, "accumulator": F.ACC_HASH},
    {"hot_columns": 32, "accumulator": F.ACC_HASH, "products_per_item": 6, "tile_threads": 512},
    {"tile_threads": 512, "hot_columns": -1},
    {"tile_threads": 640},
    {"tile_threads": 768, "products_per_item": 9},
    {"accumulator": F.ACC_HASH, "products_per_item": 5, "hash_esc": 1},    # expand-sort-reduce of split tiles
    {"accumulator": F.ACC_HASH, "hash_slots": 64, "hash_esc": 1},
    {"schedule": F.SCHED_FORCE + F.CLASS_HASH_S, "products_per_item": 40, "hash_esc": 1},
    {"accumulator": F.ACC_HASH, "hash_esc": 2},                               # every hash tile expanded
    {"accumulator": F.ACC_HASH, "hash_esc": 2, "esc_group": 3},               # ... sorted in groups of 3 tiles
    {"accumulator": F.ACC_HASH, "products_per_item": 6, "esc_group": 1},
    {"dense_kernel": 2},                                                     # flat dense items
    {"dense_kernel": 2, "products_per_item": 7, "dense_mode": F.DENSE_BITMASK},
    {"dense_kernel": 2, "rows_per_tile": 1, "dense_mode": F.DENSE_SENTINEL},
    {"dense_kernel": 2, "hot_columns": 32, "rows_per_tile": 1, "tile_threads": 512},
    {"dense_kernel": 1},
    {"dense_kernel": 3},                                                     # flat phase 2
    {"dense_kernel": 3, "products_per_item": 7, "dense_mode": F.DENSE_BITMASK, "rows_per_tile": 1},
    {"dense_kernel": 3, "hot_columns": 32, "rows_per_tile": 1},             # private hot columns, plain updates
    {"dense_kernel": 2, "hot_columns": 64, "rows_per_tile": 1, "dense_mode": F.DENSE_BITMASK,
     "products_per_item": 9},
    {"accumulator": F.ACC_HASH, "esc_reduce": 2},                             # expanded pairs radix-sorted
    {"accumulator": F.ACC_HASH, "products_per_item": 5, "esc_reduce": 2, "esc_group": 2},
    {"accumulator": F.ACC_HASH, "esc_small": 1},                              # every tile partitioned by key blocks
    {"accumulator": F.ACC_HASH, "esc_small": 24, "esc_group": 3},
    {"accumulator": F.ACC_HASH, "esc_small": 7, "capacity_hint": 5},          # ... and the exact-count retry
]


def _args(g):
    return (g["a_coords"], g["a_vals"], g["a_max"], g["b_coords"], g["b_vals"], g["b_max"],
            g["ctr_a"], g["ctr_b"])


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("vi", range(len(VARIANTS)))
def test_golden_parity(ctx, name, vi):
    g = load_golden(name)
    opts = dict(VARIANTS[vi])
    opts.setdefault("tile_size", int(g["tile"]))
    o = run_oracle(*_args(g), tile=int(g["tile"]))
    # the oracle reproduces the reference's triples bit-exactly (CPU test);
    # re-check here so the GPU comparison is anchored to the fixture
    idx = np.lexsort((o["right"], o["left"]))
    assert np.array_equal(o["values"][idx], g["values"])
    c, v, prods = run_gpu(ctx, *_args(g), **opts)
    assert prods == o["products"]
    check_parity(c, v, o["coords"], o["values"], o["abs_sum"])


def _rand_case(rng, order_a, order_b, k, max_dim=9, nnz_a=300, nnz_b=200):
    ext_a = [int(x) for x in rng.integers(1, max_dim, size=order_a)]
    ext_b = [int(x) for x in rng.integers(1, max_dim, size=order_b)]
    ca = [int(x) for x in rng.permutation(order_a)[:k]]
    cb = [int(x) for x in rng.permutation(order_b)[:k]]
    for x, y in zip(ca, cb):
        ext_b[y] = ext_a[x]

    def gen(ext, n):
        space = int(np.prod(ext))
        n = min(n, space)
        lin = rng.choice(space, size=n, replace=False)
        c = np.stack(np.unravel_index(lin, ext), axis=1).astype(np.int32)
        return c.reshape(n, len(ext)), rng.uniform(-1, 1, n)

    ac, av = gen(ext_a, nnz_a)
    bc, bv = gen(ext_b, nnz_b)
    return ac, av, np.array(ext_a, np.int32) - 1, bc, bv, np.array(ext_b, np.int32) - 1, ca, cb


@pytest.mark.parametrize("seed", range(40))
def test_random_parity(ctx, seed):
    rng = np.random.Generator(np.random.PCG64(5000 + seed))
    oa, ob = int(rng.integers(1, 6)), int(rng.integers(1, 6))
    k = int(rng.integers(0, min(oa, ob) + 1))
    case = _rand_case(rng, oa, ob, k, max_dim=int(rng.integers(2, 14)),
                      nnz_a=int(rng.integers(1, 3000)), nnz_b=int(rng.integers(1, 2000)))
    variant = VARIANTS[seed % len(VARIANTS)]
    o = run_oracle(*case)
    c, v, prods = run_gpu(ctx, *case, **variant)
    assert prods == o["products"]
    check_parity(c, v, o["coords"], o["values"], o["abs_sum"])


def test_readme_workload_full_size(ctx):
    w = workloads.readme(seed=1)
    a, b = w["a"], w["b"]
    args = (a.coords, a.values, a.max_index, b.coords, b.values, b.max_index, w["ctr_a"], w["ctr_b"])
    o = run_oracle(*args, tile=128)
    for opts in ({}, {"accumulator": F.ACC_HASH}):
        c, v, prods = run_gpu(ctx, *args, **opts)
        assert prods == o["products"]
        n, maxrel, canc = check_parity(c, v, o["coords"], o["values"], o["abs_sum"])
        assert n == len(o["values"]) > 4_000_000


def test_wide_b_span_uses_64bit_columns(ctx):
    # B external span 70000 x 70000 > 2^32 forces the hash accumulator with 64-bit columns
    rng = np.random.Generator(np.random.PCG64(77))
    n = 4000
    a_c = np.stack([rng.integers(0, 50, n), rng.integers(0, 30, n)], axis=1).astype(np.int32)
    a_c = np.unique(a_c, axis=0)
    a_v = rng.uniform(-1, 1, a_c.shape[0])
    b_c = np.stack([rng.integers(0, 70000, n), rng.integers(0, 30, n), rng.integers(0, 70000, n)], axis=1)
    b_c = np.unique(b_c.astype(np.int32), axis=0)
    b_v = rng.uniform(-1, 1, b_c.shape[0])
    am, bm = np.array([49, 29], np.int32), np.array([69999, 29, 69999], np.int32)
    args = (a_c, a_v, am, b_c, b_v, bm, [1], [1])
    o = run_oracle(*args)
    for opts in ({}, {"products_per_item": 3}):
        c, v, prods = run_gpu(ctx, *args, **opts)
        check_parity(c, v, o["coords"], o["values"], o["abs_sum"])


def test_device_resident_and_soa_inputs(ctx):
    import torch
    w = workloads.readme(seed=3, scale=0.05)
    a, b = w["a"], w["b"]
    args = (a.coords, a.values, a.max_index, b.coords, b.values, b.max_index, w["ctr_a"], w["ctr_b"])
    o = run_oracle(*args)
    ta = F.Tensor(torch.from_numpy(a.coords).cuda(), torch.from_numpy(a.values).cuda(), a.max_index)
    # SoA layout on the device: a transposed view has stride_nnz = 1
    soa = torch.from_numpy(np.ascontiguousarray(b.coords.T)).cuda().t()
    tb = F.Tensor(soa, torch.from_numpy(b.values).cuda(), b.max_index)
    r = ctx.contract(ta, tb, w["ctr_a"], w["ctr_b"])
    c, v = r.to_numpy()
    r.free()
    check_parity(c, v, o["coords"], o["values"], o["abs_sum"])


def test_repeated_calls_are_stable(ctx):
    w = workloads.readme(seed=4, scale=0.1)
    a, b = w["a"], w["b"]
    ref = None
    for _ in range(6):
        c, v = ctx.fastcc_multiply(a, b, w["ctr_a"], w["ctr_b"])
        from helpers import sort_rows
        c, v = sort_rows(c, v)
        if ref is None:
            ref = (c, v)
        else:
            assert np.array_equal(c, ref[0])
            assert np.allclose(v, ref[1], rtol=1e-12, atol=1e-14)


def test_empty_and_no_match(ctx):
    c0 = np.zeros((0, 3), np.int32)
    a = F.Tensor(c0, np.zeros(0), np.array([3, 3, 3], np.int32))
    b = F.Tensor(np.array([[1, 2]], np.int32), np.array([1.0]), np.array([3, 3], np.int32))
    r = ctx.contract(a, b, [0], [0])
    assert r.nnz == 0 and r.order == 3
    r.free()
    a = F.Tensor(np.array([[0, 0, 0]], np.int32), np.array([2.0]), np.array([3, 3, 3], np.int32))
    b = F.Tensor(np.array([[1, 2]], np.int32), np.array([1.0]), np.array([3, 3], np.int32))
    r = ctx.contract(a, b, [0], [0])  # key 0 vs key 1: no match
    assert r.nnz == 0 and r.products == 0
    r.free()


def test_exact_zero_sums_are_emitted(ctx):
    # a(i,c) * b(j,c): two keys whose products cancel exactly at (0,0)
    a = F.Tensor(np.array([[0, 0], [0, 1]], np.int32), np.array([1.0, 1.0]), np.array([0, 1], np.int32))
    b = F.Tensor(np.array([[0, 0], [0, 1]], np.int32), np.array([2.0, -2.0]), np.array([0, 1], np.int32))
    for acc in (F.ACC_DENSE, F.ACC_HASH):
        for mode in (F.DENSE_AUTO, F.DENSE_BITMASK, F.DENSE_SENTINEL):
            r = ctx.contract(a, b, [1], [1], F.Options(accumulator=acc, dense_mode=mode))
            c, v = r.to_numpy()
            r.free()
            assert c.tolist() == [[0, 0]] and v.tolist() == [0.0]


def test_zero_valued_inputs_keep_touched_positions(ctx):
    # zero inputs make products of -0.0 and +0.0; every touched position is
    # still emitted (the -0.0 sentinel is not used for such inputs)
    rng = np.random.Generator(np.random.PCG64(31))
    g = load_golden("readme_small_t16")
    av = g["a_vals"].copy()
    bv = g["b_vals"].copy()
    av[rng.choice(av.size, av.size // 3, replace=False)] = 0.0
    bv[rng.choice(bv.size, bv.size // 3, replace=False)] = -0.0
    args = (g["a_coords"], av, g["a_max"], g["b_coords"], bv, g["b_max"], g["ctr_a"], g["ctr_b"])
    o = run_oracle(*args)
    for mode in (F.DENSE_AUTO, F.DENSE_SENTINEL, F.DENSE_BITMASK):
        c, v, _ = run_gpu(ctx, *args, dense_mode=mode)
        check_parity(c, v, o["coords"], o["values"], o["abs_sum"])


def test_full_contraction_is_a_scalar(ctx):
    g = load_golden("full_contraction")
    c, v, _ = run_gpu(ctx, *_args(g))
    assert c.shape == (1, 0)
    assert abs(v[0] - g["values"][0]) <= 1e-12 * np.sum(np.abs(g["values"])) + 1e-12


def test_errors_are_statuses(ctx):
    a = F.Tensor(np.array([[0, 5]], np.int32), np.array([1.0]), np.array([3, 3], np.int32))
    b = F.Tensor(np.array([[0, 1]], np.int32), np.array([1.0]), np.array([3, 3], np.int32))
    with pytest.raises(F.FccError) as e:
        ctx.contract(a, b, [0], [0])  # coordinate 5 > max_index 3
    assert e.value.status == 1
    with pytest.raises(F.FccError) as e:
        ctx.contract(a, b, [0, 0], [0, 1])
    assert e.value.status == 1
    big = np.full(8, 2**31 - 2, np.int32)
    t = F.Tensor(np.zeros((1, 8), np.int32), np.array([1.0]), big)
    with pytest.raises(F.FccError) as e:
        ctx.contract(t, t, [0], [0])
    assert e.value.status == 6
    # the context stays usable after errors
    c, v = ctx.fastcc_multiply(b, b, [0], [0])
    assert c.tolist() == [[1, 1]] and v.tolist() == [1.0]


def test_count_products_matches_oracle(ctx):
    w = workloads.readme(seed=6, scale=0.2)
    a, b = w["a"], w["b"]
    n = ctx.count_products(a, b, w["ctr_a"], w["ctr_b"])
    assert n == oracle.count_products(a.coords, a.values, a.max_index, b.coords, b.values, b.max_index,
                                      w["ctr_a"], w["ctr_b"])


def test_launch_counter_counts_kernels(ctx):
    w = workloads.readme(seed=7, scale=0.02)
    before = F.launch_count()
    ctx.fastcc_multiply(w["a"], w["b"], w["ctr_a"], w["ctr_b"])
    assert F.launch_count() - before >= 10


@pytest.mark.parametrize("staging", [0, -1])
def test_staged_phase1_matches_oracle(ctx, staging):
    # B span 16,000: one-row dense tiles with room for the staging ring; Zipf hub
    # segments of thousands of entries put most multiply-adds in phase 1
    w = workloads.zipf3(seed=41, nnz=150_000, dims=(16_000, 16_000, 400))
    a, b = w["a"], w["b"]
    args = (a.coords, a.values, a.max_index, b.coords, b.values, b.max_index, w["ctr_a"], w["ctr_b"])
    o = run_oracle(*args, tile=128)
    for opts in ({"dense_staging": staging}, {"dense_staging": staging, "dense_mode": F.DENSE_BITMASK},
                 {"dense_staging": staging, "products_per_item": 3000}):
        c, v, prods = run_gpu(ctx, *args, **opts)
        assert prods == o["products"]
        check_parity(c, v, o["coords"], o["values"], o["abs_sum"])


@pytest.mark.parametrize("rows,cols,k", [(3, 2, 4000), (1, 1, 70_000), (40, 37, 300)])
def test_long_runs_of_equal_outputs(ctx, rows, cols, k):
    # C(i, j) = sum_k A(i, k) B(k, j) with every k present: each output gets k
    # products, so the sorted pairs of a split hash tile hold runs of k equal
    # keys that cross many 256-position chunks of the reduction
    rng = np.random.Generator(np.random.PCG64(rows * 1000 + k))
    ii, kk = np.meshgrid(np.arange(rows), np.arange(k), indexing="ij")
    a_c = np.stack([ii.ravel(), kk.ravel()], axis=1).astype(np.int32)
    kk2, jj = np.meshgrid(np.arange(k), np.arange(cols), indexing="ij")
    b_c = np.stack([kk2.ravel(), jj.ravel()], axis=1).astype(np.int32)
    a_v = rng.uniform(-1, 1, a_c.shape[0])
    b_v = rng.uniform(-1, 1, b_c.shape[0])
    am, bm = np.array([rows - 1, k - 1], np.int32), np.array([k - 1, cols - 1], np.int32)
    args = (a_c, a_v, am, b_c, b_v, bm, [1], [0])
    o = run_oracle(*args)
    for opts in ({"accumulator": F.ACC_HASH, "hash_slots": 64},
                 {"accumulator": F.ACC_HASH, "hash_slots": 64, "esc_group": 2},
                 {"accumulator": F.ACC_HASH, "hash_slots": 64, "hash_esc": -1},
                 {"accumulator": F.ACC_HASH, "products_per_item": 100},
                 {"accumulator": F.ACC_HASH, "esc_reduce": 2},
                 {"accumulator": F.ACC_HASH, "esc_small": 1}):
        c, v, prods = run_gpu(ctx, *args, **opts)
        assert prods == o["products"] == rows * cols * k
        check_parity(c, v, o["coords"], o["values"], o["abs_sum"])


@pytest.mark.parametrize("opts", [{}, {"esc_small": 1}, {"esc_small": 300}, {"esc_small": 4096, "esc_group": 7},
                                  {"esc_reduce": 2}])
def test_expanded_pairs_reduced_by_key_blocks(ctx, opts):
    # two-mode shape with a 40,000-column B span (5 key blocks of 8192): hub
    # rows hold dense blocks (over 2048 pairs) and runs of sparse ones, the
    # other rows go through the windows of small tiles
    w = workloads.twomode(seed=3, nnz=400_000, dims=(800, 800, 300, 50))
    a = w["a"]
    args = (a.coords, a.values, a.max_index, a.coords, a.values, a.max_index, w["ctr_a"], w["ctr_b"])
    o = run_oracle(*args)
    c, v, prods = run_gpu(ctx, *args, **opts)
    assert prods == o["products"]
    n, _, _ = check_parity(c, v, o["coords"], o["values"], o["abs_sum"])
    assert n == len(o["values"])
