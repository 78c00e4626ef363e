"""Generates tests/golden/*.npz from the reference's own fastcc_multiply.

Run where the reference sources are present (it builds oracle/_ref with
`make -C oracle ref`):

    python tests/golden/make_golden.py [fastcc | modes]

Each fastcc fixture stores the seeded inputs and the reference's output triples
(A external linear index, B external linear index, value) as produced by the
reference's tile-pair loop with the recording accumulator of
oracle/ref_harness.cpp, sorted by (left, right). It also stores the entry
count and sorted value multiset returned by the shipped
TileAccumulator<double> path. Inputs come from a fixed numpy PCG64 stream
and are stored in the fixture, so nothing is regenerated at test time.

The modes_*.npz fixtures hold the reference's Tensor::multiply with batch
modes (contract.hpp:286-367) on seeded inputs: its output coordinates (batch
modes, A external, B external) sorted lexicographically, with their values.
The reference infers each operand's shape from its nonzeros, so every operand
holds its corner nonzero (every mode at its largest index), which makes the
paired modes of the two operands share their extents.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402


def distinct_coords(rng, dims, nnz, zipf=None):
    dims = np.asarray(dims, np.int64)
    seen = {}
    out = []
    while len(out) < nnz:
        c = []
        for m, d in enumerate(dims):
            if zipf and zipf[m] > 0:
                w = np.arange(1, d + 1, dtype=np.float64) ** (-zipf[m])
                c.append(int(rng.choice(d, p=w / w.sum())))
            else:
                c.append(int(rng.integers(0, d)))
        t = tuple(c)
        if t not in seen:
            seen[t] = 1
            out.append(c)
    return np.array(out, np.int32).reshape(nnz, len(dims))


CASES = [
    # name, seed, dims_a, nnz_a, dims_b, nnz_b, ctr_a, ctr_b, tile, zipf_a, zipf_b, self
    ("readme_small_t16", 11, [24, 6, 20, 5], 1500, [30, 6, 5], 400, [1, 3], [1, 2], 16, None, None, False),
    ("readme_small_t128", 12, [24, 6, 20, 5], 1500, [30, 6, 5], 400, [1, 3], [1, 2], 128, None, None, False),
    ("readme_small_t1", 13, [10, 4, 9, 3], 300, [12, 4, 3], 100, [1, 3], [1, 2], 1, None, None, False),
    ("zipf3_self", 14, [60, 60, 200], 2500, None, None, [1, 2], [1, 2], 100, [1.2, 1.2, 1.2], None, True),
    ("twomode_self", 15, [40, 40, 30, 5], 2000, None, None, [0, 2], [0, 2], 64, [1.1, 1.1, 0, 0], None, True),
    ("outer_k0", 16, [7, 5], 20, [6, 4], 15, [], [], 8, None, None, False),
    ("full_contraction", 17, [9, 8, 7], 150, [9, 8, 7], 120, [0, 1, 2], [0, 1, 2], 100, None, None, False),
    ("order1_dot_like", 18, [50, 6], 120, [40, 6], 90, [0], [0], 32, None, None, False),
    ("reordered_ctr", 19, [12, 7, 9, 5], 600, [5, 11, 7], 200, [3, 1], [0, 2], 100, None, None, False),
    ("tile_2000", 20, [24, 6, 20, 5], 1500, [30, 6, 5], 400, [1, 3], [1, 2], 2000, None, None, False),
]


def make(case):
    (name, seed, da, na, db, nb, ca, cb, tile, za, zb, selfc) = case
    rng = np.random.Generator(np.random.PCG64(seed))
    a_c = distinct_coords(rng, da, na, za)
    a_v = rng.uniform(-1.0, 1.0, na)
    if selfc:
        b_c, b_v, db = a_c, a_v, da
    else:
        b_c = distinct_coords(rng, db, nb, zb)
        b_v = rng.uniform(-1.0, 1.0, nb)
    a_m = np.asarray(da, np.int32) - 1
    b_m = np.asarray(db, np.int32) - 1
    ref = oracle.reference_multiply(a_c, a_v, a_m, b_c, b_v, b_m, ca, cb, tile_size=tile)
    order = np.lexsort((ref["right"], ref["left"]))
    shipped = oracle.reference_multiply(a_c, a_v, a_m, b_c, b_v, b_m, ca, cb, tile_size=tile, shipped=True)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(
        path, a_coords=a_c, a_vals=a_v, a_max=a_m, b_coords=b_c, b_vals=b_v, b_max=b_m,
        ctr_a=np.asarray(ca, np.int32), ctr_b=np.asarray(cb, np.int32), tile=np.int32(tile),
        left=ref["left"][order], right=ref["right"][order], values=ref["values"][order],
        out_order=np.int32(ref["order"]), shipped_count=np.int64(len(shipped["values"])),
        shipped_sorted_values=np.sort(shipped["values"]))
    print(f"{name}: {len(order)} outputs, shipped {len(shipped['values'])} -> {os.path.basename(path)}")


MODE_CASES = [
    # name, seed, A extents, B extents, ctr_a, ctr_b, batch_a, batch_b, nnz_a, nnz_b
    ("modes_bik_bkj", 31, [6, 7, 5], [6, 5, 8], [2], [1], [0], [0], 150, 120),
    ("modes_two_ctr", 32, [4, 9, 3, 5], [5, 3, 4, 7], [1, 2], [2, 1], [3], [0], 300, 250),
    ("modes_no_a_ext", 33, [5, 6], [6, 5], [1], [0], [0], [1], 25, 25),
    ("modes_batched_outer", 34, [3, 4, 5], [5, 4, 3], [], [], [0, 1], [2, 1], 40, 50),
    ("modes_mid_batch", 35, [8, 6, 4], [4, 6, 9], [1], [1], [2], [0], 120, 150),
]


def corner_tensor(rng, ext, n):
    """n distinct uniform coordinates, the first at the corner (every mode at
    its largest index)."""
    space = int(np.prod(ext))
    n = min(n, space)
    lin = rng.choice(space, size=n, replace=False)
    lin[0] = space - 1 if (space - 1) not in lin[1:] else lin[0]
    if lin[0] != space - 1:
        lin[np.nonzero(lin == space - 1)[0][0]] = lin[0]
        lin[0] = space - 1
    c = np.stack(np.unravel_index(lin, ext), axis=1).astype(np.int32).reshape(n, len(ext))
    return c, rng.uniform(-1.0, 1.0, n)


def make_modes(case):
    name, seed, ea, eb, ca, cb, ba, bb, na, nb = case
    eb = list(eb)
    for x, y in list(zip(ca, cb)) + list(zip(ba, bb)):  # paired modes share their extent
        eb[y] = ea[x]
    rng = np.random.Generator(np.random.PCG64(seed))
    ac, av = corner_tensor(rng, ea, na)
    bc, bv = corner_tensor(rng, eb, nb)
    am, bm = ac.max(axis=0).astype(np.int32), bc.max(axis=0).astype(np.int32)
    coords, vals = oracle.reference_multiply_modes(ac, av, am, bc, bv, bm, ca, cb, ba, bb)
    order = np.lexsort(coords.T[::-1]) if coords.shape[0] and coords.shape[1] else np.arange(len(vals))
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(
        path, a_coords=ac, a_vals=av, a_max=am, b_coords=bc, b_vals=bv, b_max=bm,
        ctr_a=np.asarray(ca, np.int32), ctr_b=np.asarray(cb, np.int32), batch_a=np.asarray(ba, np.int32),
        batch_b=np.asarray(bb, np.int32), coords=coords[order], values=vals[order])
    print(f"{name}: {len(vals)} outputs -> {os.path.basename(path)}")


if __name__ == "__main__":
    oracle.build(ref=True)
    which = sys.argv[1] if len(sys.argv) > 1 else "all"
    if which in ("all", "fastcc"):
        for c in CASES:
            make(c)
    if which in ("all", "modes"):
        for c in MODE_CASES:
            make_modes(c)
