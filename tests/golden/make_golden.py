"""Generates tests/golden/*.npz from the reference's own fastcc_multiply.

Run where the reference sources are present (it builds oracle/_ref with
`make -C oracle ref`):

    python tests/golden/make_golden.py

Each fixture stores the seeded inputs and the reference's output triples
(A external linear index, B external linear index, value) as produced by the
reference's tile-pair loop with the recording accumulator of
oracle/ref_harness.cpp, sorted by (left, right). It also stores the entry
count and sorted value multiset returned by the shipped
TileAccumulator<double> path. Inputs come from a fixed numpy PCG64 stream
and are stored in the fixture, so nothing is regenerated at test time.
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


if __name__ == "__main__":
    oracle.build(ref=True)
    for c in CASES:
        make(c)
