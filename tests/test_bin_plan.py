"""CPU checks of the capacity arguments behind the shared-memory reduction
of expanded hash tiles (csrc/fcc_contract.cu, "expanded pairs reduced in
shared memory").

The kernels rely on bounds that follow from their constants: a window of
small tiles holds fewer than kBinWindow + small_max positions and at most
kBinWindow / 8 + 1 tiles, so its hash table (the smallest power of two above
4/3 of its positions) fits kBinSlots and its keys (rank x span + local key)
stay below kBinEmpty; a large tile's jobs are single dense blocks or runs of
sparse blocks that fit a table; the chunk and job arrays the host allocates
are large enough. This test restates the planning (tile prefixes, windows,
chunks, jobs) in numpy on the per-tile, per-block pair counts of a seeded
two-mode contraction and on adversarial size patterns, with the constants
read from the CUDA source, and checks every bound.
"""
import os
import re

import numpy as np
import pytest

import workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "fastcc-benchmark_gb300", "csrc", "fcc_contract.cu")


def constants():
    text = open(SRC).read()
    out = {}
    for name in ("kBinBits", "kBinMaxBlocks", "kBinChunk", "kBinWindow", "kBinSmallMax", "kBinDenseMin",
                 "kBinHashPairs", "kBinSlots", "kBinPer"):
        m = re.search(r"constexpr (?:u32|int) %s = (\d+)u?;" % name, text)
        assert m, name
        out[name] = int(m.group(1))
    out["kBinWidth"] = 1 << out["kBinBits"]
    return out


C = constants()


def table_slots(np_):
    lg = 5
    while (1 << lg) < np_ + np_ // 3 + 1:
        lg += 1
    return 1 << lg


def plan(pairs, block_counts, span, small_max):
    """pairs[s]: pairs of esc tile s; block_counts[s]: its pairs per key block
    (large tiles). Returns the windows, jobs and chunk count, checking the
    kernels' bounds on the way."""
    per, W, K = C["kBinPer"], C["kBinWindow"], C["kBinChunk"]
    pairs = np.asarray(pairs, np.int64)
    n = len(pairs)
    large = pairs > small_max
    pad = (pairs + per - 1) // per * per
    ssz = np.where(large, 0, pad)
    spp = np.concatenate([[0], np.cumsum(ssz)])
    srk = np.concatenate([[0], np.cumsum(~large)])
    nch = np.where(large, (pairs + K - 1) // K, 0)
    assert spp[-1] + per * n < 2 ** 32  # the host's condition for this path
    nwin = -(-int(spp[-1]) // W)
    first = np.searchsorted(spp[:n], np.arange(nwin + 1, dtype=np.int64) * W, side="left")
    windows = []
    for w in range(nwin):
        f0, f1 = first[w], first[w + 1]
        lo, hi = spp[f0], spp[f1]
        positions = int(hi - lo)
        assert positions < W + small_max
        assert table_slots(positions) <= C["kBinSlots"]
        ntiles = int(srk[f1] - srk[f0])  # small tiles in the window
        assert ntiles <= W // per + 1
        assert (ntiles - 1) * span + span - 1 < 0xFFFFFFFF  # the largest key, below the empty marker
        windows.append((positions, ntiles))
    nb = -(-span // C["kBinWidth"])
    assert nb <= C["kBinMaxBlocks"]
    jobs = []
    for s in np.nonzero(large)[0]:
        cnt = np.asarray(block_counts[s], np.int64)
        assert cnt.sum() == pairs[s] and len(cnt) == nb
        run0, runp = 0, 0
        tile_jobs = []
        for blk, c in enumerate(cnt):
            if c > C["kBinDenseMin"]:
                if runp:
                    tile_jobs.append((run0, blk, runp))
                tile_jobs.append((blk, blk + 1, int(c)))
                run0, runp = blk + 1, 0
            elif runp + c > C["kBinHashPairs"]:
                tile_jobs.append((run0, blk, runp))
                run0, runp = blk, int(c)
            else:
                runp += int(c)
        if runp:
            tile_jobs.append((run0, nb, runp))
        assert len(tile_jobs) <= nb
        for b0, b1, p in tile_jobs:
            dense = b1 == b0 + 1 and p > C["kBinDenseMin"]
            if not dense:
                assert p <= C["kBinHashPairs"] and table_slots(p) <= C["kBinSlots"]
        assert sum(p for _, _, p in tile_jobs) == pairs[s]
        jobs += tile_jobs
    total = int(pairs.sum())
    maxch = total // K + total // (small_max + 1) + 1  # the host's chunk bound
    assert nch.sum() <= maxch
    maxjobs = nb * min(n, total // (small_max + 1) + 1)  # the host's job bound
    assert len(jobs) <= maxjobs
    return windows, jobs, int(nch.sum())


def twomode_counts(nnz, dims, seed=5):
    """Per-row pairs and per-(row, block) pairs of a two-mode self-contraction
    (one row per tile, as the planner makes it for this shape)."""
    w = workloads.twomode(seed=seed, nnz=nnz, dims=dims)
    c = w["a"].coords.astype(np.int64)
    d0, d1, d2, d3 = dims
    key = c[:, 0] * d2 + c[:, 2]
    row = c[:, 1] * d3 + c[:, 3]
    span = d1 * d3
    order = np.argsort(key, kind="stable")
    ks, rows_sorted = key[order], row[order]
    starts = np.searchsorted(ks, ks, side="left")
    ends = np.searchsorted(ks, ks, side="right")
    # every (A entry, B entry) pair with equal keys: expand by segment
    seg_len = ends - starts
    a_rows = np.repeat(rows_sorted, seg_len)
    b_idx = np.concatenate([np.arange(s, e) for s, e in zip(starts, ends)]) if len(ks) else np.zeros(0, int)
    cols = rows_sorted[b_idx]
    urows, tile = np.unique(a_rows, return_inverse=True)
    pairs = np.bincount(tile, minlength=len(urows))
    nb = -(-span // C["kBinWidth"])
    blk = cols // C["kBinWidth"]
    bc = np.zeros((len(urows), nb), np.int64)
    np.add.at(bc, (tile, blk), 1)
    return pairs, bc, span


@pytest.mark.parametrize("small_max", [None, 1, 300])
def test_twomode_plan_respects_the_kernel_bounds(small_max):
    pairs, bc, span = twomode_counts(60_000, (400, 400, 150, 50))
    sm = C["kBinSmallMax"] if small_max is None else small_max
    windows, jobs, chunks = plan(pairs, bc, span, sm)
    assert sum(p for _, _, p in jobs) + sum(int(x) for x in pairs if x <= sm) == pairs.sum()
    if small_max is None:
        assert windows and jobs  # both paths taken


def test_adversarial_sizes():
    span = 250_000
    nb = -(-span // C["kBinWidth"])
    W, sm = C["kBinWindow"], C["kBinSmallMax"]
    # windows filled by the largest small tiles, by one-pair tiles, and runs of large tiles between
    pairs = [sm] * 50 + [1] * 3000 + [sm + 1] * 20 + [7, sm, 1, W - 1, W, W + 1] * 40
    bcs = {}
    for s, p in enumerate(pairs):
        if p > sm:
            v = np.zeros(nb, np.int64)
            v[0] = p  # every pair in one block: one dense job
            bcs[s] = v
    windows, jobs, _ = plan(pairs, bcs, span, sm)
    assert max(p for p, _ in windows) < W + sm
    assert max(t for _, t in windows) <= W // C["kBinPer"] + 1
    # sparse blocks exactly at the limits merge into runs that fit a table
    v = np.full(nb, C["kBinDenseMin"], np.int64)
    windows, jobs, _ = plan([int(v.sum())], {0: v}, span, sm)
    assert all(p <= C["kBinHashPairs"] for _, _, p in jobs)
