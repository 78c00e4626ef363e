"""Trains the tile-schedule cost model (FCC_SCHED_LEARNED) on timings the GPU
contraction produces itself.

For each training contraction (seeded synthetic tensors drawn like the
benchmark workloads, at reduced sizes) every enabled tile class is forced in
turn with opts.timing = 2. The tile structure does not depend on the class,
so the runs give, for each tile, its features and its measured cost in every
class: one record (x = 12 features, y = log2 cost per class, m = 1 where the
class ran the tile). The MLP (12 -> 64 -> 64 -> 5) is trained with the
library's own FP32 kernels (fcc_mlp_train) and written as a flat float32
file of FCC_SCHED_MODEL_FLOATS values.

Usage: python sched_train.py --out sched_model.f32 [--records N] [--epochs E]
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import fastcc_gpu as F  # noqa: E402
import workloads  # noqa: E402

MODEL_FILE = os.path.join(HERE, "sched_model.f32")


def training_set(seed):
    """Contractions drawn like the benchmark workloads at reduced sizes:
    (name, [(a, b)], ctr_a, ctr_b, batched)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for k in range(3):
        s = int(rng.integers(1, 1 << 30))
        nnz = int(rng.choice([1_000_000, 2_000_000, 3_000_000]))
        d = int(rng.choice([5_000, 10_000, 20_000]))
        w = workloads.zipf3(seed=s, nnz=nnz, dims=(d, d, 25 * d))
        out.append((f"zipf3-like {nnz} d{d}", [(w["a"], w["b"])], w["ctr_a"], w["ctr_b"], False))
    for k in range(4):
        s = int(rng.integers(1, 1 << 30))
        nnz = [1_000_000, 2_000_000, 5_000_000, 5_000_000][k]
        d = [2_000, 3_500, 5_000, 5_000][k]
        w = workloads.twomode(seed=s, nnz=nnz, dims=(d, d, int(0.4 * d), 50))
        out.append((f"twomode-like {nnz} d{d}", [(w["a"], w["b"])], w["ctr_a"], w["ctr_b"], False))
    for k in range(2):
        s = int(rng.integers(1, 1 << 30))
        inst = workloads.batched(seed=s, count=48, nnz_hi=1e6)
        out.append((f"batched-like 48 seed {s}", [(w["a"], w["b"]) for w in inst], [1, 3], [1, 2], True))
    return out


def run(ctx, pairs, ctr_a, ctr_b, batched, opts):
    if batched:
        r, _ = ctx.contract_batch([p[0] for p in pairs], [p[1] for p in pairs], ctr_a, ctr_b, opts)
    else:
        r = ctx.contract(pairs[0][0], pairs[0][1], ctr_a, ctr_b, opts)
    n = r.nnz
    r.free()
    return n


def record(ctx, pairs, ctr_a, ctr_b, batched, reps=2):
    """Per-tile features and cost (ns) in every class that can run the tiles.

    A tile's raw cost is the SM cycles of its work items over the CTAs per SM
    of its class. Raw costs are calibrated per run: scaled so that the tiles'
    costs add up to the run's measured contract + merge time, which folds in
    what per-item cycles miss (CTAs sharing an SM, launch tails, the merge of
    split tiles)."""
    feats, costs, mask = None, None, None
    for c in range(F.NUM_CLASSES):
        # the learned schedule's dense class runs two-phase items (dense_kernel 1)
        opts = F.Options(timing=2, schedule=F.SCHED_FORCE + c, dense_kernel=1)
        acc = None
        try:
            for _ in range(reps):
                run(ctx, pairs, ctr_a, ctr_b, batched, opts)
                t = ctx.sched_last_tiles()
                ph = ctx.timings()
                ms = ph["contract"] + ph["merge"]
                cal = t["cost"] * (ms * 1e6 / max(t["cost"].sum(), 1e-30))
                acc = cal if acc is None else acc + cal
        except F.FccError:
            continue  # class not available for this contraction (dense too wide, or out of memory)
        if feats is None:
            feats = t["features"]
            costs = np.zeros((feats.shape[0], F.NUM_CLASSES), np.float64)
            mask = np.zeros((feats.shape[0], F.NUM_CLASSES), np.float32)
        costs[:, c] = acc / reps
        mask[:, c] = 1.0
    return feats, costs, mask


def init_model(X, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    nf, nh, no = F.SCHED_FEATURES, F.SCHED_HIDDEN, F.NUM_CLASSES
    mean = X.mean(axis=0)
    std = X.std(axis=0)
    scale = np.where(std > 1e-6, 1.0 / np.maximum(std, 1e-6), 0.0)
    parts = [mean, scale,
             rng.normal(0, np.sqrt(2.0 / nf), (nf, nh)), np.zeros(nh),
             rng.normal(0, np.sqrt(2.0 / nh), (nh, nh)), np.zeros(nh),
             rng.normal(0, np.sqrt(1.0 / nh), (nh, no)), np.zeros(no)]
    m = np.concatenate([np.asarray(p, np.float64).ravel() for p in parts]).astype(np.float32)
    assert m.size == F.SCHED_MODEL_FLOATS
    return m


def regrets(pred, costs, mask):
    """Over the tiles where every hash class was measured: the measured cost
    of the classes the model picks, and of each single class run on every
    tile, relative to the per-tile best."""
    hash_cls = [F.CLASS_HASH_L, F.CLASS_HASH_M, F.CLASS_HASH_S]
    sel = mask[:, hash_cls].sum(axis=1) == len(hash_cls)
    p = np.where(mask > 0, pred, np.inf)[sel]
    c = np.where(mask > 0, costs, np.inf)[sel]
    best = c.min(axis=1).sum()
    learned = float(c[np.arange(len(c)), p.argmin(axis=1)].sum() / best)
    uniform = {int(k): float(c[:, k].sum() / best) for k in range(c.shape[1]) if np.isfinite(c[:, k]).all()}
    return learned, uniform


def dense_regrets(pred, costs, mask):
    """Over the tiles where both dense classes were measured: the measured
    cost of the model's pick between them, and of each alone, relative to the
    per-tile best of the two."""
    d = [F.CLASS_DENSE, F.CLASS_DENSE_FLAT]
    sel = mask[:, d].sum(axis=1) == len(d)
    if not sel.any():
        return None
    p, c = pred[sel][:, d], costs[sel][:, d]
    best = c.min(axis=1).sum()
    return {"learned": float(c[np.arange(len(c)), p.argmin(axis=1)].sum() / best),
            "two_phase": float(c[:, 0].sum() / best), "flat": float(c[:, 1].sum() / best), "tiles": int(sel.sum())}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=MODEL_FILE)
    ap.add_argument("--records", type=int, default=60_000, help="tiles sampled over all training contractions")
    ap.add_argument("--epochs", type=int, default=300)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--summary", default=None, help="write a JSON summary here")
    args = ap.parse_args()
    rng = np.random.Generator(np.random.PCG64(args.seed))
    ctx = F.Context(0)
    t0 = time.time()
    Xs, Ys, Ms, names = [], [], [], []
    sets = training_set(args.seed)
    per = args.records // len(sets)
    for name, pairs, ca, cb, batched in sets:
        X, C, Mk = record(ctx, pairs, ca, cb, batched)
        if X is None:
            continue
        take = rng.permutation(X.shape[0])[:per]
        Xs.append(X[take])
        Ys.append(np.log2(np.maximum(C[take], 1e-3)))
        Ms.append(Mk[take])
        names.append((name, int(X.shape[0]), int(len(take))))
        print(json.dumps({"contraction": name, "tiles": int(X.shape[0]), "sampled": int(len(take)),
                          "classes": [int(v) for v in Mk[0]]}), flush=True)
    X = np.concatenate(Xs).astype(np.float32)
    Y = np.concatenate(Ys).astype(np.float32)
    M = np.concatenate(Ms).astype(np.float32)
    perm = rng.permutation(X.shape[0])
    nval = X.shape[0] // 10
    val, tr = perm[:nval], perm[nval:]
    model = init_model(X[tr], args.seed)
    _, loss0 = ctx.mlp_grad(X[tr], Y[tr], M[tr], model)
    t1 = time.time()
    model, loss = ctx.mlp_train(X[tr], Y[tr], M[tr], model, epochs=args.epochs, batch=4096, lr=2e-3, seed=args.seed)
    t2 = time.time()
    _, vloss = ctx.mlp_grad(X[val], Y[val], M[val], model)
    pv = ctx.mlp_predict(X[val], model)
    C = np.exp2(Y[val].astype(np.float64))
    summary = {"records": int(X.shape[0]), "train": int(len(tr)), "val": int(len(val)),
               "loss_init": loss0, "loss_train": loss, "loss_val": vloss,
               "val_cost_vs_per_tile_best": {"learned": regrets(pv, C, M[val])[0],
                                              "single_class": regrets(pv, C, M[val])[1],
                                              "dense_classes": dense_regrets(pv, C, M[val])},
               "record_s": t1 - t0, "train_s": t2 - t1, "contractions": names}
    model.astype(np.float32).tofile(args.out)
    print(json.dumps(summary), flush=True)
    if args.summary:
        with open(args.summary, "w") as f:
            json.dump(summary, f, indent=1)
    ctx.close()


if __name__ == "__main__":
    main()
