#!/usr/bin/env python
"""Benchmark: FaSTCC sparse x sparse contraction on one GB300.

One step = one full contraction (index build, plan, tile contraction, output
compaction) of the Zipf 3-way self-contraction A(i,c0,c1) * A(j,c0,c1):
A 20,000 x 20,000 x 500,000 with 10M distinct nonzeros, every mode Zipf(1.2),
sign-random lognormal values, contracted over modes {1,2}.

  value  = FP64 multiply-adds per second, inputs resident on the device
  e2e    = the same through the C ABI (fcc_contract_into) with pinned host
           operands and the full output delivered to pinned host buffers
           inside the timed region (computed on the device, then copied once;
           waves_ms_per_step: the output copied in 12 waves while later waves
           compute)
  roofline: the tile contraction kernel (k_contract_dense); algorithmic bytes
           = inputs read once + outputs written once
  cpu_baseline: the CPU port of the reference's OpenMP fastcc_multiply
           (oracle/) on all host cores over the whole workload, timed inside
           the library (index build, tile loop, output concatenation)
  twomode, batched, readme: the other workloads, each with its own roofline
           and CPU baseline; batched also against 256 autotuned plain calls

--impl reference times that CPU implementation alone (all host threads), on
the whole workload every step; its inputs are generated in a child process so
that the reference arm loads no library of this package.
Multi-GPU runs (torchrun) are replicas: every rank contracts its own copy.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "fastcc-benchmark_gb300")
sys.path.insert(0, PKG)

METRIC = "FP64 multiply-adds/s & ms/contraction: learned+batched vs plain, 1 GB300"
UNIT = "multiply-adds/s"
def workload_name(nnz):
    n = f"{nnz // 1_000_000}M" if nnz % 1_000_000 == 0 else str(nnz)
    return (f"zipf3: A 20000x20000x500000, {n} nnz, Zipf(1.2) per mode, lognormal values; "
            f"A x A over modes {{1,2}}")
# dram__bytes_read.sum + dram__bytes_write.sum of one k_contract_dense launch:
# measured with ncu on the 2.5M-nonzero case of the same extents (0.142 GB read
# + 3.132 GB written for 3.381 GB of algorithmic bytes) and scaled by
# algorithmic bytes to this workload's 6.695 GB.
MEASURED_TRAFFIC = 6.695e9 * (0.1422 + 3.1322) / 3.381


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """Samples nvidia-smi every 200 ms while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        # nvidia-smi numbers GPUs its own way: name the timed device by UUID
        # (CUDA_VISIBLE_DEVICES may remap the index torch sees)
        self.index = str(index)
        try:
            import torch
            u = str(torch.cuda.get_device_properties(index).uuid)
            if u:
                self.index = u if u.startswith(("GPU-", "MIG-")) else "GPU-" + u
        except Exception:
            pass
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        def run():
            while not self._stop.is_set():
                try:
                    out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits"], capture_output=True,
                                         text=True, timeout=5).stdout.strip()
                    if out:
                        self.rows.append([x.strip() for x in out.split(",")])
                except Exception:
                    pass
                self._stop.wait(0.2)
        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for n, v in zip(names, r[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("FCC_BACKEND", "nccl") == "nccl" else "gloo")
    return ws, rank, local


def dist_max(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_port(a, b, ctr_a, ctr_b, nthreads=0):
    """One call of the CPU port of the reference's fastcc_multiply
    (oracle/fastcc_oracle.cpp, tile size 128 as benchmark.cpp:17) on all host
    threads. Returns (multiply-adds, outputs, seconds), seconds being the
    call's own time inside the library: index build, tile-pair loop with
    drain, concatenation of the thread outputs and their decode."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    o = oracle.fastcc_multiply(a.coords, a.values, a.max_index, b.coords, b.values, b.max_index, ctr_a, ctr_b,
                               tile_size=128, nthreads=nthreads or (os.cpu_count() or 1), keep=False)
    return o["products"], o["nnz"], o["total_ms"] / 1000.0


class _HostTensor:
    def __init__(self, coords, values, max_index):
        self.coords, self.values, self.max_index = coords, values, max_index

    @property
    def nnz(self):
        return int(self.values.shape[0])


def dump_inputs(path, nnz):
    """--dump-inputs: the benchmark operand, written for the reference arm."""
    import numpy as np
    import workloads
    w = workloads.zipf3(seed=1, nnz=nnz)
    a = w["a"]
    np.savez(path, coords=a.coords, values=a.values, max_index=a.max_index)


def run_reference(args, ws, rank):
    """--impl reference: the CPU port of the reference's fastcc_multiply
    (the reference's own sources do not exist on the GPU machine; the port's
    speed relative to them is measured where they do) on all host threads,
    the whole workload every step."""
    if rank != 0:
        return
    import tempfile

    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "zipf3.npz")
        subprocess.check_call([sys.executable, os.path.abspath(__file__), "--dump-inputs", path,
                               "--nnz", str(args.nnz)])
        d = np.load(path)
        a = _HostTensor(d["coords"], d["values"], d["max_index"])
    ncores = os.cpu_count() or 1
    prods, secs = [], []
    outs = 0
    for s in range(args.warmup + args.steps):
        p, outs, dt = cpu_port(a, a, [1, 2], [1, 2], ncores)
        if s >= args.warmup:
            prods.append(p)
            secs.append(dt)
    value = sum(prods) / sum(secs)
    sample = (f"the whole workload every step ({prods[0]} multiply-adds, {outs} outputs); time inside the "
              f"library: index build, tile loop, output concatenation and decode")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * sum(secs) / len(secs),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": workload_name(a.nnz), "nnz": a.nnz, "multiply_adds": prods[0], "outputs": outs,
                       "sample": "whole workload"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": ncores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_profile_case(name, extra=None):
    """A small case of the same kernels, sized for ncu: inputs above the L2
    size, a few GB on the device in all. Launch order: the warm-up
    contraction's kernels, then the timed one's."""
    import torch

    import build_lib
    build_lib.build_all()
    import fastcc_gpu as F
    import workloads
    if name == "zipf3-small":
        # same extents as the benchmark workload (same tile shape), a quarter of the nonzeros
        w = workloads.zipf3(seed=1, nnz=2_500_000)
    elif name == "twomode-small":
        w = workloads.twomode(seed=1, nnz=1_250_000, dims=(2_500, 2_500, 1_000, 50))
    else:
        w = workloads.readme(seed=1)
    a, b = w["a"], w["b"]
    A = F.Tensor(torch.from_numpy(a.coords).cuda(), torch.from_numpy(a.values).cuda(), a.max_index)
    B = A if b is a else F.Tensor(torch.from_numpy(b.coords).cuda(), torch.from_numpy(b.values).cuda(),
                                  b.max_index)
    torch.cuda.synchronize()
    with F.Context(0) as ctx:
        opts = F.Options(timing=1, **(extra or {}))
        for step in range(2):
            l0 = F.launch_count()
            r = ctx.contract(A, B, w["ctr_a"], w["ctr_b"], opts)
            print(json.dumps({"case": name, "step": step, "outputs": r.nnz, "multiply_adds": r.products,
                              "launches": F.launch_count() - l0,
                              "phases_ms": {k: round(v, 4) for k, v in ctx.timings().items()}}))
            r.free()


class _Dev:
    """A device pointer for torch.as_tensor (CUDA array interface)."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False),
                                         "version": 3, "strides": None}


def fingerprint(r):
    """Order-independent digest of a device result: (entries, sum of hashed
    coordinates mod 2^64, sum of values, sum of |values|)."""
    import torch
    cptr, stride, vptr = r.device_pointers()
    n = r.nnz
    if n == 0:
        return 0, 0, 0.0, 0.0
    v = torch.as_tensor(_Dev(vptr, n, "<f8"), device="cuda")
    h = torch.zeros(n, dtype=torch.int64, device="cuda")
    for m in range(r.order):
        c = torch.as_tensor(_Dev(cptr + 4 * m * stride, n, "<i4"), device="cuda").long()
        h = h * 1000003 + c + 1  # int64 arithmetic wraps: a hash mod 2^64
    return n, int(h.sum().item()), float(v.sum().item()), float(v.abs().sum().item())


def run_sched_eval(model_path, reps=3):
    """Held-out evaluation of the learned schedule: seeds the cost model was
    not trained on, shapes of the two-mode and batched workloads. Per case:
    the autotuner's best uniform schedule against FCC_SCHED_LEARNED (median
    total time over reps), with identical output digests required. Then the
    batched workload end to end: 256 plain contractions, each with its
    autotuned options, against one batched call with the learned schedule."""
    import numpy as np
    import torch

    import fastcc_gpu as F
    import workloads
    model = np.fromfile(model_path, np.float32)
    ctx = F.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    cuda = lambda t: F.Tensor(torch.from_numpy(t.coords).cuda(), torch.from_numpy(t.values).cuda(), t.max_index)

    def timed(call, opts):
        ts, fp = [], None
        for rep in range(reps + 1):
            r = call(opts)
            if rep == 0:
                fp = fingerprint(r)
            r.free()
            if rep:
                ts.append(ctx.timings()["total"])
        return statistics.median(ts), fp

    def same(fa, fb):
        return fa[0] == fb[0] and fa[1] == fb[1] and abs(fa[2] - fb[2]) <= 1e-9 * max(fa[3], 1e-300)

    cases = []
    for seed in (101, 102):
        w = workloads.twomode(seed=seed)
        A = cuda(w["a"])
        cases.append((f"twomode seed {seed}", lambda o, A=A, w=w: ctx.contract(A, A, w["ctr_a"], w["ctr_b"], o),
                      lambda base, A=A, w=w: ctx.autotune(A, A, w["ctr_a"], w["ctr_b"], base, reps)))
    inst = workloads.batched(seed=101, count=256)
    As = [cuda(x["a"]) for x in inst]
    Bs = [cuda(x["b"]) for x in inst]
    cases.append(("batched seed 101", lambda o: ctx.contract_batch(As, Bs, [1, 3], [1, 2], o)[0],
                  lambda base: ctx.autotune_batch(As, Bs, [1, 3], [1, 2], base, reps)))
    torch.cuda.synchronize()
    out = []
    for name, call, tune in cases:
        best, _ = tune(F.Options(timing=1))
        t_auto, fp_auto = timed(call, best)
        t_rule, fp_rule = timed(call, F.Options(timing=1))
        ctx.sched_set_model(model)
        t_learn, fp_learn = timed(call, F.Options(timing=1, schedule=F.SCHED_LEARNED))
        cls = np.bincount(ctx.sched_last_tiles(features=False, cost=False)["cls"], minlength=F.NUM_CLASSES)
        t_mix, fp_mix = timed(call, F.Options(timing=1, schedule=F.SCHED_LEARNED, sched_mix_margin=10))
        cls_mix = np.bincount(ctx.sched_last_tiles(features=False, cost=False)["cls"], minlength=F.NUM_CLASSES)
        ctx.sched_set_model(None)
        line = {"case": name, "autotuned": F.Context.options_dict(best), "autotuned_ms": t_auto, "rule_ms": t_rule,
                "learned_ms": t_learn, "learned_vs_autotuned": t_auto / t_learn,
                "learned_tiles_per_class": [int(c) for c in cls],
                "learned_margin10_ms": t_mix, "learned_margin10_tiles_per_class": [int(c) for c in cls_mix],
                "identical_output": same(fp_auto, fp_learn) and same(fp_auto, fp_rule) and same(fp_auto, fp_mix),
                "outputs": fp_auto[0]}
        print(json.dumps(line), flush=True)
        out.append(line)
    # batched + learned against 256 autotuned plain contractions
    plain_opts = []
    for a, b in zip(As, Bs):
        best, _ = ctx.autotune(a, b, [1, 3], [1, 2], F.Options(timing=1), 1)
        plain_opts.append(best)
    for a, b, o in zip(As, Bs, plain_opts):  # warm-up
        ctx.contract(a, b, [1, 3], [1, 2], o).free()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for a, b, o in zip(As, Bs, plain_opts):
        ctx.contract(a, b, [1, 3], [1, 2], o).free()
    e1.record(stream)
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1)
    ctx.sched_set_model(model)
    lo = F.Options(schedule=F.SCHED_LEARNED)
    ctx.contract_batch(As, Bs, [1, 3], [1, 2], lo)[0].free()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        ctx.contract_batch(As, Bs, [1, 3], [1, 2], lo)[0].free()
    e1.record(stream)
    torch.cuda.synchronize()
    batch_ms = e0.elapsed_time(e1) / reps
    line = {"case": "batched seed 101: 256 autotuned plain contractions vs one batched learned call",
            "plain_autotuned_ms_per_contraction": plain_ms / 256,
            "batched_learned_ms_per_contraction": batch_ms / 256, "speedup": plain_ms / batch_ms}
    print(json.dumps(line), flush=True)
    out.append(line)
    ctx.close()
    return out


def run_sweep_batched(variants, reps):
    """The batched workload: each option set timed on one fcc_contract_batch
    call (median of reps, per-phase times); the learned schedule uses the
    package's cost model."""
    import numpy as np
    import torch

    import fastcc_gpu as F
    import workloads
    inst = workloads.batched(seed=int(os.environ.get("FCC_SWEEP_BATCH_SEED", "1")), count=256)
    cuda = lambda t: F.Tensor(torch.from_numpy(t.coords).cuda(), torch.from_numpy(t.values).cuda(), t.max_index)
    As = [cuda(w["a"]) for w in inst]
    Bs = [cuda(w["b"]) for w in inst]
    torch.cuda.synchronize()
    with F.Context(0) as ctx:
        for v in variants:
            opts = F.Options(timing=1, **v)
            if opts.schedule == F.SCHED_LEARNED:
                ctx.load_default_model()
            ph = []
            clk = Clocks(0)
            for rep in range(reps + 1):
                if rep == 1:
                    clk.start()
                r, _ = ctx.contract_batch(As, Bs, [1, 3], [1, 2], opts)
                n = r.nnz
                r.free()
                if rep:
                    ph.append(ctx.timings())
            c = clk.stop()
            med = {k: statistics.median(p[k] for p in ph) for k in ph[0]}
            cls = np.bincount(ctx.sched_last_tiles(features=False, cost=False)["cls"], minlength=F.NUM_CLASSES)
            ctx.sched_set_model(None)
            print(json.dumps({"workload": "batched", "options": v, "outputs": n, "tiles_per_class": cls.tolist(),
                              "phases_ms": {k: round(x, 3) for k, x in med.items()}, "sm_mhz": c["sm_mhz"],
                              "reasons": c["reasons"]}), flush=True)


def run_sweep(name, variants, reps=10):
    """Times option sets on one workload (device-resident, median of reps),
    one JSON line per option set."""
    import torch

    import build_lib
    build_lib.build_all()
    import fastcc_gpu as F
    import workloads
    if name == "batched":
        run_sweep_batched(variants, reps)
        return
    w = {"zipf3": workloads.zipf3, "twomode": workloads.twomode, "readme": workloads.readme}[name]()
    a, b = w["a"], w["b"]
    A = F.Tensor(torch.from_numpy(a.coords).cuda(), torch.from_numpy(a.values).cuda(), a.max_index)
    B = A if b is a else F.Tensor(torch.from_numpy(b.coords).cuda(), torch.from_numpy(b.values).cuda(),
                                  b.max_index)
    torch.cuda.synchronize()
    with F.Context(0) as ctx:
        for v in variants:
            opts = F.Options(timing=1, **v)
            ph = []
            clk = Clocks(0)
            for rep in range(reps + 1):
                if rep == 1:
                    clk.start()
                r = ctx.contract(A, B, w["ctr_a"], w["ctr_b"], opts)
                t = ctx.timings()
                r.free()
                if rep:
                    ph.append(t)
            c = clk.stop()
            med = {k: round(statistics.median(p[k] for p in ph), 4) for k in ph[0]}
            print(json.dumps({"workload": name, "options": v, "total_ms": med["total"],
                              "contract_ms": med["contract"], "sm_mhz": c["sm_mhz"], "reasons": c["reasons"],
                              "phases_ms": med}), flush=True)


def hbm_roofline(alg_bytes, ms, what):
    """Achieved algorithmic bytes per second against the measured HBM peak."""
    peak, peak_kind = load_peaks()
    achieved = alg_bytes / (ms / 1000.0) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "algorithmic_bytes": alg_bytes, "ms": ms, "over": what, "peak_kind": peak_kind}


def coo_bytes(nnz, order):
    return nnz * (4 * order + 8)


def run_twomode(steps, stream, local, cpu=True):
    """The two-mode self-contraction (A 5000x5000x2000x50, 5M nnz, over {0,2}):
    GPU time per contraction with the default schedule, device-resident, next
    to the CPU port on all host cores over the same workload."""
    import torch

    import fastcc_gpu as F
    import workloads
    w = workloads.twomode(seed=1)
    a = w["a"]
    A = F.Tensor(torch.from_numpy(a.coords).cuda(), torch.from_numpy(a.values).cuda(), a.max_index)
    ctx = F.Context(local)
    ctx.set_stream(stream.cuda_stream)
    opts = F.Options(timing=1)
    for _ in range(3):
        ctx.contract(A, A, w["ctr_a"], w["ctr_b"], opts).free()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n = max(steps, 5)
    phases = []
    e0.record(stream)
    for _ in range(n):
        ctx.contract(A, A, w["ctr_a"], w["ctr_b"], opts).free()
        phases.append(ctx.timings())
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / n
    r = ctx.contract(A, A, w["ctr_a"], w["ctr_b"])
    prods, outs, order = r.products, r.nnz, r.order
    r.free()
    ctx.close()
    med = {k: round(statistics.median(p[k] for p in phases), 4) for k in phases[0]}
    alg = 2 * coo_bytes(a.nnz, a.order) + coo_bytes(outs, order)
    out = {"workload": w["name"], "multiply_adds": prods, "outputs": outs, "gpu_ms": ms,
           "multiply_adds_per_s": prods / (ms / 1000.0), "phases_ms": med,
           "roofline": hbm_roofline(alg, ms, "whole contraction (index, plan, expanded hash tiles: expanded, "
                                             "hub rows partitioned by key blocks, reduced in shared memory)")}
    if cpu:
        p, _, dt = cpu_port(a, a, w["ctr_a"], w["ctr_b"])
        out["cpu_baseline"] = {"value": p / dt, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                               "sample": f"the whole workload ({p} multiply-adds, {dt:.2f} s inside the library)"}
        out["gpu_vs_cpu"] = (prods / (ms / 1000.0)) / (p / dt)
    return out


def run_readme(steps, stream, local, cpu=True):
    """The README contraction (256x64x256x64, 200k nnz, x 512x64x64, 100k
    nnz over {1,3} x {1,2}): GPU ms per contraction (device-resident and end to
    end through the C ABI) next to the CPU port on all host cores."""
    import torch

    import fastcc_gpu as F
    import workloads
    w = workloads.readme(seed=1)
    a, b = w["a"], w["b"]
    cuda = lambda t: F.Tensor(torch.from_numpy(t.coords).cuda(), torch.from_numpy(t.values).cuda(), t.max_index)
    A, B = cuda(a), cuda(b)
    ctx = F.Context(local)
    ctx.set_stream(stream.cuda_stream)

    def timed(x, y, n):
        for _ in range(3):
            ctx.contract(x, y, w["ctr_a"], w["ctr_b"]).free()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            r = ctx.contract(x, y, w["ctr_a"], w["ctr_b"])
            if x is not A:
                r.to_numpy()
            r.free()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    ms = timed(A, B, max(steps, 10))
    ms_e2e = timed(a, b, 3)
    r = ctx.contract(A, B, w["ctr_a"], w["ctr_b"])
    prods, outs, order = r.products, r.nnz, r.order
    r.free()
    ctx.close()
    alg = coo_bytes(a.nnz, a.order) + coo_bytes(b.nnz, b.order) + coo_bytes(outs, order)
    out = {"workload": w["name"], "multiply_adds": prods, "outputs": outs, "gpu_ms": ms, "gpu_e2e_ms": ms_e2e,
           "roofline": hbm_roofline(alg, ms, "whole contraction")}
    if cpu:
        cpu_s = sorted(cpu_port(a, b, w["ctr_a"], w["ctr_b"])[2] for _ in range(5))[2]
        out.update({"cpu_ms": 1000 * cpu_s, "cpu_threads": os.cpu_count() or 1, "cpu_kind": "port",
                    "gpu_vs_cpu": 1000 * cpu_s / ms, "gpu_e2e_vs_cpu": 1000 * cpu_s / ms_e2e})
    return out


def run_batched(steps, warmup, stream, local, cpu=True):
    """The batched workload: 256 contractions of the readme pattern with
    uneven sizes. Times, per step, 256 sequential plain contractions (default
    options, and each with its autotuned options, tuned before timing), one
    batched call (fcc_contract_batch) with the rule schedule and with the
    learned schedule, on device-resident operands; then plain and batched end
    to end (pinned host operands in, every output copied back). Returns the
    JSON sub-object."""
    import torch

    import fastcc_gpu as F
    import workloads
    inst = workloads.batched(seed=1, count=256)
    dev = [(F.Tensor(torch.from_numpy(w["a"].coords).cuda(), torch.from_numpy(w["a"].values).cuda(),
                     w["a"].max_index),
            F.Tensor(torch.from_numpy(w["b"].coords).cuda(), torch.from_numpy(w["b"].values).cuda(),
                     w["b"].max_index)) for w in inst]
    As, Bs = [d[0] for d in dev], [d[1] for d in dev]
    ctr_a, ctr_b = inst[0]["ctr_a"], inst[0]["ctr_b"]
    torch.cuda.synchronize()
    ctx = F.Context(local)
    ctx.set_stream(stream.cuda_stream)

    def plain(opts_list=None):
        n = p = 0
        for i, (a, b) in enumerate(dev):
            r = ctx.contract(a, b, ctr_a, ctr_b, opts_list[i] if opts_list else None)
            n += r.nnz
            p += r.products
            r.free()
        return n, p

    def batched(opts=None):
        r, counts = ctx.contract_batch(As, Bs, ctr_a, ctr_b, opts)
        n, p = r.nnz, r.products
        r.free()
        return n, p

    def timed(fn, steps=steps):
        for _ in range(warmup):
            out = fn()
        torch.cuda.synchronize()
        l0 = F.launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps, out, (F.launch_count() - l0) // steps

    ms_plain, (n_plain, prods), l_plain = timed(plain)
    ms_batch, (n_batch, prods_b), l_batch = timed(batched)
    assert n_plain == n_batch and prods == prods_b, "batched and plain results differ in size"
    # every instance autotuned (fcc_autotune, cached per shape signature) before the timed region
    tuned = [ctx.autotune(a, b, ctr_a, ctr_b, F.Options(), 1)[0] for a, b in dev]
    ms_tuned, (n_t, _), _ = timed(lambda: plain(tuned))
    assert n_t == n_batch, "autotuned plain calls changed the output size"
    ms_learned = None
    if ctx.load_default_model():
        ms_learned, (n_l, _), _ = timed(lambda: batched(F.Options(schedule=F.SCHED_LEARNED)))
        assert n_l == n_batch, "learned schedule changed the output size"
        ctx.sched_set_model(None)

    # end to end: pinned host operands, outputs copied to pinned host buffers
    host = []
    for w in inst:
        pa = (torch.from_numpy(w["a"].coords).pin_memory(), torch.from_numpy(w["a"].values).pin_memory())
        pb = (torch.from_numpy(w["b"].coords).pin_memory(), torch.from_numpy(w["b"].values).pin_memory())
        host.append((F.Tensor(pa[0].numpy(), pa[1].numpy(), w["a"].max_index),
                     F.Tensor(pb[0].numpy(), pb[1].numpy(), w["b"].max_index), pa, pb))
    HA, HB = [h[0] for h in host], [h[1] for h in host]
    order = 4  # the instance, then i, j, k
    out_c = torch.empty((order, n_batch), dtype=torch.int32).pin_memory()
    out_v = torch.empty(n_batch, dtype=torch.float64).pin_memory()
    oc, ov = out_c.numpy(), out_v.numpy()

    def plain_e2e():
        off = 0
        for a, b, _, _ in host:
            r = ctx.contract(a, b, ctr_a, ctr_b)
            r.to_numpy_soa(oc[1:, off:], ov[off:])
            off += r.nnz
            r.free()
        return off, 0

    def batched_e2e():
        r, counts = ctx.contract_batch(HA, HB, ctr_a, ctr_b)
        r.to_numpy_soa(oc, ov)
        n = r.nnz
        r.free()
        return n, 0

    e2e_steps = max(1, min(steps, 3))
    ms_plain_e2e, _, _ = timed(plain_e2e, e2e_steps)
    ms_batch_e2e, _, _ = timed(batched_e2e, e2e_steps)
    in_bytes = sum(h[2][0].numel() * 4 + h[2][1].numel() * 8 + h[3][0].numel() * 4 + h[3][1].numel() * 8
                   for h in host)
    ctx.close()
    count = len(inst)
    alg = sum(coo_bytes(w["a"].nnz, w["a"].order) + coo_bytes(w["b"].nnz, w["b"].order) for w in inst) + \
        coo_bytes(n_batch, order)
    out = {
        "workload": "256 contractions a(i,c0,j,c1) x b(k,c0,c1), nnz(a) log-uniform [1e3, 2e6], "
                    "nnz(b) = nnz(a)/2, extents uniform [32, 1024], Zipf s uniform [1.0, 1.5]",
        "contractions": count, "multiply_adds": prods, "outputs": n_batch,
        "plain": {"ms_per_contraction": ms_plain / count, "multiply_adds_per_s": prods / (ms_plain / 1000.0),
                  "launches_per_step": l_plain,
                  "e2e_ms_per_contraction": ms_plain_e2e / count},
        "plain_autotuned": {"ms_per_contraction": ms_tuned / count,
                            "multiply_adds_per_s": prods / (ms_tuned / 1000.0),
                            "options": "fcc_autotune per instance (cached per shape signature), tuned before "
                                       "the timed region"},
        "batched": {"ms_per_contraction": ms_batch / count, "multiply_adds_per_s": prods / (ms_batch / 1000.0),
                    "launches_per_step": l_batch,
                    "e2e_ms_per_contraction": ms_batch_e2e / count},
        "batched_learned": None if ms_learned is None else {
            "ms_per_contraction": ms_learned / count, "multiply_adds_per_s": prods / (ms_learned / 1000.0),
            "speedup_vs_plain": ms_plain / ms_learned, "speedup_vs_plain_autotuned": ms_tuned / ms_learned},
        "speedup": ms_plain / ms_batch, "speedup_vs_plain_autotuned": ms_tuned / ms_batch,
        "e2e_speedup": ms_plain_e2e / ms_batch_e2e,
        "e2e_h2d_bytes_per_step": in_bytes,
        "e2e_d2h_bytes_per_step": {"plain": n_batch * ((order - 1) * 4 + 8), "batched": n_batch * (order * 4 + 8)},
        "roofline": hbm_roofline(alg, ms_batch, "one batched call (index, plan, tile kernels)"),
        "steps": steps, "e2e_steps": e2e_steps, "warmup": warmup,
    }
    if cpu:
        p = dt = 0
        for w in inst:
            pi, _, di = cpu_port(w["a"], w["b"], ctr_a, ctr_b)
            p += pi
            dt += di
        out["cpu_baseline"] = {"value": p / dt, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                               "sample": f"all 256 instances, one call each ({p} multiply-adds, {dt:.2f} s "
                                         f"inside the library)"}
        out["gpu_vs_cpu"] = (prods / (ms_batch / 1000.0)) / (p / dt)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nnz", type=int, default=10_000_000,
                    help="nonzeros of the benchmark operand (10M: the benchmark workload; smaller for tests)")
    ap.add_argument("--dump-inputs", metavar="PATH", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--profile", choices=["zipf3-small", "twomode-small", "readme"],
                    help="one warm-up and one timed contraction of a small case, for ncu captures")
    ap.add_argument("--sweep", choices=["zipf3", "twomode", "readme", "batched"],
                    help="time the option sets given by --variants (JSON list) on a workload")
    ap.add_argument("--variants", default="[{}]")
    ap.add_argument("--sched-eval", metavar="MODEL", default=None,
                    help="held-out evaluation of a cost model file against the autotuner")
    ap.add_argument("--batched", action="store_true",
                    help="print only the batched comparison (256 plain contractions vs one batched call)")
    ap.add_argument("--no-batched", action="store_true", help="leave the batched comparison out")
    ap.add_argument("--diag", action="store_true",
                    help="print the FP64 FMA rate and the shared-memory accumulation rates")
    ap.add_argument("--sort", nargs=2, type=int, metavar=("N", "BITS"), default=None,
                    help="time the library's radix sort on N seeded uniform keys of BITS bits "
                         "(32-bit payloads; 32-bit keys with 64-bit payloads when BITS <= 32 and N < 0)")
    args = ap.parse_args()
    if args.dump_inputs:
        import build_lib
        build_lib.build_synth()
        dump_inputs(args.dump_inputs, args.nnz)
        return
    if args.sort:
        import numpy as np
        import build_lib
        build_lib.build_all()
        import fastcc_gpu as F
        n, bits = args.sort
        rng = np.random.Generator(np.random.PCG64(1))
        k32 = n < 0
        n = abs(n)
        keys = rng.integers(0, 1 << bits, n, dtype=np.uint64)
        vals = np.arange(n, dtype=np.uint64 if k32 else np.uint32)
        if k32:
            keys = keys.astype(np.uint32)
        ko, vo, ms = F.radix_sort(keys, vals, bits, reps=3)
        order = np.argsort(keys, kind="stable")
        ok = bool(np.array_equal(ko, keys[order]) and np.array_equal(vo, vals[order]))
        kb, vb = keys.dtype.itemsize, vals.dtype.itemsize
        passes = (bits + 7) // 8
        alg = passes * n * (kb + 2 * (kb + vb))  # per pass: histogram read, scatter read + write
        print(json.dumps({"sort_keys": n, "bits": bits, "key_bytes": kb, "value_bytes": vb, "passes": passes,
                          "ms": ms, "algorithmic_GBps": alg / ms / 1e6, "matches_numpy_stable_sort": ok}))
        if not ok:
            sys.exit(1)
        return
    if args.diag:
        import build_lib
        build_lib.build_all()
        import fastcc_gpu as F
        import torch
        torch.cuda.set_device(0)
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        clk = 2.07e9
        line = {"fp64_fma_per_s": F.fp64_fma_rate(0)}
        for mode, name in enumerate(["atomicAdd_product", "cas_fma", "plain_fma"]):
            r = F.shared_update_rate(mode)
            line[f"shared_{name}_per_s"] = r
            line[f"shared_{name}_per_clk_per_sm"] = r / sms / clk
        line["fp64_fma_per_clk_per_sm"] = line["fp64_fma_per_s"] / sms / clk
        print(json.dumps(line))
        return
    if args.sweep:
        run_sweep(args.sweep, json.loads(args.variants))
        return
    if args.sched_eval:
        import build_lib
        build_lib.build_all()
        run_sched_eval(args.sched_eval)
        return
    args.warmup = max(args.warmup, 3)
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    if args.profile:
        run_profile_case(args.profile, json.loads(args.variants)[0])
        return
    if args.batched:
        import torch

        import build_lib
        build_lib.build_all()
        torch.cuda.set_device(local)
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        out = run_batched(args.steps, args.warmup, stream, local)
        if rank == 0:
            print(json.dumps(out))
        return

    import numpy as np
    import torch

    import build_lib
    build_lib.build_all()
    import fastcc_gpu as F
    import workloads

    torch.cuda.set_device(local)
    w = workloads.zipf3(seed=1, nnz=args.nnz)
    a = w["a"]
    nnz = a.nnz
    dev_c = torch.from_numpy(a.coords).cuda()
    dev_v = torch.from_numpy(a.values).cuda()
    A = F.Tensor(dev_c, dev_v, a.max_index)
    torch.cuda.synchronize()
    ctx = F.Context(local)
    # a dedicated (non-default) stream: the library and the timing events share it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    opts = F.Options(timing=1)

    res = None
    for _ in range(args.warmup):
        r = ctx.contract(A, A, w["ctr_a"], w["ctr_b"], opts)
        res = (r.nnz, r.products, r.order)
        r.free()
    out_nnz, products, out_order = res

    clocks = Clocks(local)
    barrier(ws)
    torch.cuda.synchronize()
    clocks.start()
    l0 = F.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    contract_ms = []
    ev0.record(stream)
    for _ in range(args.steps):
        r = ctx.contract(A, A, w["ctr_a"], w["ctr_b"], opts)
        contract_ms.append(ctx.timings()["contract"])
        r.free()
    ev1.record(stream)
    torch.cuda.synchronize()
    launches = F.launch_count() - l0
    barrier(ws)
    clk = clocks.stop()
    ms = dist_max(ev0.elapsed_time(ev1) / args.steps, ws)
    phases = ctx.timings()
    value = products * ws / (ms / 1000.0)

    # ---- end to end through the C ABI with pinned host buffers ----
    pin_c = torch.from_numpy(a.coords).pin_memory()
    pin_v = torch.from_numpy(a.values).pin_memory()
    H = F.Tensor(pin_c.numpy(), pin_v.numpy(), a.max_index)
    out_c = torch.empty((out_order, out_nnz), dtype=torch.int32).pin_memory()
    out_v = torch.empty(out_nnz, dtype=torch.float64).pin_memory()
    oc, ov = out_c.numpy(), out_v.numpy()

    def e2e_into(waves):  # fcc_contract_into: pinned host operands in, pinned host output
        def call():
            n, _ = ctx.contract_into(H, H, w["ctr_a"], w["ctr_b"], oc, ov, F.Options(timing=1, out_waves=waves))
            assert n == out_nnz
        return call

    def e2e_time(fn):
        fn()  # warm-up; with out_waves 0 the first two large calls of a context measure its copy paths
        fn()
        barrier(ws)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.e2e_steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return dist_max(e0.elapsed_time(e1) / args.e2e_steps, ws)

    e2e_ms = e2e_time(e2e_into(0))
    e2e_phases = ctx.timings()
    e2e_waves_ms = e2e_time(e2e_into(12))
    h2d = 2 * (pin_c.numel() * 4 + pin_v.numel() * 8)
    d2h = out_nnz * (4 * out_order + 8)

    peak, peak_kind = load_peaks()
    alg_bytes = 2 * nnz * (4 * 3 + 8) + out_nnz * (4 * out_order + 8)
    kms = statistics.mean(contract_ms)
    achieved = alg_bytes / (kms / 1000.0) / 1e9
    fma_peak = F.fp64_fma_rate(local)  # measured now, on this GPU
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(nnz), "nnz": nnz, "multiply_adds": products, "outputs": out_nnz,
                   "l2": "inputs 200 MB and outputs 6.4 GB exceed the 129 MB L2; no flush",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": MEASURED_TRAFFIC * alg_bytes / 6.695e9,
                     "kernel": "k_contract_dense", "kernel_ms": kms, "algorithmic_bytes": alg_bytes,
                     "peak_kind": peak_kind,
                     "fp64": {"achieved": products / (kms / 1000.0), "peak": fma_peak, "unit": "FMA/s",
                              "frac": products / (kms / 1000.0) / fma_peak,
                              "note": "every multiply-add is one FP64 FMA; peak measured by fcc_diag_fp64_fma_rate"}},
        "e2e": {"value": products * ws / (e2e_ms / 1000.0), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
                "path": "fcc_contract_into (out_waves 0): pinned host operands in, output computed in device "
                        "memory and copied to pinned host buffers, once afterwards or in 12 waves overlapping the "
                        "contraction, whichever the context measured faster on its first two such calls (warm-up)",
                "waves_ms_per_step": e2e_waves_ms,
                "phases_ms": {k: round(v, 4) for k, v in e2e_phases.items()}},
        "gpu_launches": launches,
        "clocks": clk,
        "phases_ms": {k: round(v, 4) for k, v in phases.items()},
    }
    cpu = rank == 0 and ws == 1 and not args.no_cpu_baseline
    if not args.no_batched:
        line["batched"] = run_batched(min(args.steps, 5), 3, stream, local, cpu)
        line["readme"] = run_readme(args.steps, stream, local, cpu)
        line["twomode"] = run_twomode(args.steps, stream, local, cpu)
    if cpu:
        p, _, dt = cpu_port(a, a, w["ctr_a"], w["ctr_b"])
        line["cpu_baseline"] = {"value": p / dt, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                                "sample": f"the whole workload ({p} multiply-adds, {dt:.1f} s inside the library: "
                                          f"index build, tile loop, output concatenation and decode)"}
    ctx.close()
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
