"""The header-only C++ drop-in (fastcc-benchmark_gb300/host/contract.hpp,
read.hpp): it compiles against the reference's call shape (CPU test), and a
program using it reproduces the oracle's contraction of .tns files (GPU test)."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from helpers import check_parity

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "fastcc-benchmark_gb300")
BUILD = os.path.join(ROOT, "tests", "_build")
DEMO = os.path.join(BUILD, "host_demo")


def build_demo():
    os.makedirs(BUILD, exist_ok=True)
    lib_dir = os.path.join(PKG, "_build")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(PKG, "host"), "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "host_demo", "demo.cpp"), "-L", lib_dir, "-lfastcc_gpu",
           f"-Wl,-rpath,{lib_dir}", "-o", DEMO]
    subprocess.check_call(cmd)
    return DEMO


def test_header_compiles_and_links():
    build_demo()
    assert os.path.exists(DEMO)


@pytest.mark.skipif(not oracle.reference_present(), reason="the reference's sources are not on this machine")
def test_reference_benchmark_compiles_unmodified_against_the_dropin(tmp_path):
    """The reference's own driver (benchmark.cpp: fastcc_multiply_timing and
    fastcc_multiply over TileAccumulator / TileAccumulatorMap) compiles and
    links against host/contract.hpp, read.hpp and libfastcc_gpu.so. The source
    is fed on standard input from an empty directory, so that its quoted
    includes resolve to the drop-in headers, not to the reference's."""
    src = os.path.join(oracle.reference_sources(), "benchmark.cpp")
    lib_dir = os.path.join(PKG, "_build")
    exe = tmp_path / "benchmark"
    with open(src) as f:
        subprocess.check_call(["g++", "-std=c++17", "-O1", "-x", "c++", "-I", os.path.join(PKG, "host"), "-I",
                               os.path.join(ROOT, "include"), "-", "-L", lib_dir, "-lfastcc_gpu",
                               f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], stdin=f, cwd=tmp_path)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 1 and "Usage" in out.stdout


@pytest.mark.gpu
def test_benchmark_cli_self_contraction_matches_oracle(tmp_path):
    """fcc_benchmark (host/fcc_benchmark.cpp, the reference driver's
    arguments and report) on a .tns self-contraction: every run reports the
    oracle's output count and the six medians are printed."""
    import build_lib
    cli = build_lib.build_cli()
    rng = np.random.Generator(np.random.PCG64(5))
    dims = [40, 12, 30]
    lin = rng.choice(int(np.prod(dims)), size=2000, replace=False)
    c = np.stack(np.unravel_index(lin, dims), axis=1).astype(np.int32)
    v = rng.uniform(-1, 1, 2000)
    _write_tns(tmp_path / "t.tns", c, v, dims)
    o = oracle.fastcc_multiply(c, v, oracle.infer_shape(c), c, v, oracle.infer_shape(c), [1, 2], [1, 2])
    for dense in ("0", "1"):
        out = subprocess.run([cli, str(tmp_path / "t.tns"), "1,2", "64", dense], capture_output=True, text=True,
                             timeout=300)
        assert out.returncode == 0, out.stderr
        runs = [l for l in out.stdout.splitlines() if l.startswith("run ")]
        assert len(runs) == 3 and all(l.endswith(f": {len(o['values'])} nonzeros") for l in runs), out.stdout
        assert out.stdout.count(f"Got {len(o['values'])} nonzeros") == 3
        for name in ("Index build", "Compute", "Drain", "Accumulate", "Indexing", "Total"):
            assert f"{name} time: " in out.stdout


def _write_tns(path, coords, vals, dims):
    with open(path, "w") as f:
        f.write(" ".join(str(d) for d in dims) + "\n")  # header line (skipped: has_header)
        for c, v in zip(coords, vals):
            f.write(" ".join(str(int(x)) for x in c) + " " + repr(float(v)) + "\n")


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["readme", "self3"])
def test_dropin_program_matches_oracle(tmp_path, case):
    build_demo()
    rng = np.random.Generator(np.random.PCG64(3 if case == "readme" else 4))
    if case == "readme":
        da, db, ca, cb = [20, 6, 18, 5], [25, 6, 5], [1, 3], [1, 2]
    else:
        da, db, ca, cb = [30, 12, 10], [30, 12, 10], [1, 2], [1, 2]

    def gen(dims, n):
        lin = rng.choice(int(np.prod(dims)), size=n, replace=False)
        return np.stack(np.unravel_index(lin, dims), axis=1).astype(np.int32), rng.uniform(-1, 1, n)

    ac, av = gen(da, 900)
    bc, bv = gen(db, 400) if case == "readme" else (ac, av)
    _write_tns(tmp_path / "a.tns", ac, av, da)
    _write_tns(tmp_path / "b.tns", bc, bv, db)
    out = tmp_path / "out.txt"
    subprocess.check_call([DEMO, str(tmp_path / "a.tns"), str(tmp_path / "b.tns"), ",".join(map(str, ca)),
                           ",".join(map(str, cb)), str(out)])
    lines = out.read_text().split("\n")
    n, order = map(int, lines[0].split())
    rows = [l.split() for l in lines[1:1 + n]]
    got_c = np.array([[int(x) for x in r[:order]] for r in rows], np.int64).reshape(n, order)
    got_v = np.array([float(r[order]) for r in rows])
    # the header's shape is the inferred max index (the file's rows, as _infer_shape)
    o = oracle.fastcc_multiply(ac, av, oracle.infer_shape(ac), bc, bv, oracle.infer_shape(bc), ca, cb,
                               want_abs=True)
    check_parity(got_c, got_v, o["coords"], o["values"], o["abs_sum"])
