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
