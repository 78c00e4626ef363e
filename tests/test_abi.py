"""CPU checks of the C ABI library: it loads, exports every entry point that
include/*.h declares, and reports errors by status without a GPU."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import fastcc_gpu as F

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fcc_[a-z0-9_]+)\s*\(", txt)))


def exported(lib):
    out = subprocess.check_output(["nm", "-D", "--defined-only", lib], text=True)
    return {l.split()[-1] for l in out.splitlines() if l.strip()}


def test_gpu_library_exports_every_declared_symbol():
    names = declared("fastcc_gpu.h")
    assert "fcc_contract" in names and len(names) >= 14
    missing = set(names) - exported(F.GPU_LIB)
    assert not missing, missing


def test_synth_library_exports_every_declared_symbol():
    missing = set(declared("fastcc_synth.h")) - exported(F.SYNTH_LIB)
    assert not missing, missing


def test_library_loads_and_reports_status_strings():
    L = F.lib()
    assert L.fcc_abi_version() == 5
    assert L.fcc_status_string(0) == b"ok"
    assert L.fcc_status_string(3) == b"hash accumulator full"
    o = F.Options()
    assert L.fcc_options_default(ctypes.byref(o)) == 0 and o.tile_size == 100
    assert ctypes.sizeof(F.Options) == 104


def test_bad_arguments_return_status_not_crash():
    L = F.lib()
    assert L.fcc_contract(None, None, None, None, None, 0, None, None) == 1
    assert L.fcc_result_info(None, None, None, None) == 1
    assert L.fcc_ctx_destroy(None) == 1


def test_no_device_is_a_status(tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = F.lib().fcc_ctx_create(0, ctypes.byref(h))
    assert rc == 7 and not h.value


def _c_struct_fields(header, name):
    """(type, field) pairs of `typedef struct ... { ... } name;` in a header."""
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    m = re.search(r"typedef struct \w*\s*\{([^{}]*)\}\s*" + name + r"\s*;", txt)
    assert m, name
    return re.findall(r"\b(int32_t|int64_t|uint32_t|uint64_t|double|float)\s+(\w+)\s*;", m.group(1))


def test_python_options_mirror_the_c_layout():
    # same field names, order and widths as fcc_options in the header, so the
    # binding cannot drift from the ABI
    c = _c_struct_fields("fastcc_gpu.h", "fcc_options")
    width = {"int32_t": 4, "uint32_t": 4, "int64_t": 8, "uint64_t": 8, "double": 8, "float": 4}
    py = [(name, ctypes.sizeof(t)) for name, t in F.Options._fields_]
    assert [n for _, n in c] == [n for n, _ in py]
    assert [width[t] for t, _ in c] == [w for _, w in py]
    for (t, name), (pname, _) in zip(c, py):
        assert getattr(F.Options, pname).offset % width[t] == 0


def test_shipped_cost_model_matches_the_header_layout():
    # FCC_SCHED_MODEL_FLOATS as the header computes it, the Python constant and
    # the shipped model file agree (a model trained for another output count
    # would be rejected at fcc_sched_set_model)
    txt = open(os.path.join(ROOT, "include", "fastcc_gpu.h")).read()
    m = re.search(r"#define FCC_SCHED_MODEL_FLOATS \(([^)]*)\)", txt)
    assert m
    n = eval(m.group(1), {})  # integer arithmetic only
    assert n == F.SCHED_MODEL_FLOATS
    k = int(re.search(r"FCC_NUM_CLASSES = (\d+)", txt).group(1))
    assert k == F.NUM_CLASSES and n == 2 * 12 + 12 * 64 + 64 + 64 * 64 + 64 + 64 * k + k
    path = os.path.join(ROOT, "fastcc-benchmark_gb300", "sched_model.f32")
    model = np.fromfile(path, np.float32)
    assert model.size == n and np.all(np.isfinite(model))
