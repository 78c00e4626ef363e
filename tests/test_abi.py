"""CPU checks of the C ABI library: it loads, exports every entry point that
include/*.h declares, and reports errors by status without a GPU."""
import ctypes
import os
import re
import subprocess

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
    assert L.fcc_abi_version() == 3
    assert L.fcc_status_string(0) == b"ok"
    assert L.fcc_status_string(3) == b"hash accumulator full"
    o = F.Options()
    assert L.fcc_options_default(ctypes.byref(o)) == 0 and o.tile_size == 100
    assert ctypes.sizeof(F.Options) == 88


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
