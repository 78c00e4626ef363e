"""Builds the in-tree shared libraries of the package.

* ``_build/libfastcc_gpu.so``: the CUDA kernels and the C ABI
  (include/fastcc_gpu.h), compiled for sm_103a only.
* ``_build/libfastcc_synth.so``: the seeded synthetic-tensor generator
  (include/fastcc_synth.h), host code.
* ``_build/fcc_benchmark``: the command-line benchmark (host/fcc_benchmark.cpp,
  the reference's benchmark driver's arguments and report) over the drop-in
  header, linked against libfastcc_gpu.so.

Translation units compile in parallel; a library is rebuilt only when a source
is newer than it.
"""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")

GPU_LIB = os.path.join(BUILD, "libfastcc_gpu.so")
SYNTH_LIB = os.path.join(BUILD, "libfastcc_synth.so")
CLI = os.path.join(BUILD, "fcc_benchmark")
HOST = os.path.join(HERE, "host")

CU_SOURCES = ["fcc_prims.cu", "fcc_contract.cu", "fcc_api.cu", "fcc_noalloc.cu", "fcc_diag.cu", "fcc_batch.cu", "fcc_sched.cu"]
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _deps():
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hdrs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hdrs


def build_gpu(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(CSRC, f) for f in CU_SOURCES]
    if not force and not _stale(GPU_LIB, srcs + _deps() + [__file__]):
        return GPU_LIB
    nvcc = _nvcc()
    flags = GENCODE + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE]

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        cmd = [nvcc] + flags + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = GPU_LIB + ".tmp"
    subprocess.check_call([nvcc] + GENCODE + ["-shared", "-o", tmp] + objs)
    os.replace(tmp, GPU_LIB)
    return GPU_LIB


def build_synth(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(CSRC, "fcc_synth.cpp")
    if not force and not _stale(SYNTH_LIB, [src, os.path.join(INCLUDE, "fastcc_synth.h")]):
        return SYNTH_LIB
    tmp = SYNTH_LIB + ".tmp"
    cmd = ["g++", "-std=c++17", "-O3", "-fopenmp", "-fPIC", "-shared", "-o", tmp, src]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, SYNTH_LIB)
    return SYNTH_LIB


def build_cli(verbose=False, force=False):
    src = os.path.join(HOST, "fcc_benchmark.cpp")
    deps = [src, GPU_LIB] + [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".hpp")]
    if not force and not _stale(CLI, deps):
        return CLI
    tmp = CLI + ".tmp"
    cmd = ["g++", "-std=c++17", "-O2", "-I", HOST, "-I", INCLUDE, src, "-L", BUILD, "-lfastcc_gpu",
           "-Wl,-rpath,$ORIGIN", "-o", tmp]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, CLI)
    return CLI


def build_all(verbose=False, force=False):
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_gpu, verbose, force)
        f2 = ex.submit(build_synth, verbose, force)
        out = f1.result(), f2.result()
    build_cli(verbose, force)
    return out


if __name__ == "__main__":
    print(build_all(verbose=True))
