"""Seeded synthetic workloads standing in for the FROSTT tensors the reference
benchmarks on (scripts/*.sh read them from Zenodo; none are used here).

Each builder returns a dict with host operands ``a`` and ``b`` (fastcc_gpu.Tensor
with numpy arrays), the contracted modes and a name. Operand shapes are the
declared extents minus one, set on both operands the way
``Tensor(int, int, int*)`` plus ``CoOrdinate::set_shape`` would
(contract.hpp:58-65, coordinate.hpp:653), so contracted modes of the two
operands share their radices.

* readme:  result(i,j,k) = a(i,c0,j,c1) * b(k,c0,c1); a 256x64x256x64 with
  200,000 uniform distinct coordinates, b 512x64x64 with 100,000; values
  uniform[-1,1); contract a{1,3} with b{1,2} (README.md:9-13).
* zipf3:   A(i,c0,c1) * A(j,c0,c1); A 20,000 x 20,000 x 500,000, 10M distinct
  nonzeros, every mode Zipf(1.2), values sign-random lognormal(0,1).
* twomode: A(c0,j,c1,l) * A(c0,j',c1,l'); A 5,000 x 5,000 x 2,000 x 50, 5M
  distinct nonzeros, modes 0,1 Zipf(1.1), modes 2,3 uniform, values
  uniform[-1,1); contract {0,2} with {0,2}.
* batched: 256 contractions of the readme pattern with log-uniform nnz, mode
  extents uniform in [32, 1024] and per-mode Zipf exponents in [1.0, 1.5].
"""
import numpy as np

from fastcc_gpu import Tensor, synth_coo


def _tensor(seed, extents, zipf, nnz, lognormal=False):
    c, v = synth_coo(seed, extents, zipf, nnz, lognormal)
    return Tensor(c, v, np.asarray(extents, np.int64) - 1)


def readme(seed=1, scale=1.0):
    na, nb = int(200_000 * scale), int(100_000 * scale)
    a = _tensor(seed, [256, 64, 256, 64], 0.0, na)
    b = _tensor(seed + 1000003, [512, 64, 64], 0.0, nb)
    return {"name": "readme 256x64x256x64 (200k) x 512x64x64 (100k), ctr {1,3}x{1,2}",
            "a": a, "b": b, "ctr_a": [1, 3], "ctr_b": [1, 2]}


def zipf3(seed=1, nnz=10_000_000, dims=(20_000, 20_000, 500_000)):
    a = _tensor(seed, list(dims), 1.2, nnz, lognormal=True)
    return {"name": f"zipf3 {dims[0]}x{dims[1]}x{dims[2]} ({nnz} nnz, Zipf 1.2) self-contract {{1,2}}",
            "a": a, "b": a, "ctr_a": [1, 2], "ctr_b": [1, 2]}


def twomode(seed=1, nnz=5_000_000, dims=(5_000, 5_000, 2_000, 50)):
    a = _tensor(seed, list(dims), [1.1, 1.1, 0.0, 0.0], nnz)
    return {"name": f"twomode {dims[0]}x{dims[1]}x{dims[2]}x{dims[3]} ({nnz} nnz) self-contract {{0,2}}",
            "a": a, "b": a, "ctr_a": [0, 2], "ctr_b": [0, 2]}


def _split_draws(seed, n):
    """n uniforms in [0,1) from the generator's counter stream (stable across numpy versions)."""
    from fastcc_gpu import synth_lib
    import ctypes
    raw = np.empty(n, np.uint64)
    synth_lib().fcc_synth_raw(ctypes.c_uint64(seed), ctypes.c_uint64(77), ctypes.c_int64(n),
                              ctypes.c_void_p(raw.ctypes.data))
    return (raw >> np.uint64(11)).astype(np.float64) / 9007199254740992.0


def batched(seed=1, count=256, nnz_lo=1e3, nnz_hi=2e6, dim_lo=32, dim_hi=1024):
    """Instances of the readme pattern a(i,c0,j,c1) x b(k,c0,c1) with uneven sizes."""
    u = _split_draws(seed, count * 16).reshape(count, 16)
    out = []
    for t in range(count):
        d = [int(dim_lo + np.floor(u[t, q] * (dim_hi - dim_lo + 1))) for q in range(5)]
        ea = [d[0], d[1], d[2], d[3]]          # i, c0, j, c1
        eb = [d[4], d[1], d[3]]                # k, c0, c1 (contracted extents shared)
        s = [1.0 + 0.5 * u[t, 5 + q] for q in range(5)]
        za = [s[0], s[1], s[2], s[3]]
        zb = [s[4], s[1], s[3]]
        nnz_a = float(np.exp(np.log(nnz_lo) + u[t, 10] * (np.log(nnz_hi) - np.log(nnz_lo))))
        nnz_a = int(min(nnz_a, 0.5 * np.prod(ea, dtype=np.float64)))
        nnz_b = int(min(0.5 * nnz_a, 0.5 * np.prod(eb, dtype=np.float64)))
        a = _tensor(seed * 1000 + 2 * t + 1, ea, za, max(nnz_a, 1))
        b = _tensor(seed * 1000 + 2 * t + 2, eb, zb, max(nnz_b, 1))
        out.append({"name": f"batched[{t}]", "a": a, "b": b, "ctr_a": [1, 3], "ctr_b": [1, 2]})
    return out


CONFIGS = {"readme": readme, "zipf3": zipf3, "twomode": twomode}
