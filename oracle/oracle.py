"""TEST INFRASTRUCTURE ONLY: ctypes access to the CPU oracle.

* ``liboracle.so`` (oracle/fastcc_oracle.cpp): the restatement of the
  reference's ``Tensor<DT>::fastcc_multiply`` (contract.hpp:824-912), plus a
  brute-force join and the 64-bit product count.
* ``libfastcc_ref.so`` (oracle/ref_harness.cpp): the reference's own code,
  compiled from its sources by ``make -C oracle ref``; it exists only where the
  reference sources are present, and is used to pin the restatement.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, as the checker or the timed CPU baseline.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def reference_sources():
    """Directory of the reference's sources (contract.hpp, benchmark.cpp, ...):
    $FASTCC_REFERENCE, else the read-only checkout this build was made
    against. Absent on machines that only run the tests."""
    return os.environ.get("FASTCC_REFERENCE", "/root/reference")


def reference_present():
    return os.path.exists(os.path.join(reference_sources(), "contract.hpp"))


LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libfastcc_ref.so")


class _Tensor(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int32), ("nnz", ctypes.c_int64),
                ("coords", ctypes.c_void_p), ("values", ctypes.c_void_p),
                ("max_index", ctypes.c_void_p)]


class _Result(ctypes.Structure):
    _fields_ = [("nnz", ctypes.c_int64), ("order", ctypes.c_int32),
                ("left", ctypes.POINTER(ctypes.c_uint64)),
                ("right", ctypes.POINTER(ctypes.c_uint64)),
                ("coords", ctypes.POINTER(ctypes.c_int32)),
                ("values", ctypes.POINTER(ctypes.c_double)),
                ("abs_sum", ctypes.POINTER(ctypes.c_double)),
                ("products", ctypes.c_int64),
                ("index_ms", ctypes.c_double), ("compute_ms", ctypes.c_double),
                ("total_ms", ctypes.c_double)]


def build(ref=False):
    """Compile liboracle.so (and the reference harness when ref=True)."""
    subprocess.check_call(["make", "-s", "-C", HERE] + (["ref", f"REF={reference_sources()}"] if ref else ["all"]))


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.orc_fastcc_multiply.restype = ctypes.c_int
        _lib.orc_bruteforce.restype = ctypes.c_int
        _lib.orc_count_products.restype = ctypes.c_int64
        _lib.orc_infer_shape.restype = ctypes.c_int
    return _lib


def ref_available():
    return os.path.exists(REF_PATH)


def ref_lib():
    global _ref
    if _ref is None:
        _ref = ctypes.CDLL(REF_PATH)
        _ref.ref_fastcc_multiply.restype = ctypes.c_int
    return _ref


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None and a.size else ctypes.c_void_p(0)


class _Keep:
    """Holds numpy arrays alive while a ctypes struct points at them."""

    def __init__(self, coords, values, max_index):
        self.coords = np.ascontiguousarray(coords, dtype=np.int32)
        self.values = np.ascontiguousarray(values, dtype=np.float64)
        self.max_index = np.ascontiguousarray(max_index, dtype=np.int32)
        order = self.coords.shape[1] if self.coords.ndim == 2 else len(self.max_index)
        self.t = _Tensor(order, self.values.shape[0], _ptr(self.coords), _ptr(self.values),
                         _ptr(self.max_index))


def infer_shape(coords):
    """Per-mode max index (Tensor::_infer_shape, contract.hpp:124-144)."""
    coords = np.asarray(coords)
    if coords.shape[0] == 0:
        return np.zeros(coords.shape[1], np.int32)
    return coords.max(axis=0).astype(np.int32)


def _take(res, want_abs, keep=True):
    n, d = res.nnz, res.order
    out = {
        "order": d,
        "nnz": n,
        "products": res.products,
        "index_ms": res.index_ms,
        "compute_ms": res.compute_ms,
        "total_ms": res.total_ms,
    }
    if keep:
        out["left"] = np.ctypeslib.as_array(res.left, (max(n, 1),))[:n].copy()
        out["right"] = np.ctypeslib.as_array(res.right, (max(n, 1),))[:n].copy()
        out["values"] = np.ctypeslib.as_array(res.values, (max(n, 1),))[:n].copy()
        out["coords"] = np.ctypeslib.as_array(res.coords, (max(n * d, 1),))[: n * d].reshape(n, d).copy()
        if want_abs:
            out["abs_sum"] = np.ctypeslib.as_array(res.abs_sum, (max(n, 1),))[:n].copy()
    lib().orc_free(ctypes.byref(res))
    return out


def fastcc_multiply(a_coords, a_vals, a_max, b_coords, b_vals, b_max, ctr_a, ctr_b,
                    tile_size=100, nthreads=0, want_abs=False, keep=True):
    """The restatement; returns dict of numpy arrays (unsorted, reference order).
    keep=False returns only the counts and the in-library times (index_ms,
    compute_ms, total_ms) and drops the entries."""
    ka, kb = _Keep(a_coords, a_vals, a_max), _Keep(b_coords, b_vals, b_max)
    ca = np.ascontiguousarray(ctr_a, np.int32)
    cb = np.ascontiguousarray(ctr_b, np.int32)
    res = _Result()
    rc = lib().orc_fastcc_multiply(ctypes.byref(ka.t), ctypes.byref(kb.t), _ptr(ca), _ptr(cb),
                                   ctypes.c_int32(len(ca)), ctypes.c_int32(tile_size),
                                   ctypes.c_int32(nthreads), ctypes.c_int32(1 if want_abs else 0),
                                   ctypes.byref(res))
    if rc != 0:
        raise ValueError("oracle rejected the arguments")
    return _take(res, want_abs, keep)


def bruteforce(a_coords, a_vals, a_max, b_coords, b_vals, b_max, ctr_a, ctr_b):
    ka, kb = _Keep(a_coords, a_vals, a_max), _Keep(b_coords, b_vals, b_max)
    ca = np.ascontiguousarray(ctr_a, np.int32)
    cb = np.ascontiguousarray(ctr_b, np.int32)
    res = _Result()
    rc = lib().orc_bruteforce(ctypes.byref(ka.t), ctypes.byref(kb.t), _ptr(ca), _ptr(cb),
                              ctypes.c_int32(len(ca)), ctypes.byref(res))
    if rc != 0:
        raise ValueError("oracle rejected the arguments")
    return _take(res, True)


def multiply_batch_modes(a_coords, a_vals, b_coords, b_vals, ctr_a, ctr_b, batch_a, batch_b):
    """Tensor<DT>::multiply(other, left_contr, left_batch, right_contr,
    right_batch) (contract.hpp:284-367), restated with Python dictionaries for
    small cases: A entries are grouped by (batch coordinates in left_batch
    order, contracted coordinates) and joined with B's groups; each pair adds
    a * b into the output (batch, A external, B external), externals in
    ascending mode order (OutputCoordinate(batch, left, right).merge()).
    Returns (coords (n, order) int64 sorted, values, sums of |a*b|)."""
    a_coords = np.asarray(a_coords)
    b_coords = np.asarray(b_coords)
    ext_a = [m for m in range(a_coords.shape[1]) if m not in list(ctr_a) + list(batch_a)]
    ext_b = [m for m in range(b_coords.shape[1]) if m not in list(ctr_b) + list(batch_b)]
    groups = {}
    for i in range(b_coords.shape[0]):
        key = tuple(int(b_coords[i, m]) for m in list(batch_b) + list(ctr_b))
        groups.setdefault(key, []).append(i)
    acc, mag = {}, {}
    for i in range(a_coords.shape[0]):
        key = tuple(int(a_coords[i, m]) for m in list(batch_a) + list(ctr_a))
        for j in groups.get(key, ()):
            out = key[:len(batch_a)] + tuple(int(a_coords[i, m]) for m in ext_a) + \
                tuple(int(b_coords[j, m]) for m in ext_b)
            p = float(a_vals[i]) * float(b_vals[j])
            acc[out] = acc.get(out, 0.0) + p
            mag[out] = mag.get(out, 0.0) + abs(p)
    order = len(batch_a) + len(ext_a) + len(ext_b)
    keys = sorted(acc)
    coords = np.array(keys, np.int64).reshape(len(keys), order)
    return coords, np.array([acc[k] for k in keys]), np.array([mag[k] for k in keys])


def count_products(a_coords, a_vals, a_max, b_coords, b_vals, b_max, ctr_a, ctr_b):
    ka, kb = _Keep(a_coords, a_vals, a_max), _Keep(b_coords, b_vals, b_max)
    ca = np.ascontiguousarray(ctr_a, np.int32)
    cb = np.ascontiguousarray(ctr_b, np.int32)
    return int(lib().orc_count_products(ctypes.byref(ka.t), ctypes.byref(kb.t), _ptr(ca), _ptr(cb),
                                        ctypes.c_int32(len(ca))))


def reference_multiply(a_coords, a_vals, a_max, b_coords, b_vals, b_max, ctr_a, ctr_b,
                       tile_size=100, shipped=False):
    """The reference's own fastcc_multiply (needs oracle/_ref). shipped=False plugs
    in the recording accumulator; shipped=True runs TileAccumulator<double>."""
    r = ref_lib()
    ac = np.ascontiguousarray(a_coords, np.int32)
    bc = np.ascontiguousarray(b_coords, np.int32)
    av = np.ascontiguousarray(a_vals, np.float64)
    bv = np.ascontiguousarray(b_vals, np.float64)
    am = np.ascontiguousarray(a_max, np.int32)
    bm = np.ascontiguousarray(b_max, np.int32)
    ca = np.ascontiguousarray(ctr_a, np.int32)
    cb = np.ascontiguousarray(ctr_b, np.int32)
    n = ctypes.c_int64()
    left = ctypes.POINTER(ctypes.c_uint64)()
    right = ctypes.POINTER(ctypes.c_uint64)()
    vals = ctypes.POINTER(ctypes.c_double)()
    coords = ctypes.POINTER(ctypes.c_int32)()
    order = ctypes.c_int32()
    ms = ctypes.c_double()
    i32, i64 = ctypes.c_int32, ctypes.c_int64
    rc = r.ref_fastcc_multiply(i32(ac.shape[1]), i64(ac.shape[0]), _ptr(ac), _ptr(av), _ptr(am),
                               i32(bc.shape[1]), i64(bc.shape[0]), _ptr(bc), _ptr(bv), _ptr(bm),
                               _ptr(ca), _ptr(cb), ctypes.c_int32(len(ca)),
                               ctypes.c_int32(tile_size), ctypes.c_int32(1 if shipped else 0),
                               ctypes.byref(n), ctypes.byref(left), ctypes.byref(right),
                               ctypes.byref(vals), ctypes.byref(coords), ctypes.byref(order),
                               ctypes.byref(ms))
    if rc != 0:
        raise ValueError("reference harness rejected the arguments")
    k = n.value
    out = {"order": order.value, "ms": ms.value,
           "values": np.ctypeslib.as_array(vals, (k + 1,))[:k].copy()}
    if shipped:
        d = order.value
        out["coords"] = np.ctypeslib.as_array(coords, (k * d + 1,))[: k * d].reshape(k, d).copy()
        r.ref_free(coords)
    else:
        out["left"] = np.ctypeslib.as_array(left, (k + 1,))[:k].copy()
        out["right"] = np.ctypeslib.as_array(right, (k + 1,))[:k].copy()
        r.ref_free(left)
        r.ref_free(right)
    r.ref_free(vals)
    return out


def reference_multiply_modes(a_coords, a_vals, a_max, b_coords, b_vals, b_max, ctr_a, ctr_b, batch_a, batch_b):
    """The reference's own Tensor<double>::multiply with batch modes
    (contract.hpp:286-367; needs oracle/_ref). Returns (coords (n, order)
    int32 in the reference's entry order, values)."""
    r = ref_lib()
    r.ref_multiply_modes.restype = ctypes.c_int
    arr = lambda x, t: np.ascontiguousarray(x, t)
    ac, bc = arr(a_coords, np.int32), arr(b_coords, np.int32)
    av, bv = arr(a_vals, np.float64), arr(b_vals, np.float64)
    am, bm = arr(a_max, np.int32), arr(b_max, np.int32)
    ca, cb, ba, bb = (arr(x, np.int32) for x in (ctr_a, ctr_b, batch_a, batch_b))
    n = ctypes.c_int64()
    coords = ctypes.POINTER(ctypes.c_int32)()
    vals = ctypes.POINTER(ctypes.c_double)()
    order = ctypes.c_int32()
    i32, i64 = ctypes.c_int32, ctypes.c_int64
    rc = r.ref_multiply_modes(i32(ac.shape[1]), i64(ac.shape[0]), _ptr(ac), _ptr(av), _ptr(am),
                              i32(bc.shape[1]), i64(bc.shape[0]), _ptr(bc), _ptr(bv), _ptr(bm),
                              _ptr(ca), _ptr(cb), ctypes.c_int32(len(ca)), _ptr(ba), _ptr(bb),
                              ctypes.c_int32(len(ba)), ctypes.byref(n), ctypes.byref(coords),
                              ctypes.byref(order), ctypes.byref(vals))
    if rc != 0:
        raise ValueError("reference harness rejected the arguments")
    k, d = n.value, order.value
    out_c = np.ctypeslib.as_array(coords, (k * d + 1,))[: k * d].reshape(k, d).copy()
    out_v = np.ctypeslib.as_array(vals, (k + 1,))[:k].copy()
    r.ref_free(coords)
    r.ref_free(vals)
    return out_c, out_v


def external_radices(max_index, ctr):
    """Radices (max+1) of the non-contracted modes in ascending mode order."""
    ctr = set(int(c) for c in ctr)
    return [int(max_index[m]) + 1 for m in range(len(max_index)) if m not in ctr]


def decode(lin, radices):
    """Mixed-radix decode, last mode least significant."""
    lin = np.asarray(lin, dtype=np.uint64).copy()
    out = np.zeros((lin.shape[0], len(radices)), np.int64)
    for e in range(len(radices) - 1, -1, -1):
        r = np.uint64(radices[e])
        out[:, e] = (lin % r).astype(np.int64)
        lin //= r
    return out


def sort_output(coords, values, *extra):
    """Lexicographic sort of output coordinates (for order-free comparison)."""
    coords = np.asarray(coords)
    if coords.shape[0] == 0 or coords.shape[1] == 0:
        return (coords, values) + tuple(extra)
    idx = np.lexsort(coords.T[::-1])
    return (coords[idx], values[idx]) + tuple(e[idx] for e in extra)
