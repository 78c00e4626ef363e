"""ctypes binding of libfastcc_gpu.so (include/fastcc_gpu.h) and of the seeded
generator libfastcc_synth.so (include/fastcc_synth.h).

Loads the in-tree libraries from ``_build/`` and raises if they are missing:
there is no CPU fallback. ``Tensor`` and ``Context.fastcc_multiply`` mirror the
reference call ``a.fastcc_multiply<TileAccumulator<double>, double>(b, ctrA,
ctrB, tile_size)`` (contract.hpp:824-912); the C++ header host/contract.hpp is
the drop-in for C++ callers.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
GPU_LIB = os.path.join(BUILD, "libfastcc_gpu.so")
SYNTH_LIB = os.path.join(BUILD, "libfastcc_synth.so")

FCC_HOST, FCC_DEVICE = 0, 1
ACC_AUTO, ACC_DENSE, ACC_HASH = 0, 1, 2
RADIX_PER_OPERAND, RADIX_SHARED = 0, 1
DENSE_AUTO, DENSE_BITMASK, DENSE_SENTINEL = 0, 1, 2
PHASES = ["upload", "index", "plan", "contract", "merge", "total"]
CLASS_DENSE, CLASS_HASH_L, CLASS_HASH_M, CLASS_HASH_S, CLASS_DENSE_FLAT = 0, 1, 2, 3, 4
NUM_CLASSES = 5
SCHED_RULE, SCHED_LEARNED, SCHED_FORCE = 0, 1, 2
SCHED_FEATURES, SCHED_HIDDEN = 12, 64
SCHED_MODEL_FLOATS = 2 * 12 + 12 * 64 + 64 + 64 * 64 + 64 + 64 * NUM_CLASSES + NUM_CLASSES
STATUS = {0: "ok", 1: "invalid argument", 2: "out of memory", 3: "hash accumulator full",
          4: "bounded device wait timed out", 5: "CUDA error", 6: "index space exceeds 64 bits",
          7: "no usable sm_103 device", 8: "output buffer too small"}


class FccError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class _CTensor(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int32), ("nnz", ctypes.c_int64),
                ("max_index", ctypes.c_void_p), ("coords", ctypes.c_void_p),
                ("stride_nnz", ctypes.c_int64), ("stride_mode", ctypes.c_int64),
                ("values", ctypes.c_void_p), ("location", ctypes.c_int32)]


class Options(ctypes.Structure):
    _fields_ = [("tile_size", ctypes.c_int32), ("accumulator", ctypes.c_int32),
                ("radix_mode", ctypes.c_int32), ("rows_per_tile", ctypes.c_int32),
                ("products_per_item", ctypes.c_int64), ("dense_cap", ctypes.c_int32),
                ("hash_slots", ctypes.c_int32), ("timing", ctypes.c_int32),
                ("esc_small", ctypes.c_int32), ("capacity_hint", ctypes.c_int64),
                ("dense_mode", ctypes.c_int32), ("tile_threads", ctypes.c_int32),
                ("hot_columns", ctypes.c_int32), ("schedule", ctypes.c_int32),
                ("dense_fill_log2", ctypes.c_int32), ("dense_staging", ctypes.c_int32),
                ("sched_mix_margin", ctypes.c_int32), ("hash_esc", ctypes.c_int32),
                ("out_waves", ctypes.c_int32), ("esc_group", ctypes.c_int32),
                ("wait_polls", ctypes.c_int32), ("fault_wait", ctypes.c_int32),
                ("dense_kernel", ctypes.c_int32), ("esc_reduce", ctypes.c_int32)]

    def __init__(self, **kw):
        super().__init__()
        self.tile_size = 100
        for k, v in kw.items():
            setattr(self, k, v)


_lib = None
_synth = None


def lib():
    """The CUDA library; raises when it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(GPU_LIB):
            raise RuntimeError(f"{GPU_LIB} is missing: run __graft_entry__.build() first")
        L = ctypes.CDLL(GPU_LIB)
        vp, i32, i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
        L.fcc_ctx_create.argtypes = [i32, ctypes.POINTER(vp)]
        L.fcc_ctx_destroy.argtypes = [vp]
        L.fcc_ctx_set_stream.argtypes = [vp, vp]
        L.fcc_last_error.argtypes = [vp]
        L.fcc_last_error.restype = ctypes.c_char_p
        L.fcc_contract.argtypes = [vp, ctypes.POINTER(_CTensor), ctypes.POINTER(_CTensor), vp, vp, i32,
                                   ctypes.POINTER(Options), ctypes.POINTER(vp)]
        L.fcc_count_products.argtypes = [vp, ctypes.POINTER(_CTensor), ctypes.POINTER(_CTensor), vp, vp,
                                         i32, ctypes.POINTER(Options), ctypes.POINTER(i64)]
        L.fcc_contract_batch.argtypes = [vp, i32, ctypes.POINTER(_CTensor), ctypes.POINTER(_CTensor), vp, vp,
                                         i32, ctypes.POINTER(Options), ctypes.POINTER(vp), vp]
        L.fcc_contract_into.argtypes = [vp, ctypes.POINTER(_CTensor), ctypes.POINTER(_CTensor), vp, vp, i32,
                                        ctypes.POINTER(Options), vp, i64, vp, i64, ctypes.POINTER(i64),
                                        ctypes.POINTER(i64)]
        L.fcc_contract_modes.argtypes = [vp, ctypes.POINTER(_CTensor), ctypes.POINTER(_CTensor), vp, vp, i32, vp,
                                         vp, i32, ctypes.POINTER(Options), ctypes.POINTER(vp)]
        L.fcc_autotune.argtypes = [vp, ctypes.POINTER(_CTensor), ctypes.POINTER(_CTensor), vp, vp, i32,
                                   ctypes.POINTER(Options), i32, ctypes.POINTER(Options),
                                   ctypes.POINTER(ctypes.c_double)]
        L.fcc_autotune_batch.argtypes = [vp, i32, ctypes.POINTER(_CTensor), ctypes.POINTER(_CTensor), vp, vp,
                                         i32, ctypes.POINTER(Options), i32, ctypes.POINTER(Options),
                                         ctypes.POINTER(ctypes.c_double)]
        L.fcc_sched_set_model.argtypes = [vp, vp, i64]
        L.fcc_sched_last_tiles.argtypes = [vp, vp, vp, vp, i64, ctypes.POINTER(i64)]
        L.fcc_mlp_predict.argtypes = [vp, vp, i64, vp, vp]
        L.fcc_mlp_grad.argtypes = [vp, vp, vp, vp, i64, vp, vp, ctypes.POINTER(ctypes.c_float)]
        L.fcc_mlp_train.argtypes = [vp, vp, vp, vp, i64, i32, i32, ctypes.c_float, ctypes.c_uint64, vp,
                                    ctypes.POINTER(ctypes.c_float)]
        L.fcc_result_info.argtypes = [vp, ctypes.POINTER(i32), ctypes.POINTER(i64), ctypes.POINTER(i64)]
        L.fcc_result_device.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(i64), ctypes.POINTER(vp)]
        L.fcc_result_copy_to_host.argtypes = [vp, vp, i64, i64, vp]
        L.fcc_result_free.argtypes = [vp]
        L.fcc_last_timings.argtypes = [vp, ctypes.POINTER(ctypes.c_double), i32]
        L.fcc_status_string.restype = ctypes.c_char_p
        L.fcc_launch_count.restype = ctypes.c_int64
        _lib = L
    return _lib


def synth_lib():
    global _synth
    if _synth is None:
        if not os.path.exists(SYNTH_LIB):
            raise RuntimeError(f"{SYNTH_LIB} is missing: run __graft_entry__.build() first")
        _synth = ctypes.CDLL(SYNTH_LIB)
        _synth.fcc_synth_coo.restype = ctypes.c_int
    return _synth


# ------------------------------------------------------------- tensors ----

class Tensor:
    """A COO operand: coords (nnz, order) int32, values (nnz,) float64 and the
    per-mode max index (the reference's ``shape`` after ``_infer_shape``,
    contract.hpp:124-144). coords/values may be numpy arrays (host) or CUDA
    torch tensors (device)."""

    def __init__(self, coords, values, max_index=None):
        self.coords = coords
        self.values = values
        if max_index is None:
            c = np.asarray(coords) if isinstance(coords, np.ndarray) else coords.cpu().numpy()
            max_index = c.max(axis=0) if c.shape[0] else np.zeros(c.shape[1], np.int32)
        self.max_index = np.ascontiguousarray(max_index, dtype=np.int32)

    @property
    def order(self):
        return int(self.max_index.shape[0])

    @property
    def nnz(self):
        return int(self.values.shape[0])

    def _struct(self):
        c, v = self.coords, self.values
        if isinstance(c, np.ndarray):
            c = np.ascontiguousarray(c, dtype=np.int32)
            v = np.ascontiguousarray(v, dtype=np.float64)
            self._keep = (c, v)
            cp, vp_, loc = c.ctypes.data, v.ctypes.data, FCC_HOST
            sn, sm = c.strides[0] // 4, (c.strides[1] // 4 if c.ndim == 2 else 1)
        else:  # torch CUDA tensors
            import torch
            assert c.dtype == torch.int32 and v.dtype == torch.float64 and c.is_cuda and v.is_cuda
            cp, vp_, loc = c.data_ptr(), v.data_ptr(), FCC_DEVICE
            sn, sm = c.stride(0), c.stride(1)
            self._keep = (c, v)
        return _CTensor(self.order, self.nnz, self.max_index.ctypes.data, cp or None, sn, sm,
                        vp_ or None, loc)


class Result:
    """A device-resident contraction result (order, nnz, SoA coords, values)."""

    def __init__(self, ctx, handle):
        self._ctx = ctx
        self._h = ctypes.c_void_p(handle)
        o, n, p = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int64()
        lib().fcc_result_info(self._h, ctypes.byref(o), ctypes.byref(n), ctypes.byref(p))
        self.order, self.nnz, self.products = o.value, n.value, p.value

    def device_pointers(self):
        c, s, v = ctypes.c_void_p(), ctypes.c_int64(), ctypes.c_void_p()
        lib().fcc_result_device(self._h, ctypes.byref(c), ctypes.byref(s), ctypes.byref(v))
        return c.value, s.value, v.value

    def to_numpy(self, coords_out=None, values_out=None):
        """(coords (nnz, order) int32, values (nnz,) float64) on the host."""
        coords = coords_out if coords_out is not None else np.empty((self.nnz, self.order), np.int32)
        vals = values_out if values_out is not None else np.empty(self.nnz, np.float64)
        if self.nnz:
            rc = lib().fcc_result_copy_to_host(self._h, coords.ctypes.data if self.order else None,
                                               coords.strides[0] // 4 if self.order else 1, 1,
                                               vals.ctypes.data)
            self._ctx._check(rc)
        return coords, vals

    def to_numpy_soa(self, coords_out, values_out):
        """Copies into caller buffers: coords_out (order, >= nnz) int32 (one row
        per mode), values_out (>= nnz) float64. Pinned buffers copy fastest."""
        assert coords_out.dtype == np.int32 and values_out.dtype == np.float64
        assert values_out.shape[0] >= self.nnz
        if self.order:
            assert coords_out.shape[0] == self.order and coords_out.shape[1] >= self.nnz
        if self.nnz:
            rc = lib().fcc_result_copy_to_host(self._h, coords_out.ctypes.data if self.order else None, 1,
                                               coords_out.strides[0] // 4 if self.order else 0,
                                               values_out.ctypes.data)
            self._ctx._check(rc)

    def free(self):
        if self._h:
            lib().fcc_result_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Context:
    """One device, one stream, one workspace (fcc_ctx)."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        rc = lib().fcc_ctx_create(device, ctypes.byref(h))
        if rc != 0:
            raise FccError(rc, lib().fcc_last_error(None).decode())
        self._h = h

    def _check(self, rc):
        if rc != 0:
            raise FccError(rc, lib().fcc_last_error(self._h).decode())

    def set_stream(self, stream_ptr):
        self._check(lib().fcc_ctx_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)))

    def contract(self, a, b, ctr_a, ctr_b, opts=None):
        ca = np.ascontiguousarray(ctr_a, dtype=np.int32)
        cb = np.ascontiguousarray(ctr_b, dtype=np.int32)
        if ca.shape != cb.shape:
            raise ValueError("contracted mode lists differ in length")
        ta, tb = a._struct(), b._struct()
        out = ctypes.c_void_p()
        o = opts if opts is not None else Options()
        rc = lib().fcc_contract(self._h, ctypes.byref(ta), ctypes.byref(tb),
                                ca.ctypes.data if ca.size else None, cb.ctypes.data if cb.size else None,
                                int(ca.size), ctypes.byref(o), ctypes.byref(out))
        self._check(rc)
        return Result(self, out.value)

    def contract_into(self, a, b, ctr_a, ctr_b, out_coords, out_values, opts=None):
        """fcc_contract_into: the output written into caller buffers, out_coords
        (order, capacity) int32/uint32 and out_values (capacity,) float64, as
        numpy arrays in pinned host memory (filled wave by wave while the
        contraction runs)
        or CUDA torch tensors. Returns (entries, multiply-adds); raises
        FccError(FCC_ERR_CAPACITY) with .needed when they do not fit."""
        ca = np.ascontiguousarray(ctr_a, dtype=np.int32)
        cb = np.ascontiguousarray(ctr_b, dtype=np.int32)
        ta, tb = a._struct(), b._struct()
        if isinstance(out_values, np.ndarray):
            cptr, vptr = out_coords.ctypes.data, out_values.ctypes.data
            stride = out_coords.strides[0] // 4 if out_coords.ndim == 2 else out_values.shape[0]
        else:
            cptr, vptr = out_coords.data_ptr(), out_values.data_ptr()
            stride = out_coords.stride(0) if out_coords.dim() == 2 else out_values.shape[0]
        cap = int(out_values.shape[0])
        n, p = ctypes.c_int64(), ctypes.c_int64()
        o = opts if opts is not None else Options()
        rc = lib().fcc_contract_into(self._h, ctypes.byref(ta), ctypes.byref(tb),
                                     ca.ctypes.data if ca.size else None, cb.ctypes.data if cb.size else None,
                                     int(ca.size), ctypes.byref(o), cptr or None, stride, vptr or None, cap,
                                     ctypes.byref(n), ctypes.byref(p))
        if rc != 0:
            err = FccError(rc, lib().fcc_last_error(self._h).decode())
            err.needed = n.value
            raise err
        return n.value, p.value

    def contract_modes(self, a, b, ctr_a, ctr_b, batch_a, batch_b, opts=None):
        """Contraction with batch modes (fcc_contract_modes; the reference's
        Tensor::multiply(other, left_contr, left_batch, right_contr,
        right_batch)): output modes = batch modes, A's external, B's external."""
        arrs = [np.ascontiguousarray(x, dtype=np.int32) for x in (ctr_a, ctr_b, batch_a, batch_b)]
        if arrs[0].shape != arrs[1].shape or arrs[2].shape != arrs[3].shape:
            raise ValueError("mode lists differ in length")
        ta, tb = a._struct(), b._struct()
        out = ctypes.c_void_p()
        o = opts if opts is not None else Options()
        ptr = lambda x: x.ctypes.data if x.size else None
        self._check(lib().fcc_contract_modes(self._h, ctypes.byref(ta), ctypes.byref(tb), ptr(arrs[0]), ptr(arrs[1]),
                                             int(arrs[0].size), ptr(arrs[2]), ptr(arrs[3]), int(arrs[2].size),
                                             ctypes.byref(o), ctypes.byref(out)))
        return Result(self, out.value)

    def contract_batch(self, As, Bs, ctr_a, ctr_b, opts=None):
        """n independent products As[t] x Bs[t] in one pipeline
        (fcc_contract_batch). Returns (Result, counts): the result's mode 0 is
        the instance, counts[t] the entries of instance t."""
        if len(As) != len(Bs) or not As:
            raise ValueError("As and Bs must be non-empty and of one length")
        ca = np.ascontiguousarray(ctr_a, dtype=np.int32)
        cb = np.ascontiguousarray(ctr_b, dtype=np.int32)
        if ca.shape != cb.shape:
            raise ValueError("contracted mode lists differ in length")
        n = len(As)
        ta = (_CTensor * n)(*[a._struct() for a in As])
        tb = (_CTensor * n)(*[b._struct() for b in Bs])
        counts = np.zeros(n, np.int64)
        out = ctypes.c_void_p()
        o = opts if opts is not None else Options()
        rc = lib().fcc_contract_batch(self._h, n, ta, tb, ca.ctypes.data if ca.size else None,
                                      cb.ctypes.data if cb.size else None, int(ca.size), ctypes.byref(o),
                                      ctypes.byref(out), counts.ctypes.data)
        self._check(rc)
        return Result(self, out.value), counts

    def fastcc_multiply(self, a, b, ctr_a, ctr_b, tile_size=100, accumulator=ACC_AUTO):
        """Mirror of Tensor<DT>::fastcc_multiply<AccType, RES>(other, left_contr,
        right_contr, tile_size) (contract.hpp:824-827): returns host arrays."""
        r = self.contract(a, b, ctr_a, ctr_b, Options(tile_size=tile_size, accumulator=accumulator))
        try:
            return r.to_numpy()
        finally:
            r.free()

    def count_products(self, a, b, ctr_a, ctr_b, opts=None):
        ca = np.ascontiguousarray(ctr_a, dtype=np.int32)
        cb = np.ascontiguousarray(ctr_b, dtype=np.int32)
        ta, tb = a._struct(), b._struct()
        n = ctypes.c_int64()
        o = opts if opts is not None else Options()
        self._check(lib().fcc_count_products(self._h, ctypes.byref(ta), ctypes.byref(tb),
                                             ca.ctypes.data if ca.size else None,
                                             cb.ctypes.data if cb.size else None, int(ca.size),
                                             ctypes.byref(o), ctypes.byref(n)))
        return n.value

    # ---- autotuner ----
    def autotune(self, a, b, ctr_a, ctr_b, base=None, reps=2):
        """Fastest candidate schedule for this problem (fcc_autotune): (Options, ms)."""
        ca = np.ascontiguousarray(ctr_a, dtype=np.int32)
        cb = np.ascontiguousarray(ctr_b, dtype=np.int32)
        ta, tb = a._struct(), b._struct()
        best, ms = Options(), ctypes.c_double()
        self._check(lib().fcc_autotune(self._h, ctypes.byref(ta), ctypes.byref(tb),
                                       ca.ctypes.data if ca.size else None, cb.ctypes.data if cb.size else None,
                                       int(ca.size), ctypes.byref(base if base is not None else Options()),
                                       int(reps), ctypes.byref(best), ctypes.byref(ms)))
        return best, ms.value

    def autotune_batch(self, As, Bs, ctr_a, ctr_b, base=None, reps=2):
        """fcc_autotune_batch: (Options, ms) for one fcc_contract_batch call."""
        ca = np.ascontiguousarray(ctr_a, dtype=np.int32)
        cb = np.ascontiguousarray(ctr_b, dtype=np.int32)
        n = len(As)
        ta = (_CTensor * n)(*[x._struct() for x in As])
        tb = (_CTensor * n)(*[x._struct() for x in Bs])
        best, ms = Options(), ctypes.c_double()
        self._check(lib().fcc_autotune_batch(self._h, n, ta, tb, ca.ctypes.data if ca.size else None,
                                             cb.ctypes.data if cb.size else None, int(ca.size),
                                             ctypes.byref(base if base is not None else Options()), int(reps),
                                             ctypes.byref(best), ctypes.byref(ms)))
        return best, ms.value

    @staticmethod
    def options_dict(o):
        return {name: getattr(o, name) for name, _ in Options._fields_ if name not in ("reserved",)}

    def load_default_model(self):
        """Installs the cost model shipped with the package (sched_model.f32); False when absent."""
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "sched_model.f32")
        if not os.path.exists(path):
            return False
        self.sched_set_model(np.fromfile(path, np.float32))
        return True

    # ---- learned tile schedule ----
    def sched_set_model(self, model):
        """Installs an FP32 cost model (SCHED_MODEL_FLOATS floats) or removes it (None)."""
        if model is None:
            self._check(lib().fcc_sched_set_model(self._h, None, 0))
            return
        m = np.ascontiguousarray(model, dtype=np.float32)
        self._check(lib().fcc_sched_set_model(self._h, m.ctypes.data, int(m.size)))

    def sched_last_tiles(self, features=True, cost=True):
        """Per-tile record of the last contraction: dict with 'cls' and, when
        recorded (timing=2), 'features' (ntiles x 12) and 'cost' (ntiles)."""
        n = ctypes.c_int64()
        self._check(lib().fcc_sched_last_tiles(self._h, None, None, None, 0, ctypes.byref(n)))
        nt = n.value
        cls = np.empty(nt, np.int32)
        f = np.empty((nt, SCHED_FEATURES), np.float32) if features else None
        c = np.empty(nt, np.float64) if cost else None
        self._check(lib().fcc_sched_last_tiles(self._h, f.ctypes.data if f is not None else None, cls.ctypes.data,
                                               c.ctypes.data if c is not None else None, nt, ctypes.byref(n)))
        out = {"cls": cls}
        if f is not None:
            out["features"] = f
        if c is not None:
            out["cost"] = c
        return out

    def mlp_predict(self, X, model):
        X = np.ascontiguousarray(X, dtype=np.float32)
        m = np.ascontiguousarray(model, dtype=np.float32)
        Y = np.empty((X.shape[0], NUM_CLASSES), np.float32)
        self._check(lib().fcc_mlp_predict(self._h, X.ctypes.data, X.shape[0], m.ctypes.data, Y.ctypes.data))
        return Y

    def mlp_grad(self, X, Y, M, model):
        X, Y, M = (np.ascontiguousarray(a, dtype=np.float32) for a in (X, Y, M))
        m = np.ascontiguousarray(model, dtype=np.float32)
        g = np.empty(SCHED_MODEL_FLOATS, np.float32)
        loss = ctypes.c_float()
        self._check(lib().fcc_mlp_grad(self._h, X.ctypes.data, Y.ctypes.data, M.ctypes.data, X.shape[0],
                                       m.ctypes.data, g.ctypes.data, ctypes.byref(loss)))
        return g, loss.value

    def mlp_train(self, X, Y, M, model, epochs=200, batch=4096, lr=1e-3, seed=1):
        X, Y, M = (np.ascontiguousarray(a, dtype=np.float32) for a in (X, Y, M))
        m = np.array(model, dtype=np.float32, copy=True)
        loss = ctypes.c_float()
        self._check(lib().fcc_mlp_train(self._h, X.ctypes.data, Y.ctypes.data, M.ctypes.data, X.shape[0],
                                        int(epochs), int(batch), float(lr), int(seed), m.ctypes.data,
                                        ctypes.byref(loss)))
        return m, loss.value

    def timings(self):
        ms = (ctypes.c_double * 6)()
        lib().fcc_last_timings(self._h, ms, 6)
        return dict(zip(PHASES, list(ms)))

    def close(self):
        if self._h:
            lib().fcc_ctx_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def launch_count():
    """Kernels launched by the library in this process so far."""
    return int(lib().fcc_launch_count())


def shared_update_rate(mode):
    """Measured FP64 shared-memory accumulation rate (updates per second);
    mode 0 atomicAdd of a product, 1 compare-and-swap FMA, 2 plain FMA."""
    r = ctypes.c_double()
    rc = lib().fcc_diag_shared_update_rate(ctypes.c_int32(mode), ctypes.byref(r))
    if rc != 0:
        raise FccError(rc, "fcc_diag_shared_update_rate failed")
    return r.value


def radix_sort(keys, vals, nbits, reps=1):
    """The library's stable radix sort of (keys, vals) on the low nbits of
    each key: returns (sorted keys, permuted vals, mean ms per sort)."""
    keys = np.ascontiguousarray(keys)
    vals = np.ascontiguousarray(vals)
    if keys.dtype not in (np.uint32, np.uint64) or vals.dtype.itemsize not in (4, 8) or vals.shape != keys.shape:
        raise ValueError("keys: uint32 or uint64; vals: one 32- or 64-bit payload per key")
    ko, vo = np.empty_like(keys), np.empty_like(vals)
    ms = ctypes.c_double()
    rc = lib().fcc_diag_radix_sort(keys.ctypes.data_as(ctypes.c_void_p), ctypes.c_int32(keys.dtype.itemsize),
                                   vals.ctypes.data_as(ctypes.c_void_p), ctypes.c_int32(vals.dtype.itemsize),
                                   ctypes.c_int64(keys.size), ctypes.c_int32(nbits), ctypes.c_int32(reps),
                                   ko.ctypes.data_as(ctypes.c_void_p), vo.ctypes.data_as(ctypes.c_void_p),
                                   ctypes.byref(ms))
    if rc != 0:
        raise FccError(rc, "fcc_diag_radix_sort failed")
    return ko, vo, ms.value


def fp64_fma_rate(device=0):
    """Measured FP64 FMA instructions per second of the device."""
    r = ctypes.c_double()
    rc = lib().fcc_diag_fp64_fma_rate(ctypes.c_int32(device), ctypes.byref(r))
    if rc != 0:
        raise FccError(rc, "fcc_diag_fp64_fma_rate failed")
    return r.value


# ----------------------------------------------------------- generator ----

def synth_coo(seed, extents, zipf_s=None, nnz=1000, lognormal=False):
    """Seeded distinct-coordinate COO tensor (include/fastcc_synth.h).
    Returns (coords (n, order) int32, values (n,) float64)."""
    extents = np.ascontiguousarray(extents, dtype=np.int64)
    order = extents.shape[0]
    zs = np.zeros(order) if zipf_s is None else np.broadcast_to(np.asarray(zipf_s, np.float64), (order,))
    zs = np.ascontiguousarray(zs, dtype=np.float64)
    coords = np.empty((nnz, order), np.int32)
    vals = np.empty(nnz, np.float64)
    got = ctypes.c_int64()
    rc = synth_lib().fcc_synth_coo(ctypes.c_uint64(seed), ctypes.c_int32(order),
                                   ctypes.c_void_p(extents.ctypes.data), ctypes.c_void_p(zs.ctypes.data),
                                   ctypes.c_int64(nnz), ctypes.c_int32(1 if lognormal else 0),
                                   ctypes.c_void_p(coords.ctypes.data), ctypes.c_void_p(vals.ctypes.data),
                                   ctypes.byref(got))
    if rc != 0:
        raise ValueError("fcc_synth_coo rejected the arguments")
    n = got.value
    return coords[:n], vals[:n]
