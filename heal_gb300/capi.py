"""ctypes binding of the C ABI in include/heal_gb300.h.

This is the binding a Python host would add for the backend (the same calls
a cgo / JNI / N-API binding makes); the parity tests and bench.py drive the
GPU through it.  `DeviceArray` is a strided view of HBM owned by the
backend's allocator, the C-ABI counterpart of HEAL's DeviceTensor.
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libheal_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "heal_gb300.h")
MAX_DIMS = 8
DTYPES = {np.dtype(np.int32): 0, np.dtype(np.int64): 1, np.dtype(np.float64): 2}
NP_OF = {v: k for k, v in DTYPES.items()}


class Tensor(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("dtype", ctypes.c_int32), ("ndim", ctypes.c_int32),
                ("dims", ctypes.c_int64 * MAX_DIMS), ("strides", ctypes.c_int64 * MAX_DIMS)]


class NttJob(ctypes.Structure):
    """heal_ntt_job: one transform of a heal_ntt_batch call."""
    _fields_ = [("a", Tensor), ("p", Tensor), ("perm", Tensor), ("twiddles", Tensor), ("m_inv", Tensor),
                ("result", Tensor)]


class KeyswitchJob(ctypes.Structure):
    """heal_keyswitch_job: one fused keyswitch step of a heal_keyswitch_batch call."""
    _fields_ = [("ct", Tensor), ("p", Tensor), ("perm", Tensor), ("inv_twiddles", Tensor), ("m_inv", Tensor),
                ("x", Tensor), ("power", ctypes.c_int64), ("base_bits", ctypes.c_int64), ("p_digits", Tensor),
                ("twiddles_digits", Tensor), ("digits", Tensor), ("tail_a", Tensor), ("tail_b", Tensor),
                ("tail_axis", ctypes.c_int64), ("galois", Tensor), ("elementwise_axis", ctypes.c_int64),
                ("perm_axis", ctypes.c_int64), ("result", Tensor)]


_P = ctypes.POINTER(Tensor)
_I64, _U64, _I32, _VP, _SZ = ctypes.c_int64, ctypes.c_uint64, ctypes.c_int32, ctypes.c_void_p, ctypes.c_size_t
SIGNATURES = {
    "heal_init": ([ctypes.c_int], ctypes.c_int),
    "heal_last_error": ([], ctypes.c_char_p),
    "heal_synchronize": ([], ctypes.c_int),
    "heal_get_stream": ([], _VP),
    "heal_set_stream": ([_VP], ctypes.c_int),
    "heal_kernel_launch_count": ([], _U64),
    "heal_graph_begin": ([], ctypes.c_int),
    "heal_graph_end": ([ctypes.POINTER(_VP)], ctypes.c_int),
    "heal_graph_launch": ([_VP], ctypes.c_int),
    "heal_graph_destroy": ([_VP], ctypes.c_int),
    "heal_graph_fork": ([ctypes.c_int], ctypes.c_int),
    "heal_graph_branch": ([ctypes.c_int], ctypes.c_int),
    "heal_alloc": ([_SZ, ctypes.c_int, ctypes.POINTER(_VP)], ctypes.c_int),
    "heal_free": ([_VP], ctypes.c_int),
    "heal_h2d": ([_VP, _VP, _SZ], ctypes.c_int),
    "heal_d2h": ([_VP, _VP, _SZ], ctypes.c_int),
    "heal_h2d_async": ([_VP, _VP, _SZ], ctypes.c_int),
    "heal_d2h_async": ([_VP, _VP, _SZ], ctypes.c_int),
    "heal_host_alloc": ([_SZ, ctypes.POINTER(_VP)], ctypes.c_int),
    "heal_host_free": ([_VP], ctypes.c_int),
    "heal_base64_decode": ([_VP, _SZ, _VP, _SZ, ctypes.POINTER(_SZ), ctypes.c_int], ctypes.c_int),
    "heal_set_reference_compat": ([ctypes.c_int], ctypes.c_int),
    "heal_get_reference_compat": ([], ctypes.c_int),
    "heal_mark_modified": ([_VP], ctypes.c_int),
    "heal_copy_strided": ([_P, _P], ctypes.c_int),
    "heal_tensor_reshape": ([_P, _I32, ctypes.POINTER(_I64)], ctypes.c_int),
    "heal_tensor_expand": ([_P, _I64, _I64], ctypes.c_int),
    "heal_tensor_squeeze": ([_P, _I64], ctypes.c_int),
    "heal_tensor_unsqueeze": ([_P, _I64], ctypes.c_int),
    "heal_tensor_moveaxis": ([_P, _I64, _I64], ctypes.c_int),
    "heal_tensor_slice": ([_P, _I64, _I64, _I64, _I64], ctypes.c_int),
    "heal_tensor_is_contiguous": ([_P], ctypes.c_int),
    "heal_tensor_span": ([_P], _I64),
    "heal_modmul_ttt": ([_P, _P, _P, _P], ctypes.c_int),
    "heal_modmul_ttc": ([_P, _P, _I64, _P], ctypes.c_int),
    "heal_modmul_tct": ([_P, _I64, _P, _P], ctypes.c_int),
    "heal_modmul_tcc": ([_P, _I64, _I64, _P], ctypes.c_int),
    "heal_modsum_ttt": ([_P, _P, _P, _P], ctypes.c_int),
    "heal_modsum_ttc": ([_P, _P, _I64, _P], ctypes.c_int),
    "heal_modsum_tct": ([_P, _I64, _P, _P], ctypes.c_int),
    "heal_modsum_tcc": ([_P, _I64, _I64, _P], ctypes.c_int),
    "heal_modmul_ttt_noalloc": ([_P, _P, _P, _P, _VP], ctypes.c_int),
    "heal_mod_tt": ([_P, _P, _P], ctypes.c_int),
    "heal_mod_tc": ([_P, _I64, _P], ctypes.c_int),
    "heal_mod_ct": ([_I64, _P, _P], ctypes.c_int),
    "heal_modneg_tt": ([_P, _P, _P], ctypes.c_int),
    "heal_modneg_tc": ([_P, _I64, _P], ctypes.c_int),
    "heal_axis_modsum": ([_P, _P, _P, _I64], ctypes.c_int),
    "heal_g_decomposition": ([_P, _P, _U64, _U64], ctypes.c_int),
    "heal_ntt": ([_P, _P, _P, _P, _P, _P, _P], ctypes.c_int),
    "heal_intt": ([_P, _P, _P, _P, _P, _P, _P, _P], ctypes.c_int),
    "heal_permute": ([_P, _P, _P, _I64, _I64], ctypes.c_int),
    "heal_modmul_axis_sum": ([_P, _P, _P, _P, _I64, _P, _I64], ctypes.c_int),
    "heal_modmul_axis_sum_permute": ([_P, _P, _P, _I64, _P, _I64, _I64, _P], ctypes.c_int),
    "heal_g_decomposition_ntt": ([_P, _I64, _I64, _P, _P, _P, _P], ctypes.c_int),
    "heal_ntt_butterfly_peak": ([ctypes.c_int, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
    "heal_ntt_batch": ([ctypes.c_int, ctypes.POINTER(NttJob), _I64], ctypes.c_int),
    "heal_keyswitch_batch": ([ctypes.POINTER(KeyswitchJob), _I64], ctypes.c_int),
    "heal_keyswitch_batch_test_wait": ([ctypes.c_uint32, ctypes.c_int], ctypes.c_int),
    "heal_ntt_set_plan": ([ctypes.c_int, ctypes.c_int, _I64, _I64, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "heal_ntt_get_plan": ([ctypes.c_int, ctypes.c_int, _I64, _I64, ctypes.POINTER(ctypes.c_int),
                           ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    "heal_ntt_clear_plans": ([], ctypes.c_int),
    "heal_ntt_autotune": ([ctypes.c_int, _P, _P, _P, _P, _P, _P, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                           ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
}


def declared_symbols(header: str = HEADER) -> list[str]:
    """Names of the functions include/heal_gb300.h declares."""
    text = open(header).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*|void \*|uint64_t|int64_t)\s*\*?(heal_\w+)\(",
                                 text, re.M)))


_lib = None


def lib():
    """The loaded C ABI; raises if the CUDA extension has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build the backend first (heal_gb300.build())")
        L = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


class HealError(RuntimeError):
    pass


_EXC = {1: ValueError, 2: IndexError, 3: RuntimeError, 4: MemoryError, 5: RuntimeError}


def check(rc: int):
    if rc:
        raise _EXC.get(rc, HealError)(lib().heal_last_error().decode())


def desc(data, dtype, shape, strides) -> Tensor:
    t = Tensor()
    t.data = data
    t.dtype = DTYPES[np.dtype(dtype)]
    t.ndim = len(shape)
    for i in range(MAX_DIMS):
        t.dims[i] = shape[i] if i < len(shape) else 1
        t.strides[i] = strides[i] if i < len(shape) else 0
    return t


def _rowmajor(shape):
    s, out = 1, []
    for d in reversed(shape):
        out.append(s)
        s *= d
    return tuple(reversed(out))


class Buffer:
    """One heal_alloc allocation, freed when the last view drops it."""

    def __init__(self, nbytes: int, zero: bool = True):
        self.ptr = ctypes.c_void_p()
        self.nbytes = nbytes
        if nbytes:
            check(lib().heal_alloc(nbytes, 1 if zero else 0, ctypes.byref(self.ptr)))

    def __del__(self):
        if self.ptr and self.ptr.value and _lib is not None:
            _lib.heal_free(self.ptr)
            self.ptr = ctypes.c_void_p()


class DeviceArray:
    """A strided view (shape, strides in elements, byte offset) of a Buffer."""

    def __init__(self, buf: Buffer, dtype, shape, strides=None, offset: int = 0):
        self.buf = buf
        self.dtype = np.dtype(dtype)
        self.shape = tuple(int(s) for s in shape)
        self.strides = tuple(int(s) for s in (strides if strides is not None else _rowmajor(self.shape)))
        self.offset = offset

    # ---- construction
    @classmethod
    def empty(cls, shape, dtype, zero: bool = True) -> "DeviceArray":
        n = int(np.prod(shape)) if len(shape) else 1
        return cls(Buffer(n * np.dtype(dtype).itemsize, zero), dtype, shape)

    @classmethod
    def from_numpy(cls, arr: np.ndarray) -> "DeviceArray":
        """Upload keeping the array's strides, as HEAL's host_to_device does."""
        arr = np.asarray(arr)
        if arr.dtype not in DTYPES:
            raise TypeError(f"unsupported dtype {arr.dtype}")
        st = tuple(s // arr.itemsize for s in arr.strides)
        if any(s < 0 for s in st):
            arr = np.ascontiguousarray(arr)
            st = tuple(s // arr.itemsize for s in arr.strides)
        span = 0 if arr.size == 0 else 1 + sum((d - 1) * s for d, s in zip(arr.shape, st))
        buf = Buffer(span * arr.itemsize, zero=False)
        if span:
            check(lib().heal_h2d(buf.ptr, ctypes.c_void_p(arr.ctypes.data), span * arr.itemsize))
        return cls(buf, arr.dtype, arr.shape, st)

    # ---- access
    @property
    def ptr(self) -> int:
        return (self.buf.ptr.value or 0) + self.offset

    @property
    def size(self) -> int:
        return int(np.prod(self.shape)) if self.shape else 1

    def desc(self) -> Tensor:
        """A new descriptor of the view (the caller may edit it)."""
        return desc(self.ptr if self.buf.ptr.value else None, self.dtype, self.shape, self.strides)

    def cdesc(self) -> Tensor:
        """The view's descriptor, built on first use and shared by every call
        that only reads it (a view never changes after construction)."""
        d = self.__dict__.get("_cdesc")
        if d is None:
            d = self._cdesc = self.desc()
        return d

    def numpy(self) -> np.ndarray:
        n = self.size
        if n == 0:
            check(lib().heal_synchronize())
            return np.zeros(self.shape, self.dtype)
        span = 1 + sum((d - 1) * s for d, s in zip(self.shape, self.strides))
        host = np.empty(span, self.dtype)
        check(lib().heal_d2h(ctypes.c_void_p(host.ctypes.data), ctypes.c_void_p(self.ptr), span * self.dtype.itemsize))
        view = np.lib.stride_tricks.as_strided(host, self.shape, [s * self.dtype.itemsize for s in self.strides])
        return np.array(view)

    def _meta(self, fn, *args) -> "DeviceArray":
        d = self.desc()
        check(fn(ctypes.byref(d), *args))
        nd = d.ndim
        off = (d.data or 0) - (self.buf.ptr.value or 0) if d.data else self.offset
        return DeviceArray(self.buf, self.dtype, list(d.dims)[:nd], list(d.strides)[:nd], off)

    def reshape(self, shape) -> "DeviceArray":
        arr = (_I64 * len(shape))(*shape)
        return self._meta(lib().heal_tensor_reshape, len(shape), arr)

    def moveaxis(self, src: int, dst: int) -> "DeviceArray":
        return self._meta(lib().heal_tensor_moveaxis, src, dst)

    def expand(self, axis: int, repeats: int) -> "DeviceArray":
        return self._meta(lib().heal_tensor_expand, axis, repeats)


def _arg(x):
    if x is None:
        return None
    if isinstance(x, DeviceArray):
        return ctypes.byref(x.cdesc())
    return x


def call(name: str, *args):
    """Calls C-ABI function `name`, passing DeviceArrays as descriptors."""
    check(getattr(lib(), name)(*[_arg(a) for a in args]))


def ntt_jobs(jobs) -> "ctypes.Array":
    """heal_ntt_job array from (a, p, perm, twiddles, m_inv or None, result)
    DeviceArrays; the caller keeps the arrays alive while it is used."""
    arr = (NttJob * max(1, len(jobs)))()
    for i, (a, p, perm, tw, minv, res) in enumerate(jobs):
        arr[i].a, arr[i].p, arr[i].perm, arr[i].twiddles = a.desc(), p.desc(), perm.desc(), tw.desc()
        if minv is not None:
            arr[i].m_inv = minv.desc()
        arr[i].result = res.desc()
    return arr


def ntt_batch(inverse: bool, jobs):
    """heal_ntt_batch over (a, p, perm, twiddles, m_inv or None, result) tuples."""
    check(lib().heal_ntt_batch(int(bool(inverse)), ntt_jobs(jobs), len(jobs)))


def keyswitch_jobs(jobs) -> "ctypes.Array":
    """heal_keyswitch_job array from dicts of DeviceArrays and integers keyed
    by the struct's field names; the caller keeps the arrays alive."""
    arr = (KeyswitchJob * max(1, len(jobs)))()
    for i, j in enumerate(jobs):
        for name, _ in KeyswitchJob._fields_:
            v = j[name]
            setattr(arr[i], name, v.desc() if isinstance(v, DeviceArray) else int(v))
    return arr


def keyswitch_batch(jobs):
    """heal_keyswitch_batch over keyswitch job dicts (see keyswitch_jobs)."""
    check(lib().heal_keyswitch_batch(keyswitch_jobs(jobs), len(jobs)))


def synchronize():
    check(lib().heal_synchronize())


def launches() -> int:
    return int(lib().heal_kernel_launch_count())


def stream() -> int:
    return int(lib().heal_get_stream() or 0)


class Graph:
    """A captured sequence of C-ABI calls, replayed with one launch."""

    def __init__(self, record, branches: int = 0):
        """`record()` issues the calls to capture; run it once uncaptured
        first so that every table it needs is cached.  With `branches` > 0
        the capture forks that many parallel branch streams first and
        `record(branch)` gets a function that sends the following calls to
        branch i (-1: the capture's own stream)."""
        check(lib().heal_graph_begin())
        try:
            if branches:
                check(lib().heal_graph_fork(branches))
                record(lambda i: check(lib().heal_graph_branch(i)))
            else:
                record()
        except BaseException:
            h = ctypes.c_void_p()
            lib().heal_graph_end(ctypes.byref(h))
            if h.value:
                lib().heal_graph_destroy(h)
            raise
        self.handle = ctypes.c_void_p()
        check(lib().heal_graph_end(ctypes.byref(self.handle)))

    def launch(self):
        check(lib().heal_graph_launch(self.handle))

    def __del__(self):
        if getattr(self, "handle", None) is not None and self.handle.value and _lib is not None:
            _lib.heal_graph_destroy(self.handle)
            self.handle = ctypes.c_void_p()


def autotune_ntt(inverse: bool, a, p, perm, tw, minv, out, reps: int = 5) -> tuple[int, int]:
    """Runs heal_ntt_autotune on these operands (`out` is overwritten) and
    returns the chosen (tile_limbs, first_pass_log2)."""
    c, s = ctypes.c_int(), ctypes.c_int()
    check(lib().heal_ntt_autotune(int(inverse), _arg(a), _arg(p), _arg(perm), _arg(tw), _arg(minv), _arg(out),
                                  reps, ctypes.byref(c), ctypes.byref(s)))
    return c.value, s.value


def ntt_plan(dtype, inverse: bool, m: int, k: int) -> tuple[int, int]:
    c, s = ctypes.c_int(), ctypes.c_int()
    check(lib().heal_ntt_get_plan(DTYPES[np.dtype(dtype)], int(inverse), m, k, ctypes.byref(c), ctypes.byref(s)))
    return c.value, s.value
