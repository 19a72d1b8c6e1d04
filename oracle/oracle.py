"""ctypes wrapper of oracle/heal_oracle.c — the CPU checker (test infrastructure).

Arrays are numpy int32/int64 arrays of any strides (including the 0-stride
views np.broadcast_to makes); each call returns new arrays.  Status codes
raise the exception pybind11 maps HEAL's C++ exceptions to:
invalid_argument -> ValueError, out_of_range -> IndexError,
runtime_error -> RuntimeError.
"""
import ctypes
import os

import numpy as np

from . import build as _build

MAX_DIMS = 8
_DT = {np.dtype(np.int32): 0, np.dtype(np.int64): 1, np.dtype(np.float64): 2}


class Tensor(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("dtype", ctypes.c_int32), ("ndim", ctypes.c_int32),
                ("dims", ctypes.c_int64 * MAX_DIMS), ("strides", ctypes.c_int64 * MAX_DIMS)]


def _t(arr):
    if arr is None:
        return None
    d = Tensor()
    d.data = arr.ctypes.data if arr.size else None
    d.dtype = _DT[arr.dtype]
    d.ndim = arr.ndim
    for i in range(arr.ndim):
        d.dims[i] = arr.shape[i]
        d.strides[i] = arr.strides[i] // arr.itemsize
    return d


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        P = ctypes.POINTER(Tensor)
        I64 = ctypes.c_int64
        L.ora_last_error.restype = ctypes.c_char_p
        L.ora_ntt.argtypes = [P, P, P, P, P, ctypes.c_int]
        L.ora_intt.argtypes = [P, P, P, P, P, P, ctypes.c_int]
        L.ora_modop.argtypes = [ctypes.c_int, P, P, I64, P, I64, P]
        L.ora_mod.argtypes = [P, I64, P, I64, P]
        L.ora_axis_modsum.argtypes = [P, P, P, I64, ctypes.c_int]
        L.ora_g_decomposition.argtypes = [P, P, ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(I64)]
        L.ora_permute.argtypes = [P, P, P, I64, I64]
        L.ora_copy_strided.argtypes = [P, P]
        L.ora_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def set_threads(n: int) -> int:
    return lib().ora_set_threads(int(n))


def _check(rc):
    if rc:
        msg = lib().ora_last_error().decode()
        raise {1: ValueError, 2: IndexError}.get(rc, RuntimeError)(msg)


def _ref(t):
    return ctypes.byref(t) if t is not None else None


def _arr(x, dtype):
    return np.asarray(x, dtype=dtype)


def ntt(a, p, perm, tw, exact=True):
    """ntt<T> (example_impl/ntt_impl.cpp:69-116); a is [l, m, r, k]."""
    out = np.zeros(a.shape, a.dtype)
    ta, tp, tperm, ttw, to = _t(a), _t(_arr(p, a.dtype)), _t(_arr(perm, a.dtype)), _t(_arr(tw, a.dtype)), _t(out)
    _check(lib().ora_ntt(_ref(ta), _ref(tp), _ref(tperm), _ref(ttw), _ref(to), int(exact)))
    return out


def intt(a, p, perm, itw, minv, exact=True, result=None):
    """intt<T> (example_impl/ntt_impl.cpp:118-170); `result` supplies the
    prior contents the scatter leaves in place for a non-bijective perm."""
    out = np.zeros(a.shape, a.dtype) if result is None else np.array(result, dtype=a.dtype, copy=True)
    ts = [_t(a), _t(_arr(p, a.dtype)), _t(_arr(perm, a.dtype)), _t(_arr(itw, a.dtype)),
          _t(_arr(minv, a.dtype)), _t(out)]
    _check(lib().ora_intt(*[_ref(x) for x in ts], int(exact)))
    return out


def _modop(op, a, b, p, out_shape, dtype):
    out = np.zeros(out_shape, dtype)
    tb = _t(b) if isinstance(b, np.ndarray) else None
    tp = _t(p) if isinstance(p, np.ndarray) else None
    bs = 0 if tb is not None else int(b)
    ps = 0 if tp is not None else int(p)
    _check(lib().ora_modop(op, _ref(_t(a)), _ref(tb), bs, _ref(tp), ps, _ref(_t(out))))
    return out


def modmul(a, b, p, out_shape=None):
    """modmul_{ttt,ttc,tct,tcc} (example_impl/modop_impl.cpp:108-180,239)."""
    return _modop(0, a, b, p, out_shape or a.shape, a.dtype)


def modsum(a, b, p, out_shape=None):
    """modsum_{ttt,ttc,tct,tcc} (example_impl/modop_impl.cpp:108-180,238)."""
    return _modop(1, a, b, p, out_shape or a.shape, a.dtype)


def modneg(a, p, out_shape=None):
    """Extension: (p - a % p) % p in the double-width type."""
    return _modop(2, a, 0, p, out_shape or a.shape, a.dtype)


def mod(a, b, dtype=None, shape=None):
    """mod_{tt,tc,ct} (example_impl/modop_impl.cpp:188-235)."""
    ref = a if isinstance(a, np.ndarray) else b
    out = np.zeros(ref.shape, ref.dtype)
    ta = _t(a) if isinstance(a, np.ndarray) else None
    tb = _t(b) if isinstance(b, np.ndarray) else None
    _check(lib().ora_mod(_ref(ta), 0 if ta else int(a), _ref(tb), 0 if tb else int(b), _ref(_t(out))))
    return out


def axis_modsum(a, p, axis, exact=True):
    """axis_modsum<T> (example_impl/axis_modsum_impl.cpp:12-76)."""
    shape = tuple(d for i, d in enumerate(a.shape) if i != axis) if 0 <= axis < a.ndim else a.shape[:-1]
    out = np.zeros(shape, a.dtype)
    _check(lib().ora_axis_modsum(_ref(_t(a)), _ref(_t(_arr(p, a.dtype))), _ref(_t(out)), int(axis), int(exact)))
    return out


def g_decomposition(a, power, base_bits):
    """g_decomposition<T> (example_impl/g_decomposition_impl.cpp:10-67);
    returns (digits, number of elements whose residual exceeded capacity)."""
    out = np.zeros(a.shape + (power,), a.dtype)
    w = ctypes.c_int64(0)
    _check(lib().ora_g_decomposition(_ref(_t(a)), _ref(_t(out)), power, base_bits, ctypes.byref(w)))
    return out, w.value


def permute(a, perms, ew, pa):
    """permute<T> (example_impl/permute_impl.cpp:8-65)."""
    out = np.zeros(a.shape, a.dtype)
    _check(lib().ora_permute(_ref(_t(a)), _ref(_t(_arr(perms, a.dtype))), _ref(_t(out)), int(ew), int(pa)))
    return out


def contiguous(a):
    """The gather of make_contiguous (example_impl/contiguous_impl.cpp:31-40)."""
    out = np.zeros(a.shape, a.dtype)
    _check(lib().ora_copy_strided(_ref(_t(a)), _ref(_t(out))))
    return out
