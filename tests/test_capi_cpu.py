"""CPU-only checks of the C ABI: the library loads and exports every symbol
include/heal_gb300.h declares, the `lattica_hw` module exposes HEAL's names,
and the stride-only metadata edits follow DeviceTensor::reshape and the
virtual ops of example_impl (no device memory is touched)."""
import ctypes

import numpy as np
import pytest

import heal_gb300
from heal_gb300 import capi


@pytest.fixture(scope="module", autouse=True)
def built():
    heal_gb300.build()


def test_exports_every_declared_symbol():
    names = capi.declared_symbols()
    assert len(names) >= 40
    L = ctypes.CDLL(capi.LIB_PATH)
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) == set(capi.SIGNATURES), set(names) ^ set(capi.SIGNATURES)


def test_lattica_hw_module_names():
    m = heal_gb300.lattica_hw()
    # every name HEAL's example_impl/py_bindings.cpp:87-133 binds
    names = ["DeviceTensor32", "DeviceTensor64", "DeviceTensorfloat64", "axis_modsum_32", "axis_modsum_64",
             "ntt_32", "ntt_64", "intt_32", "intt_64", "permute_32", "permute_64"]
    for sfx in ("32", "64", "float64"):
        names += [f"{n}_{sfx}" for n in ("allocate_on_hardware", "host_to_device", "device_to_host", "expand",
                                          "squeeze", "unsqueeze", "make_contiguous")]
    for sfx in ("32", "64"):
        names += [f"{op}_{v}_{sfx}" for op in ("modmul", "modsum") for v in ("ttt", "ttc", "tct", "tcc")]
        names += [f"g_decomposition_{sfx}"]
    missing = [n for n in names if not hasattr(m, n)]
    assert not missing, missing
    for cls in ("DeviceTensor32", "DeviceTensor64", "DeviceTensorfloat64"):
        for meth in ("print", "print_metadata", "reshape"):
            assert hasattr(getattr(m, cls), meth)


def t(shape, strides=None, dtype=np.int64):
    st = strides or capi._rowmajor(shape)
    return capi.desc(None, dtype, shape, st)


def dims(d):
    return list(d.dims)[:d.ndim], list(d.strides)[:d.ndim]


def test_reshape_rules():
    L = capi.lib()
    d = t((2, 2, 3))
    nd = (ctypes.c_int64 * 2)(6, 2)
    assert L.heal_tensor_reshape(ctypes.byref(d), 2, nd) == 0
    assert dims(d) == ([6, 2], [2, 1])
    bad = (ctypes.c_int64 * 2)(5, 2)
    assert L.heal_tensor_reshape(ctypes.byref(d), 2, bad) == 1
    assert b"Total size of new shape" in L.heal_last_error()
    # a broadcast (stride-0) axis does not count (device_memory_impl.cpp:45-50)
    e = t((3, 4), (0, 1))
    four = (ctypes.c_int64 * 1)(4)
    assert L.heal_tensor_reshape(ctypes.byref(e), 1, four) == 0
    assert dims(e) == ([4], [1])


def test_virtual_ops():
    L = capi.lib()
    d = t((1, 1, 3))
    assert L.heal_tensor_squeeze(ctypes.byref(d), 1) == 0 and dims(d) == ([1, 3], [3, 1])
    assert L.heal_tensor_squeeze(ctypes.byref(d), 1) == 1   # size 3: invalid_argument
    d = t((2, 2))
    assert L.heal_tensor_unsqueeze(ctypes.byref(d), -1) == 0 and dims(d) == ([2, 2, 1], [2, 1, 0])
    d = t((2, 3))
    assert L.heal_tensor_unsqueeze(ctypes.byref(d), 4) == 1
    assert L.heal_tensor_unsqueeze(ctypes.byref(d), -4) == 1
    d = t((2, 1))
    assert L.heal_tensor_expand(ctypes.byref(d), 1, 3) == 0 and dims(d) == ([2, 3], [1, 0])
    assert L.heal_tensor_expand(ctypes.byref(d), 1, 3) == 1  # not size 1
    assert L.heal_tensor_expand(ctypes.byref(d), 0, 0) == 1  # repeats <= 0
    d = t((2, 3, 4))
    assert L.heal_tensor_moveaxis(ctypes.byref(d), 2, 0) == 0 and dims(d) == ([4, 2, 3], [1, 12, 4])
    d = t((5, 6))
    assert L.heal_tensor_slice(ctypes.byref(d), 1, 1, 5, 2) == 0 and dims(d) == ([5, 2], [6, 2])


def test_contiguity_and_span():
    L = capi.lib()
    assert L.heal_tensor_is_contiguous(ctypes.byref(t((3, 4)))) == 1
    assert L.heal_tensor_is_contiguous(ctypes.byref(t((4, 3), (1, 4)))) == 0
    assert L.heal_tensor_is_contiguous(ctypes.byref(t((3, 1, 4), (4, 99, 1)))) == 1  # size-1 axes skipped
    assert L.heal_tensor_span(ctypes.byref(t((4, 3), (1, 4)))) == 12
    assert L.heal_tensor_span(ctypes.byref(t((3, 4), (0, 1)))) == 4
    assert L.heal_tensor_span(ctypes.byref(t((0, 4)))) == 0


def test_ntt_plan_table_host_side():
    L = capi.lib()
    I64, I32 = capi.DTYPES[np.dtype(np.int64)], capi.DTYPES[np.dtype(np.int32)]
    try:
        assert capi.ntt_plan(np.int64, False, 1 << 16, 24) == (4, 8)     # default: even split
        assert capi.ntt_plan(np.int32, True, 1 << 12, 4) == (4, 0)       # one pass
        capi.check(L.heal_ntt_set_plan(I64, 0, 1 << 16, 24, 8, 6))
        assert capi.ntt_plan(np.int64, False, 1 << 16, 24) == (8, 6)
        assert capi.ntt_plan(np.int64, True, 1 << 16, 24) == (4, 8)       # per direction
        assert capi.ntt_plan(np.int64, False, 1 << 16, 23) == (4, 8)      # per limb count
        bad = [(I64, 0, 1 << 16, 24, 3, 8),      # tile width not a power of two
               (I64, 0, 1 << 16, 24, 32, 8),     # too wide
               (I64, 0, 1 << 16, 24, 4, 0),      # one pass above 4096 points
               (I64, 0, 1 << 16, 24, 4, 3),      # second pass of 13 stages
               (I64, 0, 1 << 16, 24, 4, 16),     # empty second pass
               (I32, 0, 3000, 4, 4, 0),          # not a power of two
               (2, 0, 1 << 10, 4, 4, 0),         # float64
               (I64, 2, 1 << 10, 4, 4, 0),       # direction
               (I64, 0, 1 << 10, 0, 4, 0)]       # no limbs
        for args in bad:
            assert L.heal_ntt_set_plan(*args) == 1, args
            assert L.heal_last_error()
    finally:
        capi.check(L.heal_ntt_clear_plans())
    assert capi.ntt_plan(np.int64, False, 1 << 16, 24) == (4, 8)


def test_header_is_plain_c(tmp_path):
    """include/heal_gb300.h compiles as C11 on its own (the header a cgo,
    JNI or N-API binding includes), with every declared entry point callable
    from C: a C program that takes the address of each links against the
    library."""
    import os
    import subprocess
    names = capi.declared_symbols()
    src = tmp_path / "use_header.c"
    table = "".join(f"  (void (*)(void))&{n},\n" for n in names)
    src.write_text('#include "heal_gb300.h"\n#include <stdio.h>\n'
                   f"static void (*const entry[])(void) = {{\n{table}}};\n"
                   'int main(void) {\n  printf("%zu\\n", sizeof entry / sizeof entry[0]);\n'
                   "  return entry[0] == 0;\n}\n")
    inc = os.path.dirname(capi.HEADER)
    lib_dir = os.path.dirname(capi.LIB_PATH)
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", inc, str(src),
                    "-o", str(tmp_path / "use_header"), "-L", lib_dir, "-lheal_gb300",
                    f"-Wl,-rpath,{lib_dir}"], check=True)
    run = subprocess.run([str(tmp_path / "use_header")], capture_output=True, text=True, check=True)
    assert int(run.stdout) == len(names)


def test_reference_compat_switch_is_host_state():
    """heal_set_reference_compat only sets a process-wide flag (no GPU
    call): off by default, on and off again as asked."""
    L = capi.lib()
    assert L.heal_get_reference_compat() == 0
    try:
        assert L.heal_set_reference_compat(7) == 0 and L.heal_get_reference_compat() == 1
    finally:
        assert L.heal_set_reference_compat(0) == 0
    assert L.heal_get_reference_compat() == 0
