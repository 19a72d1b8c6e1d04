"""The allocation-free modmul (heal_modmul_ttt_noalloc) against the regular
heal_modmul_ttt, through the C ABI.

It exists for callers that cannot let the library allocate device memory
(a process that reserves HBM up front, a host runtime that owns every device
buffer, a loop that must not stall in an allocator): its scratch is a fixed
device array of the library instead of pool memory.  This file is collected
last, so a failure here comes after every other test has run.  Its inputs
are torch tensors.  Because the other GPU tests have initialised the backend
by the time these run, one test repeats the check in a fresh child process
whose first library call is the allocation-free one."""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

import heal_gb300
from heal_gb300 import capi
from heal_gb300 import params as P

pytestmark = pytest.mark.gpu


def desc_of(t: torch.Tensor):
    dt = {torch.int32: np.int32, torch.int64: np.int64}[t.dtype]
    return capi.desc(t.data_ptr(), dt, tuple(t.shape), tuple(t.stride()))


def noalloc(a, b, p, out, stream):
    da, db, dp, do = desc_of(a), desc_of(b), desc_of(p), desc_of(out)
    capi.check(capi.lib().heal_modmul_ttt_noalloc(ctypes.byref(da), ctypes.byref(db), ctypes.byref(dp),
                                                  ctypes.byref(do), ctypes.c_void_p(stream)))


def regular(a, b, p, out):
    torch.cuda.synchronize()   # torch's stream filled `out`; the backend runs on its own stream
    da, db, dp, do = desc_of(a), desc_of(b), desc_of(p), desc_of(out)
    capi.check(capi.lib().heal_modmul_ttt(ctypes.byref(da), ctypes.byref(db), ctypes.byref(dp), ctypes.byref(do)))
    capi.synchronize()


@pytest.mark.parametrize("dtype,bound", [(torch.int64, 2**50), (torch.int32, 2**30)])
def test_noalloc_matches_modmul_ttt_twice(dtype, bound):
    heal_gb300.build()
    assert torch.cuda.is_available(), "needs a CUDA GPU"
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev).cuda_stream
    npdt = np.int64 if dtype == torch.int64 else np.int32
    # two calls in a row with different moduli and shapes: the second must
    # overwrite the constants the first left in the shared array
    cases = [((2, 4096, 1, 24), P.ntt_primes(bound, 4096, 24)),
             ((3, 1000, 7), P.ntt_primes(bound // 2, 8, 7))]
    for i, (shape, qs) in enumerate(cases):
        qs = np.array(qs, npdt)
        a = torch.from_numpy(P.residues(10 + i, shape, qs, npdt)).to(dev)
        b = torch.from_numpy(P.residues(20 + i, shape, qs, npdt)).to(dev)
        p = torch.from_numpy(qs).to(dev)
        got = torch.zeros(shape, dtype=dtype, device=dev)
        noalloc(a, b, p, got, stream)
        torch.cuda.synchronize()
        want = torch.zeros(shape, dtype=dtype, device=dev)
        regular(a, b, p, want)
        assert torch.equal(got, want), f"call {i}"
        # the product itself, checked independently in Python integers
        ref = (a.cpu().numpy().astype(object) * b.cpu().numpy().astype(object)) % qs.astype(object)
        assert np.array_equal(got.cpu().numpy(), ref.astype(npdt))


def test_noalloc_rejects_too_many_moduli():
    dev = torch.device("cuda:0")
    qs = torch.full((4097,), 97, dtype=torch.int64, device=dev)
    a = torch.ones((2, 4097), dtype=torch.int64, device=dev)
    out = torch.zeros_like(a)
    with pytest.raises(ValueError, match="at most 4096"):
        noalloc(a, a, qs, out, torch.cuda.current_stream(dev).cuda_stream)


def python_product(a, b, qs):
    """a * b mod p broadcast like modmul (p along the last axes), in Python integers."""
    return (a.astype(object) * b.astype(object)) % qs.astype(object)


@pytest.mark.parametrize("dtype,bound", [(torch.int64, 2**50), (torch.int32, 2**30)])
def test_noalloc_broadcast_and_strided_operands(dtype, bound):
    """Operands that take the general (strided) kernel with the fixed table:
    a broadcast along the first axis, a 2-D p, a transposed result, and a p
    whose leading axis has size 1; each against heal_modmul_ttt and the
    product in Python integers, two calls in a row."""
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev).cuda_stream
    npdt = np.int64 if dtype == torch.int64 else np.int32
    m, k, L = 5, 33, 7
    qs = np.array(P.ntt_primes(bound, 8, L), npdt)
    p2 = np.ascontiguousarray(np.broadcast_to(qs, (k, L)))
    # 1: a [1, k, L] broadcast over m, p [k, L], result [m, k, L] dense
    a1 = P.residues(31, (1, k, L), qs, npdt)
    b1 = P.residues(32, (m, k, L), qs, npdt)
    # 2: result [k, L] as the transpose of an [L, k] buffer, a and b dense, p [1, L]
    a2 = P.residues(33, (k, L), qs, npdt)
    b2 = P.residues(34, (k, L), qs, npdt)
    cases = [(a1, b1, p2, lambda: torch.zeros((m, k, L), dtype=dtype, device=dev)),
             (a2, b2, qs.reshape(1, L), lambda: torch.zeros((L, k), dtype=dtype, device=dev).t())]
    for i, (a, b, pp, make_out) in enumerate(cases):
        ta, tb, tp = (torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in (a, b, pp))
        got = make_out()
        noalloc(ta, tb, tp, got, stream)
        torch.cuda.synchronize()
        want = make_out()
        regular(ta, tb, tp, want)
        assert torch.equal(got, want), f"case {i}"
        ref = python_product(np.broadcast_to(a, got.shape), b, np.broadcast_to(pp, got.shape))
        assert np.array_equal(got.cpu().numpy(), ref.astype(npdt)), f"case {i}"


CHILD = r"""
import ctypes, sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
from heal_gb300 import capi
from heal_gb300 import params as P
dev = torch.device("cuda:0")
qs = np.array(P.ntt_primes(2**50, 4096, 12), np.int64)
out = []
for i in range(2):
    a = torch.from_numpy(P.residues(50 + i, (2, 4096, 1, 12), qs)).to(dev)
    b = torch.from_numpy(P.residues(60 + i, (2, 4096, 1, 12), qs)).to(dev)
    p = torch.from_numpy(qs).to(dev)
    got = torch.zeros_like(a)
    d = lambda t: capi.desc(t.data_ptr(), np.int64, tuple(t.shape), tuple(t.stride()))
    da, db, dp, do = d(a), d(b), d(p), d(got)
    capi.check(capi.lib().heal_modmul_ttt_noalloc(ctypes.byref(da), ctypes.byref(db), ctypes.byref(dp),
                                                  ctypes.byref(do), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()
    want = (a.cpu().numpy().astype(object) * b.cpu().numpy().astype(object)) % qs.astype(object)
    assert np.array_equal(got.cpu().numpy(), want.astype(np.int64)), i
print("noalloc-first-call-ok")
"""


def test_noalloc_first_call_in_a_fresh_process():
    """The first library call of a new process is the allocation-free one
    (its set-up looks the array's address up on that first call)."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", CHILD, root], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "noalloc-first-call-ok" in r.stdout, r.stdout + r.stderr
