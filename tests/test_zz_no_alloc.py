"""The allocation-free modmul (heal_modmul_ttt_noalloc) against the regular
heal_modmul_ttt, through the C ABI.

It exists for callers that cannot let the library allocate device memory
(a process that reserves HBM up front, a host runtime that owns every device
buffer, a loop that must not stall in an allocator): its scratch is a fixed
device array of the library instead of pool memory.  This file is collected
last, so a failure here comes after every other test has run.  Its inputs
are torch tensors, and its first call happens before anything else has
initialised the backend, so it also covers a fresh process."""
import ctypes

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
