"""Calls on several streams: tables derived on one stream are safe to use
at once on another, and two keyswitch chains alternating between two streams
(the benchmark's configuration) give the single-stream results."""
import numpy as np
import pytest

from heal_gb300 import capi
from heal_gb300 import params as P
from heal_gb300.chain import KeyswitchChain
from oracle import oracle as O
from _gpu import ready, up

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def gpu():
    return ready()


def test_tables_built_on_one_stream_used_on_another():
    import torch
    side = torch.cuda.Stream()
    lib = capi.lib()
    for trial in range(3):
        n, k = 1 << 14, 16
        qs = P.ntt_primes(1 << 50, n, k)
        p, perm, tw, itw, minv = P.ntt_tables(qs, n)
        x = P.residues(40 + trial, (2, n, 1, k), qs)
        dx, dp, dperm, dtw = (up(v) for v in (x, p, perm, tw))     # fresh tensors: no cached tables
        o1, o2 = capi.DeviceArray.empty(x.shape, np.int64), capi.DeviceArray.empty(x.shape, np.int64)
        capi.check(lib.heal_set_stream(side.cuda_stream))
        capi.call("heal_ntt", dx, dp, dperm, dtw, None, None, o1)      # builds the tables on `side`
        capi.check(lib.heal_set_stream(None))
        capi.call("heal_ntt", dx, dp, dperm, dtw, None, None, o2)      # uses them on the library stream at once
        torch.cuda.synchronize()
        want = O.ntt(x, p, perm, tw)
        assert np.array_equal(o1.numpy(), want) and np.array_equal(o2.numpy(), want)


def test_two_chains_on_two_streams_match_one_stream():
    import torch
    ch = KeyswitchChain(n=1 << 12, limbs=6, digits=3, base_bits=17, bound_bits=50)
    twin = ch.twin()
    side = torch.cuda.Stream()
    lib = capi.lib()
    cts = [up(P.residues(500 + i, ch.shape(), ch.qs)) for i in range(6)]
    ref = [capi.DeviceArray.empty(ch.shape(), np.int64) for _ in cts]
    got = [capi.DeviceArray.empty(ch.shape(), np.int64) for _ in cts]
    for c, r in zip(cts, ref):
        ch.run(c, r)
    capi.synchronize()
    for i, (c, g) in enumerate(zip(cts, got)):
        if i % 2:
            capi.check(lib.heal_set_stream(side.cuda_stream))
            twin.run(c, g)
            capi.check(lib.heal_set_stream(None))
        else:
            ch.run(c, g)
    torch.cuda.synchronize()
    for r, g in zip(ref, got):
        assert np.array_equal(r.numpy(), g.numpy())
