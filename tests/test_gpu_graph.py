"""CUDA graphs of HEAL calls (heal_graph_*): a captured round-trip step replays
bit-exact against the reference's hashes, a capture that would have to
build a table fails cleanly, and the backend keeps working afterwards."""
import hashlib

import numpy as np
import pytest

from heal_gb300 import capi
from heal_gb300.configs import RoundTripChain
from heal_gb300 import params as P
from _gpu import ready

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def gpu():
    return ready()


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_captured_roundtrip_step_matches_reference(golden_hash):
    h = golden_hash["roundtrip_n4096"]
    c = RoundTripChain()
    c.run()                      # builds every table the step needs
    for name in ("NA", "NB", "RA", "PR", "AS"):
        getattr(c, name).numpy()
    before = capi.launches()
    g = capi.Graph(c.run)
    assert capi.launches() == before          # recorded, not run
    # wipe the outputs, replay twice
    for name in ("NA", "NB", "RA", "PR", "AS"):
        arr = getattr(c, name)
        zeros = capi.DeviceArray.from_numpy(np.zeros(arr.shape, np.int64))
        capi.call("heal_copy_strided", zeros, arr)
    g.launch()
    g.launch()
    assert capi.launches() - before >= 10
    assert sha(c.NA.numpy()) == h["ntt_a"] and sha(c.NB.numpy()) == h["ntt_b"]
    assert sha(c.RA.numpy()) == h["intt_ntt_a"] and sha(c.PR.numpy()) == h["modmul"]
    assert sha(c.AS.numpy()) == h["axis_modsum"]


def test_capture_refuses_to_build_tables():
    qs = P.ntt_primes(2**30, 64, 2)
    p, perm, tw, itw, minv = P.ntt_tables(qs, 64)
    a = capi.DeviceArray.from_numpy(P.residues(5, (1, 64, 1, 2), qs))
    out = capi.DeviceArray.empty((1, 64, 1, 2), np.int64)
    dp, dperm, dtw = (capi.DeviceArray.from_numpy(x) for x in (p, perm, tw))
    with pytest.raises(RuntimeError, match="not cached"):
        capi.Graph(lambda: capi.call("heal_ntt", a, dp, dperm, dtw, None, None, out))
    # the backend still works, and the same call captures once its tables exist
    capi.call("heal_ntt", a, dp, dperm, dtw, None, None, out)
    want = out.numpy()
    g = capi.Graph(lambda: capi.call("heal_ntt", a, dp, dperm, dtw, None, None, out))
    capi.call("heal_copy_strided", capi.DeviceArray.from_numpy(np.zeros((1, 64, 1, 2), np.int64)), out)
    g.launch()
    assert np.array_equal(out.numpy(), want)
