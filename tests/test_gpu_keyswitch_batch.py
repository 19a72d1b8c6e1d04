"""heal_keyswitch_batch: many fused keyswitch steps of mixed ring degree and
limb count in one persistent launch, bit-identical to the same three calls
(intt, g_decomposition_ntt, modmul_axis_sum_permute) made ciphertext after
ciphertext, and to the oracle's chain."""
import numpy as np
import pytest

from heal_gb300 import capi
from heal_gb300 import params as P
from heal_gb300.configs import RaggedKeyswitch
from oracle.chain import oracle_chain
from _gpu import ready

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def gpu():
    return ready()


@pytest.fixture(scope="module")
def ragged():
    # every ring degree (passes of 2^6, 2^7 and 2^8 points), limb counts 2..9
    return RaggedKeyswitch(count=14, lmin=2, lmax=9, seed=31)


def per_call(rk):
    outs = []
    for i in range(len(rk.specs)):
        rk.run_calls(i)
        outs.append(rk.outs[i].numpy())
    return outs


def clear(rk):
    for o in rk.outs:
        capi.call("heal_copy_strided", capi.DeviceArray.from_numpy(np.zeros(o.shape, np.int64)), o)


def test_batch_equals_calls_and_oracle(ragged):
    rk = ragged
    assert {n for n, _ in rk.specs} == {1 << 12, 1 << 13, 1 << 14, 1 << 15, 1 << 16}
    want = per_call(rk)
    for rep in range(2):  # two launches in a row: the counters start from zero each time
        clear(rk)
        rk.run_batched()
        capi.synchronize()
        for i, w in enumerate(want):
            assert np.array_equal(rk.outs[i].numpy(), w), (rep, i, rk.specs[i])
    # the oracle on the two smallest ciphertexts
    for i in sorted(range(len(rk.specs)), key=lambda i: rk.specs[i][0] * rk.specs[i][1])[:2]:
        got = rk.outs[i].numpy()
        assert np.array_equal(got, oracle_chain(rk.host_tables(i), rk.host_cts[i], rk.D, rk.BITS)), rk.specs[i]


def test_batch_with_negative_values_takes_the_exact_path():
    rk = RaggedKeyswitch(count=4, logns=(12, 13), lmin=2, lmax=4, seed=5)
    ct = rk.host_cts[1].copy()
    ct[0, 17, 0, 1] = -3   # a negative residue: that INTT tile runs the reference's arithmetic
    capi.call("heal_copy_strided", capi.DeviceArray.from_numpy(ct), rk.cts[1])
    rk.host_cts[1] = ct
    want = per_call(rk)
    clear(rk)
    rk.run_batched()
    for i, w in enumerate(want):
        assert np.array_equal(rk.outs[i].numpy(), w), i
    assert np.array_equal(want[1], oracle_chain(rk.host_tables(1), ct, rk.D, rk.BITS))


def test_batch_argument_errors_write_nothing():
    rk = RaggedKeyswitch(count=3, logns=(12,), lmin=2, lmax=3, seed=9)
    clear(rk)
    jobs = [dict(j) for j in rk.jobs]
    # a ring degree below 2^12
    small = capi.DeviceArray.from_numpy(P.residues(1, (2, 2048, 1, 2), rk.qs[4096][:2]))
    bad = dict(jobs[2], ct=small)
    with pytest.raises(ValueError, match="job 2"):
        capi.keyswitch_batch(jobs[:2] + [bad])
    # two jobs writing the same result
    with pytest.raises(ValueError, match="writes memory"):
        capi.keyswitch_batch([jobs[0], dict(jobs[1], result=jobs[0]["result"])])
    # more jobs than one call takes
    with pytest.raises(ValueError, match="256"):
        capi.check(capi.lib().heal_keyswitch_batch(capi.keyswitch_jobs(jobs), 257))
    for o in rk.outs:
        assert not o.numpy().any()
    capi.keyswitch_batch([])  # nothing to do


def test_wait_that_runs_out_is_reported_and_the_context_stays_usable():
    """Failure path: with the test hook every tail waits for a tile that never
    comes; the waits give up after their limit (here 2^15 polls, ~10 ms), the
    kernel ends, heal_synchronize reports the timeout, and the next batch
    runs normally on the same context."""
    rk = RaggedKeyswitch(count=3, logns=(12,), lmin=2, lmax=3, seed=11)
    want = per_call(rk)
    lib = capi.lib()
    capi.check(lib.heal_keyswitch_batch_test_wait(1 << 15, 1))
    try:
        clear(rk)
        rk.run_batched()
        with pytest.raises(RuntimeError, match="ran out"):
            capi.synchronize()
    finally:
        capi.check(lib.heal_keyswitch_batch_test_wait(1 << 22, 0))
    capi.synchronize()  # the report was consumed
    clear(rk)
    rk.run_batched()
    for i, w in enumerate(want):
        assert np.array_equal(rk.outs[i].numpy(), w), i
