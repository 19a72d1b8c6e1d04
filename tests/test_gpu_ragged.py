"""Ragged batches and NTT plans.

A reduced ragged batch (the shape family of the 256-ciphertext benchmark:
ring degrees and limb counts differ per ciphertext) runs the five-call chain
ntt(A), ntt(B), intt(ntt(A)), modmul, axis_modsum per ciphertext, as a plain
loop and as one CUDA graph with parallel branches; every output equals the
oracle's.  Every NTT plan (tile width, two-pass split) gives the oracle's
result, and the autotuner keeps a valid plan."""
import numpy as np
import pytest

from heal_gb300 import capi
from heal_gb300 import params as P
from heal_gb300.configs import RaggedBatch
from oracle import oracle as O
from _gpu import ready, up

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def gpu():
    return ready()


def zero(arr):
    capi.call("heal_copy_strided", capi.DeviceArray.from_numpy(np.zeros(arr.shape, arr.dtype)), arr)


def check_against_oracle(c, i):
    n, l = c.specs[i]
    qs = c.qs[n][:l]
    p, perm, tw, itw, minv = P.ntt_tables(qs, n)
    a, b = c.A[i].numpy(), c.B[i].numpy()
    na, nb = O.ntt(a, p, perm, tw), O.ntt(b, p, perm, tw)
    assert np.array_equal(c.NA[i].numpy(), na), (i, n, l)
    assert np.array_equal(c.NB[i].numpy(), nb), (i, n, l)
    assert np.array_equal(c.RA[i].numpy(), a), (i, n, l)          # round trip
    assert np.array_equal(c.RA[i].numpy(), O.intt(na, p, perm, itw, minv)), (i, n, l)
    pr = O.modmul(na, nb, p)
    assert np.array_equal(c.PR[i].numpy(), pr), (i, n, l)
    assert np.array_equal(c.AS[i].numpy(), O.axis_modsum(pr, p, 0)), (i, n, l)


@pytest.fixture(scope="module")
def ragged():
    return RaggedBatch(count=12, logns=(6, 9, 12, 13, 14), seed=77)


def test_ragged_loop_vs_oracle(ragged):
    c = ragged
    assert len({n for n, _ in c.specs}) >= 3 and len({l for _, l in c.specs}) >= 4
    c.run()
    for i in range(len(c.specs)):
        check_against_oracle(c, i)


@pytest.mark.parametrize("branches", [1, 5])
def test_ragged_graph_with_branches_vs_oracle(ragged, branches):
    c = ragged
    c.run()                                     # caches every table first
    g = c.graph(branches)
    for lst in (c.NA, c.NB, c.RA, c.PR, c.AS):
        for arr in lst:
            zero(arr)
    before = capi.launches()
    g.launch()
    assert capi.launches() - before >= 5 * len(c.specs)
    for i in range(len(c.specs)):
        check_against_oracle(c, i)


def test_ragged_batched_vs_oracle(ragged):
    """The transforms of every ciphertext in two heal_ntt_batch calls, plain
    and as a graph with branches, against the oracle."""
    c = ragged
    c.run()
    for lst in (c.NA, c.NB, c.RA, c.PR, c.AS):
        for arr in lst:
            zero(arr)
    c.run_batched()
    for i in range(len(c.specs)):
        check_against_oracle(c, i)
    g = c.graph_batched(3)
    for lst in (c.NA, c.NB, c.RA, c.PR, c.AS):
        for arr in lst:
            zero(arr)
    g.launch()
    for i in range(len(c.specs)):
        check_against_oracle(c, i)


def test_schedule_balances_branches(ragged):
    plan = ragged.schedule(4)
    assert sorted(i for b in plan for i in b) == list(range(len(ragged.specs)))
    loads = [sum(ragged.work(i) for i in b) for b in plan]
    assert max(loads) <= sum(loads) / 4 + max(ragged.work(i) for i in range(len(ragged.specs)))


def test_graph_branch_errors():
    capi.check(capi.lib().heal_graph_begin())
    try:
        assert capi.lib().heal_graph_branch(0) != 0              # nothing forked yet
        assert capi.lib().heal_graph_fork(0) != 0
        assert capi.lib().heal_graph_fork(65) != 0
        capi.check(capi.lib().heal_graph_fork(2))
        assert capi.lib().heal_graph_fork(2) != 0                # once per capture
        assert capi.lib().heal_graph_branch(2) != 0
        assert capi.lib().heal_synchronize() != 0                # would break the capture
        assert b"captured" in capi.lib().heal_last_error()
        capi.check(capi.lib().heal_graph_branch(1))
        capi.check(capi.lib().heal_graph_branch(-1))
    finally:
        import ctypes
        h = ctypes.c_void_p()
        capi.check(capi.lib().heal_graph_end(ctypes.byref(h)))
        capi.check(capi.lib().heal_graph_destroy(h))
    capi.synchronize()                                           # usable afterwards


# ------------------------------------------------------------------ plans
def all_plans(m, k):
    logm = m.bit_length() - 1
    splits = ([0] if logm <= 12 else []) + [s for s in range(1, 13) if 1 <= logm - s <= 12]
    return [(c, s) for c in (1, 2, 4, 8, 16) for s in splits]


@pytest.mark.parametrize("dt,bound,shape", [
    (np.int64, 1 << 50, (2, 1 << 13, 1, 5)),
    (np.int32, 1 << 31, (3, 1 << 10, 1, 3)),
    (np.int64, 1 << 30, (1, 1 << 16, 2, 3)),
])
def test_every_plan_matches_oracle(dt, bound, shape):
    l, m, r, k = shape
    qs = P.ntt_primes(bound, m, k)
    p, perm, tw, itw, minv = P.ntt_tables(qs, m, dt)
    x = P.residues(11, shape, qs, dt)
    wide = lambda v: v.astype(np.int64)
    want = O.ntt(wide(x), wide(p), wide(perm), wide(tw)).astype(dt)
    back = x
    dx, dp, dperm, dtw, ditw, dminv = (up(v) for v in (x, p, perm, tw, itw, minv))
    dwant = up(want)
    out = capi.DeviceArray.empty(shape, dt)
    code = capi.DTYPES[np.dtype(dt)]
    plans = all_plans(m, k)
    if m == 1 << 16:
        plans = [pl for pl in plans if pl[1] in (4, 6, 8, 10, 12)]
    try:
        for c, s in plans:
            for inv in (0, 1):
                capi.check(capi.lib().heal_ntt_set_plan(code, inv, m, k, c, s))
            capi.call("heal_ntt", dx, dp, dperm, dtw, None, None, out)
            assert np.array_equal(out.numpy(), want), (c, s)
            capi.call("heal_intt", dwant, dp, dperm, ditw, dminv, None, None, out)
            assert np.array_equal(out.numpy(), back), (c, s)
    finally:
        capi.check(capi.lib().heal_ntt_clear_plans())


def test_autotune_keeps_a_valid_plan():
    shape = (2, 1 << 14, 1, 6)
    l, m, r, k = shape
    qs = P.ntt_primes(1 << 50, m, k)
    p, perm, tw, itw, minv = P.ntt_tables(qs, m)
    x = P.residues(12, shape, qs)
    dx, dp, dperm, dtw, ditw, dminv = (up(v) for v in (x, p, perm, tw, itw, minv))
    out, back = capi.DeviceArray.empty(shape, np.int64), capi.DeviceArray.empty(shape, np.int64)
    try:
        c, s = capi.autotune_ntt(False, dx, dp, dperm, dtw, None, out, reps=2)
        assert c in (1, 2, 4, 8) and 4 <= s <= 10 and capi.ntt_plan(np.int64, False, m, k) == (c, s)
        assert np.array_equal(out.numpy(), O.ntt(x, p, perm, tw))
        ci, si = capi.autotune_ntt(True, out, dp, dperm, ditw, dminv, back, reps=2)
        assert capi.ntt_plan(np.int64, True, m, k) == (ci, si)
        assert np.array_equal(back.numpy(), x)
    finally:
        capi.check(capi.lib().heal_ntt_clear_plans())
    assert capi.ntt_plan(np.int64, False, m, k) == (4, 7)       # the default again
