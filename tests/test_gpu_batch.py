"""heal_ntt_batch: a ragged batch of transforms (every shape, element type and
modulus width of the per-call tests mixed in one call) equals the transforms
called one by one, bit for bit; argument errors leave every result
untouched; the batch records into a CUDA graph."""
import numpy as np
import pytest

from heal_gb300 import capi
from heal_gb300 import params as P
from oracle import oracle as O
from _gpu import ready, up

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def gpu():
    return ready()


# (l, m, r, k, dtype, prime bound): one- and two-pass, 32- and 64-bit words,
# lazy and growing 64-bit ranges, the small kernel (m <= 4), r > 1
SHAPES = [
    (2, 4096, 1, 3, np.int64, 2**30), (1, 8192, 1, 5, np.int64, 2**50), (2, 1 << 14, 1, 2, np.int64, 2**40),
    (1, 1024, 2, 4, np.int32, 2**31), (3, 2048, 1, 6, np.int32, 2**30), (1, 256, 1, 9, np.int64, 2**62),
    (2, 4, 1, 3, np.int64, 2**50), (1, 1 << 16, 1, 2, np.int64, 2**50), (1, 512, 3, 1, np.int64, 2**50),
    (2, 8192, 1, 3, np.int32, 2**31),
]


def make_jobs(seed, shapes, inverse, negative=False):
    rng = np.random.default_rng(seed)
    host, dev = [], []
    for i, (l, m, r, k, dt, bound) in enumerate(shapes):
        qs = P.ntt_primes(bound, max(m, 2), k)
        p, perm, tw, itw, minv = P.ntt_tables(qs, m, dt)
        a = P.residues(seed * 100 + i, (l, m, r, k), qs, dt)
        if negative and i % 3 == 0:
            a.reshape(-1)[rng.integers(0, a.size)] = -5
        d = [up(a), up(p), up(perm), up(itw if inverse else tw), up(minv) if inverse else None,
             capi.DeviceArray.empty(a.shape, dt)]
        host.append((a, p, perm, itw if inverse else tw, minv))
        dev.append(d)
    return host, dev


def one_by_one(inverse, dev):
    outs = []
    for a, p, perm, tw, minv, _ in dev:
        out = capi.DeviceArray.empty(a.shape, np.dtype(a.dtype))
        if inverse:
            capi.call("heal_intt", a, p, perm, tw, minv, None, None, out)
        else:
            capi.call("heal_ntt", a, p, perm, tw, None, None, out)
        outs.append(out.numpy())
    return outs


@pytest.mark.parametrize("inverse", [False, True])
@pytest.mark.parametrize("negative", [False, True])
def test_batch_equals_calls(inverse, negative):
    host, dev = make_jobs(5 + inverse, SHAPES * 3, inverse, negative)
    capi.ntt_batch(inverse, dev)
    want = one_by_one(inverse, dev)
    for i, (d, w) in enumerate(zip(dev, want)):
        assert np.array_equal(d[5].numpy(), w), i
    # and against the oracle for a few
    for i in (0, 1, 6):
        a, p, perm, tw, minv = host[i]
        wide = lambda v: np.asarray(v).astype(np.int64)
        ref = (O.intt(wide(a), wide(p), wide(perm), wide(tw), wide(minv), exact=1) if inverse
               else O.ntt(wide(a), wide(p), wide(perm), wide(tw))).astype(a.dtype)
        assert np.array_equal(dev[i][5].numpy(), ref), i


def test_batch_general_permutations_and_in_place():
    m = 8192
    qs = P.ntt_primes(2**40, m, 2)
    p, _, tw, itw, minv = P.ntt_tables(qs, m)
    perm = np.argsort(P.splitmix64(7, m)).astype(np.int64)
    dup = perm.copy()
    dup[3] = dup[9]                                   # non-bijective: the forward's extra gather
    jobs, want = [], []
    for i, pm in enumerate((perm, dup, perm)):
        a = P.residues(40 + i, (1, m, 1, 2), qs)
        want.append(O.ntt(a, p, pm, tw))
        da = up(a)
        res = da if i == 2 else capi.DeviceArray.empty(a.shape, np.int64)   # job 2 in place
        jobs.append((da, up(p), up(pm), up(tw), None, res))
    capi.ntt_batch(False, jobs)
    for j, w in zip(jobs, want):
        assert np.array_equal(j[5].numpy(), w)


def test_batch_errors_write_nothing():
    host, dev = make_jobs(9, SHAPES[:4], False)
    before = [d[5].numpy().copy() for d in dev]
    bad = list(dev)
    a, p, perm, tw, _, res = bad[2]
    bad[2] = (a, p, perm, up(np.zeros((1, 3), np.int64)), None, res)   # twiddles of the wrong shape
    L = capi.lib()
    arr = capi.ntt_jobs(bad)
    assert L.heal_ntt_batch(0, arr, len(bad)) == 1
    assert "job 2" in capi.lib().heal_last_error().decode()
    for d, b in zip(dev, before):
        assert np.array_equal(d[5].numpy(), b)
    # one job writing another's input
    clash = list(dev)
    clash[1] = list(dev[1][:5]) + [dev[0][0]]
    arr = capi.ntt_jobs(clash)
    assert L.heal_ntt_batch(0, arr, len(clash)) == 1
    assert L.heal_ntt_batch(0, None, 0) == 0


@pytest.mark.parametrize("inverse", [False, True])
def test_batch_in_a_graph(inverse):
    host, dev = make_jobs(11, SHAPES, inverse)
    capi.ntt_batch(inverse, dev)                      # tables built outside the capture
    want = [d[5].numpy().copy() for d in dev]
    fresh = [list(d[:5]) + [capi.DeviceArray.empty(d[0].shape, np.dtype(d[0].dtype))] for d in dev]
    g = capi.Graph(lambda: capi.ntt_batch(inverse, fresh))
    g.launch()
    g.launch()
    for d, w in zip(fresh, want):
        assert np.array_equal(d[5].numpy(), w)


def test_batch_larger_than_one_flush():
    """More than 512 jobs: the recorded passes are launched in several groups."""
    shapes = [(1, 64 << (i % 4), 1, 1 + i % 3, np.int64, 2**50) for i in range(1100)]
    host, dev = make_jobs(13, shapes[:8], False)
    jobs = []
    for i in range(len(shapes)):
        a, p, perm, tw, _, _ = dev[i % 8]
        jobs.append((a, p, perm, tw, None, capi.DeviceArray.empty(a.shape, np.int64)))
    capi.ntt_batch(False, jobs)
    want = one_by_one(False, dev[:8])
    for i, j in enumerate(jobs):
        assert np.array_equal(j[5].numpy(), want[i % 8]), i
