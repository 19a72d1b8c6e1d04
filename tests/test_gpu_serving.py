"""Serving loop on the GPU at reduced sizes: every request of a burst that
the arena budget forces to queue gives the oracle's
permute -> modmul -> axis_modsum result, and the same result as when the
request runs alone."""
import numpy as np
import pytest

from heal_gb300 import serving as S
from oracle.chain import oracle_matvec
from _gpu import ready

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def gpu():
    return ready()


def oracle_product(srv, req):
    n, l, d = req.n, req.l, req.d
    return oracle_matvec(srv.ct[(n, l)][req.ct].numpy(), srv.perms[(n, d)].numpy(),
                         srv.host_mats[(d, l, req.mat)][n].numpy(), np.array(srv.qs[n][:l], np.int64))


@pytest.mark.parametrize("fused", [False, True])
def test_serving_outputs_match_oracle_and_standalone(fused):
    srv = S.MatVecServer(ns=(256, 512), ds=(2, 4, 8), lmin=2, lmax=4, bits=40, cts=2, mats=2,
                         budget=1 << 20, streams=3, seed=21, fused=fused)
    srv.warm()
    reqs = S.poisson_schedule(60, 50000.0, 8, srv.ns, srv.ds, srv.lmin, srv.lmax, srv.cts, srv.mats)
    st = srv.run(reqs, keep=[r.rid for r in reqs])
    assert len(st.latencies) == len(reqs) and st.max_queue > 1 and st.max_inflight > 1
    assert st.peak_bytes <= 1 << 20
    for r in reqs:
        got = srv.out_host[r.rid]
        assert np.array_equal(got, oracle_product(srv, r)), r
        assert np.array_equal(got, srv.alone(r)), r


@pytest.mark.parametrize("fused", [False, True])
def test_requests_arriving_as_transcripts(fused):
    """A burst whose requests arrive as HEAL transcripts (decoded on arrival)
    gives, request by request, what the same requests give issued directly
    and what the oracle gives."""
    srv = S.MatVecServer(ns=(256, 512), ds=(2, 4, 8), lmin=2, lmax=4, bits=40, cts=2, mats=2,
                         budget=1 << 20, streams=3, seed=23, fused=fused)
    srv.warm()
    reqs = S.poisson_schedule(40, 50000.0, 12, srv.ns, srv.ds, srv.lmin, srv.lmax, srv.cts, srv.mats)
    texts = {r.rid: S.matvec_transcript(S.ct_name(r.n, r.l, r.ct), srv.host_mats[(r.d, r.l, r.mat)][r.n])
             for r in reqs if r.rid % 2 == 0}
    direct = {r.rid: srv.alone(S.Request(r.rid, 0.0, r.n, r.l, r.d, r.ct, r.mat)) for r in reqs}
    st = srv.run(reqs, keep=[r.rid for r in reqs], transcripts=texts)
    assert len(st.latencies) == len(reqs)
    for r in reqs:
        assert np.array_equal(srv.out_host[r.rid], direct[r.rid]), r
        assert np.array_equal(srv.out_host[r.rid], oracle_product(srv, r)), r
    with pytest.raises(ValueError, match="resident"):
        srv.from_transcript(S.matvec_transcript("ct/999/2/0", srv.host_mats[(2, 2, 0)][256]), 0, 0.0)


def test_large_transcripts_decoded_natively():
    """Requests whose diagonals (up to 64 x 64 x 6 int64, 256 KB of base64)
    are cut out of the JSON and decoded by heal_base64_decode, as np.save
    payloads used in place and as torch.save payloads, arriving as bytes:
    every result equals the request issued directly and the oracle."""
    srv = S.MatVecServer(ns=(4096,), ds=(16, 64), lmin=4, lmax=6, bits=40, cts=2, mats=2,
                         budget=1 << 26, streams=3, seed=29, fused=True)
    srv.warm()
    reqs = S.poisson_schedule(24, 20000.0, 31, srv.ns, srv.ds, srv.lmin, srv.lmax, srv.cts, srv.mats)
    assert {r.d for r in reqs} == {16, 64}
    texts = {}
    for r in reqs:
        diag = srv.host_mats[(r.d, r.l, r.mat)][r.n]
        texts[r.rid] = S.matvec_transcript(S.ct_name(r.n, r.l, r.ct), diag.numpy() if r.rid % 2 else diag).encode()
    direct = {r.rid: srv.alone(S.Request(r.rid, 0.0, r.n, r.l, r.d, r.ct, r.mat)) for r in reqs}
    for threads in (0, 3):  # decoded on the loop's thread, then on three intake threads
        st = srv.run(reqs, keep=[r.rid for r in reqs], transcripts=texts, intake_threads=threads)
        assert len(st.latencies) == len(reqs)
        for r in reqs:
            assert np.array_equal(srv.out_host[r.rid], direct[r.rid]), (threads, r)
    for r in reqs[:4]:
        assert np.array_equal(srv.out_host[r.rid], oracle_product(srv, r)), r
    assert srv.pinned_bytes  # numpy payloads landed in pooled pinned buffers
