"""Host logic of the serving loop (no GPU): the HBM arena's first-fit
allocator, the seeded Poisson schedule, and the admission loop driven by a
fake clock and fake completion handles."""
import numpy as np
import pytest

from heal_gb300 import serving as S


def test_arena_first_fit_and_coalescing():
    a = S.Arena(4096)
    x, y, z = a.alloc(1000), a.alloc(1000), a.alloc(1000)
    assert (x, y, z) == (0, 1024, 2048) and a.used == 3072
    assert a.alloc(2048) is None                       # 1024 left
    a.free(y)
    assert a.alloc(1500) is None                       # the holes are 1024 + 1024, not adjacent
    a.free(z)                                          # y and z merge with the tail: 3072 free
    assert a.free_list == [(1024, 3072)]
    w = a.alloc(3000)
    assert w == 1024
    a.free(x)
    a.free(w)
    assert a.free_list == [(0, 4096)] and a.used == 0 and a.peak == 4096


def test_arena_random_alloc_free_keeps_ranges_disjoint():
    rng = np.random.default_rng(0)
    a = S.Arena(1 << 20)
    live = {}
    for _ in range(2000):
        if live and rng.random() < 0.5:
            off = list(live)[rng.integers(len(live))]
            a.free(off)
            del live[off]
        else:
            n = int(rng.integers(1, 50000))
            off = a.alloc(n)
            if off is not None:
                live[off] = n
        spans = sorted((o, o + ((n + 255) // 256) * 256) for o, n in live.items())
        assert all(e0 <= s1 for (_, e0), (s1, _) in zip(spans, spans[1:]))
        assert all(0 <= s and e <= a.size for s, e in spans)
        assert a.used + sum(ln for _, ln in a.free_list) == a.size


def test_poisson_schedule_is_seeded_with_the_requested_rate():
    r1 = S.poisson_schedule(20000, 2000.0, 9, (1 << 14, 1 << 15), (16, 64, 256), 8, 16, 2, 2)
    r2 = S.poisson_schedule(20000, 2000.0, 9, (1 << 14, 1 << 15), (16, 64, 256), 8, 16, 2, 2)
    assert [(r.arrival, r.n, r.l, r.d) for r in r1] == [(r.arrival, r.n, r.l, r.d) for r in r2]
    t = np.array([r.arrival for r in r1])
    assert np.all(np.diff(t) > 0)
    assert abs(len(t) / t[-1] - 2000.0) < 60                 # mean rate
    gaps = np.diff(t)
    assert abs(np.std(gaps) / np.mean(gaps) - 1.0) < 0.05     # exponential gaps
    assert {r.d for r in r1} == {16, 64, 256} and {r.l for r in r1} == set(range(8, 17))


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        self.t += 1e-5
        return self.t


def test_admission_by_footprint_in_arrival_order():
    clock = FakeClock()
    reqs = S.poisson_schedule(300, 20000.0, 4, (256, 512), (2, 4, 8), 2, 4, 2, 2)
    budget = 3 * max(r.footprint() for r in reqs)
    arena = S.Arena(budget)
    order = []

    class Handle:
        def __init__(self, req):
            self.end = clock.t + 2e-4 * req.d

        def query(self):
            return clock.t >= self.end

        def finish(self):
            pass

    def issue(req, off):
        order.append(req.rid)
        assert arena.used <= budget
        return Handle(req)

    st = S.serve(reqs, arena, lambda r, o: issue(r, o), clock=clock)
    assert order == sorted(order)                              # FIFO admission
    assert len(st.latencies) == len(reqs) and all(x > 0 for x in st.latencies)
    assert st.peak_bytes <= budget and arena.used == 0
    assert st.max_queue > 1                                   # the budget made requests wait
    assert all(r.admitted >= r.arrival and r.done > r.admitted for r in reqs)


def test_request_larger_than_the_arena_fails():
    reqs = [S.Request(0, 0.0, 1 << 15, 16, 256, 0, 0)]
    with pytest.raises(MemoryError):
        S.serve(reqs, S.Arena(1 << 20), lambda r, o: None, clock=FakeClock())


def test_unfinished_request_times_out():
    """A request whose completion never comes (a fake handle that stays
    unfinished) ends the loop with TimeoutError once the limit has passed;
    the requests that finished before it were served."""
    clock = FakeClock()
    reqs = S.poisson_schedule(5, 1000.0, 3, (256,), (2,), 2, 2, 1, 1)

    class Handle:
        def __init__(self, req):
            self.never = req.rid == 2

        def query(self):
            return not self.never

        def finish(self):
            pass

    done = []
    with pytest.raises(TimeoutError, match="request 2 unfinished"):
        S.serve(reqs, S.Arena(1 << 30), lambda r, o: (done.append(r.rid), Handle(r))[1], clock=clock, timeout=0.01)
    assert done[:3] == [0, 1, 2]
    assert all(r.done is not None for r in reqs[:2])
    # without a limit the same loop is unchanged for requests that finish
    st = S.serve(S.poisson_schedule(5, 1000.0, 3, (256,), (2,), 2, 2, 1, 1), S.Arena(1 << 30),
                 lambda r, o: Handle(S.Request(0, 0.0, 256, 2, 2, 0, 0)), clock=FakeClock(), timeout=0.01)
    assert len(st.latencies) == 5


def test_matvec_request_transcript_round_trips_through_heal_json():
    """A request written as a HEAL transcript (JSON, base64 tensors) decodes
    back to its ciphertext name, d and diagonals; other transcripts are
    refused."""
    import torch
    from heal_gb300.runtime import TranscriptBuilder, dumps, loads
    diag = torch.arange(4 * 4 * 3, dtype=torch.int64).reshape(4, 1, 1, 4, 3)
    text = S.matvec_transcript(S.ct_name(256, 3, 1), diag)
    name, d, got = S.parse_matvec_transcript(loads(text))
    assert (name, d) == ("ct/256/3/1", 4) and torch.equal(torch.as_tensor(got), diag)
    # a transcript with another op, or diagonals of the wrong shape
    tb = TranscriptBuilder()
    x = tb.host_to_device(diag)
    tb.op("axis_modsum", x, 0, dtype=torch.int64)
    with pytest.raises(ValueError, match="not a matvec request"):
        S.parse_matvec_transcript(loads(dumps(tb.transcript())))
    with pytest.raises(ValueError, match="shape"):
        S.parse_matvec_transcript(loads(S.matvec_transcript("ct/256/3/1", diag.reshape(4, 1, 4, 1, 3))))


def test_intake_decodes_each_request_on_arrival():
    """serve(..., intake=) replaces each request by intake(request) when it
    arrives, before admission."""
    seen = []

    def intake(r):
        seen.append(r.rid)
        return S.Request(r.rid, r.arrival, r.n, r.l, r.d, r.ct, r.mat)

    class Done:
        def query(self):
            return True

        def finish(self):
            pass

    reqs = [S.Request(i, 0.0, 256, 2, 4, 0, 0) for i in range(5)]
    st = S.serve(reqs, S.Arena(1 << 20), lambda r, off: Done(), intake=intake)
    assert seen == list(range(5)) and len(st.latencies) == 5


def test_intake_on_worker_threads_keeps_arrival_order():
    """With an intake that returns Futures (decoding on worker threads, some
    slower than others), requests are still admitted in arrival order, each
    only once decoded, and every one completes; a decoding error ends the
    loop with that error."""
    import concurrent.futures as cf
    import random
    import time as _time

    rng = random.Random(5)
    delays = {i: rng.choice([0.0, 0.0005, 0.002]) for i in range(40)}
    order = []

    def decode(r):
        _time.sleep(delays.get(r.rid, 0.0))
        if r.rid == 999:
            raise ValueError("no resident ciphertext named 'x'")
        return S.Request(r.rid, r.arrival, r.n, r.l, r.d, r.ct, r.mat)

    class Done:
        def query(self):
            return True

        def finish(self):
            pass

    def issue(req, off):
        order.append(req.rid)
        return Done()

    reqs = [S.Request(i, i * 1e-4, 256, 2, 4, 0, 0) for i in range(40)]
    with cf.ThreadPoolExecutor(max_workers=4) as pool:
        st = S.serve(reqs, S.Arena(1 << 24), issue, intake=lambda r: pool.submit(decode, r),
                     idle=lambda: _time.sleep(0))
    assert order == list(range(40)) and len(st.latencies) == 40
    assert st.span > 0 and all(x > 0 for x in st.latencies)
    bad = [S.Request(0, 0.0, 256, 2, 4, 0, 0), S.Request(999, 0.0, 256, 2, 4, 0, 0)]
    with cf.ThreadPoolExecutor(max_workers=2) as pool:
        with pytest.raises(ValueError, match="resident"):
            S.serve(bad, S.Arena(1 << 24), issue, intake=lambda r: pool.submit(decode, r))
