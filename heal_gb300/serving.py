"""Serving loop: encrypted-vector x plaintext-matrix products on one GB300.

A request multiplies a resident NTT-domain ciphertext ct[2, N, L] by a d x d
plaintext matrix with the diagonal method: out = sum_i diag_i * rot_i(ct),
where rot_i is the Galois automorphism X -> X^(5^i) (a permutation of the
NTT-domain evaluation points) and diag_i is the i-th generalised diagonal of
the matrix tiled over the N slots.  Three HEAL calls do it:

  permute      ct expanded (stride 0) to [d, 2, N, L], rows of perms[d, N]
               = the d Galois maps, elementwise axis 0, permuted axis 2
               -> the rotated stack R[d, 2, N, L]
  modmul       R viewed as [d, 2, N/d, d, L] times the diagonals
               [d, 1, 1, d, L] (broadcast over both polynomials and the
               N/d tiles), in place
  axis_modsum  R over axis 0 -> out[2, N, L]

with the matrix copied in (H2D, pinned) before and the result copied out
(D2H, pinned) after, all on the request's stream.  The fused path does the
same in one heal_modmul_axis_sum over S = [d, N/d, d, 2, L] (slot j = u*d + s):
the ciphertext and the d x d diagonals enter as stride-only views and the
rotation gathers over the flattened slot pair, so no stack is written.

Intake.  A request can arrive as a transcript in HEAL's wire format (JSON
with base64 tensors, python_execution/lattica_heal_runtime/serialization.py:
15-148, read as runtime.py:79-93 reads it): a host_to_device of the d x d
matrix's diagonals, a `matvec` device op on a resident ciphertext the server
names ("ct/N/L/c") and on the uploaded diagonals, and a device_to_host of the
result.  matvec_transcript writes one (the client side);
MatVecServer.from_transcript decodes and checks it and returns the Request
that the loop admits like any other, the decoded diagonals taking the place
of the server's own matrix.

Scheduling.  Arrivals follow a seeded Poisson process.  A request is
admitted, in arrival order, once its device footprint (rotated stack,
diagonals, output) fits in a fixed HBM arena; the arena's host-side
first-fit allocator hands out byte ranges of one heal_alloc buffer, and a
range returns to it only after the request's completion event has fired, so
no stream can still be using memory that another request receives.
Admitted requests go round-robin over a set of CUDA streams.  Latency is
completion (observed by polling the event) minus arrival.
"""
from __future__ import annotations

import bisect
import concurrent.futures as cf
import ctypes
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import params as P

ALIGN = 256


# ------------------------------------------------------------ host logic
class Arena:
    """First-fit allocator over [0, size) with coalescing of free ranges."""

    def __init__(self, size: int):
        self.size = size
        self.free_list = [(0, size)]          # sorted, disjoint (offset, length)
        self.live = {}
        self.peak = 0

    @property
    def used(self) -> int:
        return sum(self.live.values())

    def alloc(self, nbytes: int):
        n = max(ALIGN, (nbytes + ALIGN - 1) // ALIGN * ALIGN)
        for i, (off, ln) in enumerate(self.free_list):
            if ln >= n:
                if ln == n:
                    self.free_list.pop(i)
                else:
                    self.free_list[i] = (off + n, ln - n)
                self.live[off] = n
                self.peak = max(self.peak, self.used)
                return off
        return None

    def free(self, off: int):
        n = self.live.pop(off)
        i = bisect.bisect(self.free_list, (off, 0))
        self.free_list.insert(i, (off, n))
        # merge with the neighbours
        if i + 1 < len(self.free_list) and off + n == self.free_list[i + 1][0]:
            self.free_list[i] = (off, n + self.free_list.pop(i + 1)[1])
        if i > 0 and self.free_list[i - 1][0] + self.free_list[i - 1][1] == off:
            po, pn = self.free_list[i - 1]
            self.free_list[i - 1] = (po, pn + self.free_list.pop(i)[1])


@dataclass
class Request:
    rid: int
    arrival: float          # seconds from the start of the run
    n: int
    l: int
    d: int
    ct: int                 # resident ciphertext index for (n, l)
    mat: int                # matrix variant for (d, l)
    admitted: float = -1.0
    done: float = -1.0

    fused: bool = False
    host_diag: object = None  # decoded from the request's transcript (else the server's own matrix)
    host_buf: object = None   # the pinned byte buffer host_diag lies in, when it was decoded in place

    def footprint(self) -> int:
        """Device bytes the request holds while in flight: the rotated stack
        (three calls only), the diagonals as sent, and the output."""
        stack = 0 if self.fused else stack_bytes(self.n, self.l, self.d)
        return stack + diag_bytes(self.l, self.d) + out_bytes(self.n, self.l)


def stack_bytes(n, l, d):
    return d * 2 * n * l * 8


def diag_bytes(l, d):
    return d * d * l * 8


def out_bytes(n, l):
    return 2 * n * l * 8


def ct_name(n: int, l: int, c: int) -> str:
    """The name a transcript uses for resident ciphertext c of shape [2, n, l]."""
    return f"ct/{n}/{l}/{c}"


def matvec_transcript(ct: str, diagonals) -> str:
    """A request as a HEAL transcript (JSON): upload the diagonals
    [d, 1, 1, d, L] (int64; a numpy array travels as np.save bytes, a torch
    tensor as torch.save bytes, both base64, as HEAL encodes them),
    `matvec` of resident ciphertext `ct` by them, download of the result
    [2, N, L].  The download's expected tensor is an empty placeholder (in
    the diagonals' own encoding): the client has no result to verify."""
    import torch
    from .runtime import DeviceTensorPointer, TranscriptBuilder, dumps
    tb = TranscriptBuilder(prefix="r")
    tb.segment("matvec")
    dg = tb.host_to_device(diagonals)
    out = tb.op("matvec", DeviceTensorPointer(ct, torch.int64), dg, int(diagonals.shape[0]), dtype=torch.int64)
    empty = np.zeros(0, np.int64) if isinstance(diagonals, np.ndarray) else torch.zeros(0, dtype=torch.int64)
    tb.device_to_host(out, empty)
    tb.free(dg, out)
    tb.end_segment()
    return dumps(tb.transcript())


def parse_matvec_transcript(transcript):
    """(ciphertext name, d, diagonals) of a matvec request transcript; raises
    ValueError for any other shape of transcript."""
    from .runtime import DeviceOpArgType as A
    from .runtime import ExecutionTranscriptOpType as K
    ops = [(k, v) for k, v in transcript.transcript if k in (K.DEVICE_OP, K.FREE_DEVICE_TENSOR)]
    names = [v.name for k, v in ops if k == K.DEVICE_OP]
    if names != ["host_to_device", "matvec", "device_to_host"]:
        raise ValueError(f"not a matvec request: device ops {names}")
    h2d, mv, d2h = [v for k, v in ops if k == K.DEVICE_OP]
    up = h2d.out.value.inf_name
    a0, a1, a2 = (mv.args + [None, None, None])[:3]
    if not (len(mv.args) == 3 and a0.arg_type == A.DEVICE_TENSOR and a1.arg_type == A.DEVICE_TENSOR and
            a1.value.inf_name == up and a2.arg_type == A.INT):
        raise ValueError("matvec takes (resident ciphertext, the uploaded diagonals, d)")
    if d2h.args[0].value.inf_name != mv.out.value.inf_name:
        raise ValueError("the request must download the matvec result")
    diag = h2d.args[0].value.tensor
    d = int(a2.value)
    if diag.ndim != 5 or diag.shape[0] != d or diag.shape[3] != d or diag.shape[1] != 1 or diag.shape[2] != 1:
        raise ValueError(f"diagonals must have shape [d, 1, 1, d, L], got {tuple(diag.shape)}")
    return a0.value.inf_name, d, diag


def poisson_schedule(count: int, rate: float, seed: int, ns, ds, lmin: int, lmax: int, cts: int, mats: int):
    """`count` requests with exponential inter-arrival gaps of mean 1/rate;
    ring degree, dimension, limb count, ciphertext and matrix are drawn
    uniformly, all from SplitMix64 streams of `seed`."""
    u = (P.splitmix64(seed, count) >> np.uint64(11)).astype(np.float64) / float(1 << 53)
    gaps = -np.log1p(-u) / rate
    t = np.cumsum(gaps)
    pick = lambda s, lo, hi: P.uniform(seed + s, (count,), lo, hi)
    ni, di, ls = pick(1, 0, len(ns)), pick(2, 0, len(ds)), pick(3, lmin, lmax + 1)
    ci, mi = pick(4, 0, cts), pick(5, 0, mats)
    return [Request(i, float(t[i]), int(ns[ni[i]]), int(ls[i]), int(ds[di[i]]), int(ci[i]), int(mi[i]))
            for i in range(count)]


@dataclass
class LoopStats:
    latencies: list = field(default_factory=list)
    waits: list = field(default_factory=list)
    max_queue: int = 0
    max_inflight: int = 0
    peak_bytes: int = 0
    span: float = 0.0


def serve(requests, arena: Arena, issue, clock=time.perf_counter, idle=None, max_inflight: int = 64,
          timeout: float | None = None, intake=None):
    """Runs the admission loop.  issue(req, offset) enqueues the request's GPU
    work and returns an object with query() -> bool (True once finished) and
    finish() (called once, after query() turned True).  Requests are admitted
    in arrival order when their footprint fits in the arena.  A request larger
    than the whole arena raises MemoryError; with `timeout` (seconds), a
    request still unfinished that long after its admission raises
    TimeoutError, so a device that stopped answering ends the loop instead
    of leaving it polling.  With `intake`, each request is replaced on
    arrival by intake(request) (a transcript decoded into the request it
    describes), or by a concurrent.futures.Future of it (decoded on another
    thread): a request is admitted only once it is decoded, still in
    arrival order, and a decoding error ends the loop with that error.
    The decoding time counts toward the request's latency."""
    pending = sorted(requests, key=lambda r: r.arrival)
    queue, inflight, st = [], [], LoopStats()   # queue: (index in pending, request or its Future)
    nxt, t0 = 0, clock()
    while nxt < len(pending) or queue or inflight:
        now = clock() - t0
        while nxt < len(pending) and pending[nxt].arrival <= now:
            item = pending[nxt] if intake is None else intake(pending[nxt])
            if not isinstance(item, cf.Future):
                pending[nxt] = item
            queue.append((nxt, item))
            nxt += 1
        st.max_queue = max(st.max_queue, len(queue))
        progressed = False
        for item in list(inflight):
            req, off, h = item
            if h.query():
                req.done = clock() - t0
                h.finish()
                arena.free(off)
                inflight.remove(item)
                st.latencies.append(req.done - req.arrival)
                progressed = True
            elif timeout is not None and now - req.admitted > timeout:
                raise TimeoutError(f"request {req.rid} unfinished {now - req.admitted:.3f} s after admission "
                                   f"(limit {timeout} s)")
        while queue and len(inflight) < max_inflight:
            idx, req = queue[0]
            if isinstance(req, cf.Future):
                if not req.done():
                    break
                req = pending[idx] = req.result()
                queue[0] = (idx, req)
            off = arena.alloc(req.footprint())
            if off is None:
                if not inflight:
                    raise MemoryError(f"request {req.rid} needs {req.footprint()} bytes, more than the arena")
                break
            queue.pop(0)
            req.admitted = clock() - t0
            st.waits.append(req.admitted - req.arrival)
            inflight.append((req, off, issue(req, off)))
            progressed = True
        st.max_inflight = max(st.max_inflight, len(inflight))
        st.peak_bytes = max(st.peak_bytes, arena.used)
        if not progressed and idle is not None:
            idle()
    st.span = (max(r.done for r in pending) - pending[0].arrival) if pending else 0.0
    return st


def percentile(xs, q):
    return float(np.percentile(np.asarray(xs), q)) if xs else 0.0


# ------------------------------------------------------------- the device
class MatVecServer:
    """Resident ciphertexts, rotation tables and the HBM arena for the
    matrix-vector requests; `issue` runs one request on the next stream."""

    def __init__(self, ns=(1 << 14, 1 << 15), ds=(16, 64, 256), lmin=8, lmax=16, bits=40, cts=2, mats=2,
                 budget=16 << 30, streams=8, seed=505, fused=False):
        import torch
        from . import capi
        self.capi, self.torch = capi, torch
        self.ns, self.ds, self.lmin, self.lmax, self.cts, self.mats = ns, ds, lmin, lmax, cts, mats
        self.fused = fused
        D = capi.DeviceArray.from_numpy
        self.qs = {n: P.ntt_primes(1 << bits, n, lmax) for n in ns}
        self.p = {(n, l): D(np.array(self.qs[n][:l], np.int64)) for n in ns for l in range(lmin, lmax + 1)}
        # resident NTT-domain ciphertexts, uniform mod q
        self.ct = {(n, l): [D(P.residues(seed + 7919 * c + 31 * l + n, (2, n, l), self.qs[n][:l]))
                            for c in range(cts)] for n in ns for l in range(lmin, lmax + 1)}
        # Galois maps X -> X^(5^i), i < d, per ring degree
        self.perms = {}
        for n in ns:
            for d in ds:
                elts = [pow(5, i, 2 * n) for i in range(d)]
                self.perms[(n, d)] = D(np.stack([P.galois_perm(n, e) for e in elts]).astype(np.int64))
        # matrix diagonals [d, 1, 1, d, L] (uniform mod q), pinned for the H2D
        self.host_mats = {}
        for d in ds:
            for l in range(lmin, lmax + 1):
                for v in range(mats):
                    self.host_mats[(d, l, v)] = {
                        n: torch.from_numpy(P.residues(seed + 104729 * v + 613 * d + l + n, (d, 1, 1, d, l),
                                                       self.qs[n][:l])).pin_memory() for n in ns}
        self.arena_size = budget
        self.arena_buf = capi.Buffer(budget, zero=False)
        self.arena = Arena(budget)
        self.streams = [torch.cuda.Stream() for _ in range(streams)]
        self.rr = 0
        self.out_host = {}
        self.keep = set()                    # request ids whose output is kept
        self.pinned = {}                     # shape -> free pinned buffers for decoded diagonals
        self.pinned_bytes = {}               # size -> free pinned byte buffers that payloads decode into
        self.pool_lock = threading.Lock()    # the pools are shared with the intake threads

    # views into the arena
    def _view(self, off, shape):
        return self.capi.DeviceArray(self.arena_buf, np.int64, shape, None, off)

    def calls(self, req: Request, off: int) -> dict:
        """The request's HEAL calls (name -> thunk) on its arena range at
        `off`, in order: the rotated stack, the diagonal product and the sum
        (three calls), or one modmul_axis_sum (fused)."""
        capi, n, l, d = self.capi, req.n, req.l, req.d
        o_diag = off if self.fused else off + stack_bytes(n, l, d)
        out = self._view(o_diag + diag_bytes(l, d), (2, n, l))
        ct = self.ct[(n, l)][req.ct]
        p, perms = self.p[(n, l)], self.perms[(n, d)]
        if self.fused:
            # S = [d, N/d, d, 2, L] over (i, u, s, c, t), slot j = u * d + s:
            # a = ct (stride 0 on i), b = diag[i, s, t] (broadcast over u and c),
            # the rotation gathers over the flattened slot pair (u, s)
            A = capi.DeviceArray(ct.buf, np.int64, (d, n // d, d, 2, l), (0, d * l, l, n * l, 1), ct.offset)
            B = capi.DeviceArray(self.arena_buf, np.int64, (d, 1, d, 1, l), (d * l, 0, l, 0, 1), o_diag)
            perms3 = capi.DeviceArray(perms.buf, np.int64, (d, n // d, d), (n, d, 1), perms.offset)
            o = capi.DeviceArray(self.arena_buf, np.int64, (n // d, d, 2, l), (d * l, l, n * l, 1),
                                 o_diag + diag_bytes(l, d))
            return {"modmul_axis_sum": lambda: capi.call("heal_modmul_axis_sum", A, B, p, perms3, 1, o, 0)}
        R = self._view(off, (d, 2, n, l))
        R5 = self._view(off, (d, 2, n // d, d, l))
        diag = self._view(o_diag, (d, 1, 1, d, l))
        src = ct.reshape((1, 2, n, l)).expand(0, d)
        return {"permute": lambda: capi.call("heal_permute", src, perms, R, 0, 2),
                "modmul": lambda: capi.call("heal_modmul_ttt", R5, diag, p, R5),
                "axis_modsum": lambda: capi.call("heal_axis_modsum", R, p, out, 0)}

    def enqueue(self, req: Request, off: int, stream):
        """Issues the request's copies and HEAL calls on `stream`; the output
        lands in a pinned host array returned with the event."""
        capi, n, l, d = self.capi, req.n, req.l, req.d
        capi.check(capi.lib().heal_set_stream(stream.cuda_stream))
        try:
            o_diag = off if self.fused else off + stack_bytes(n, l, d)
            out = self._view(o_diag + diag_bytes(l, d), (2, n, l))
            host = req.host_diag if req.host_diag is not None else self.host_mats[(d, l, req.mat)][n]
            capi.check(capi.lib().heal_h2d_async(ctypes.c_void_p(self.arena_buf.ptr.value + o_diag),
                                                 ctypes.c_void_p(host.data_ptr()), diag_bytes(l, d)))
            for fn in self.calls(req, off).values():
                fn()
            res = self.torch.empty((2, n, l), dtype=self.torch.int64, pin_memory=True)
            capi.check(capi.lib().heal_d2h_async(ctypes.c_void_p(res.data_ptr()), ctypes.c_void_p(out.ptr),
                                                 out_bytes(n, l)))
            ev = self.torch.cuda.Event()
            ev.record(stream)
        finally:
            capi.check(capi.lib().heal_set_stream(None))
        return ev, res

    def issue(self, req: Request, off: int):
        stream = self.streams[self.rr % len(self.streams)]
        self.rr += 1
        ev, res = self.enqueue(req, off, stream)
        server = self

        class Handle:
            def query(self):
                return ev.query()

            def finish(self):
                if req.rid in server.keep:
                    server.out_host[req.rid] = res.numpy().copy()
                server.recycle(req)  # its upload has completed
        return Handle()

    def recycle(self, req: Request):
        """Returns a decoded request's pinned buffer to its pool (once
        nothing reads it any more)."""
        if req.host_buf is not None:
            self._give(self.pinned_bytes, req.host_buf.numel(), req.host_buf)
        elif req.host_diag is not None:
            self._give(self.pinned, tuple(req.host_diag.shape), req.host_diag)
        req.host_diag = req.host_buf = None

    def split_ms(self, req: Request, reps: int = 5) -> dict:
        """Median CUDA-event time of each HEAL call of the request (its
        copies excluded), for the server's path."""
        torch = self.torch
        req.fused = self.fused
        off = self.arena.alloc(req.footprint())
        stream = self.streams[0]
        self.capi.check(self.capi.lib().heal_set_stream(stream.cuda_stream))
        try:
            res = {}
            for name, fn in self.calls(req, off).items():
                ts = []
                for _ in range(reps):
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    fn()
                    e1.record(stream)
                    e1.synchronize()
                    ts.append(e0.elapsed_time(e1))
                res[name] = sorted(ts)[len(ts) // 2]
            return res
        finally:
            self.capi.check(self.capi.lib().heal_set_stream(None))
            self.arena.free(off)

    def _take(self, pool: dict, key, make):
        with self.pool_lock:
            free = pool.get(key)
            if free:
                return free.pop()
        return make()

    def _give(self, pool: dict, key, buf):
        with self.pool_lock:
            pool.setdefault(key, []).append(buf)

    def from_transcript(self, text, rid: int, arrival: float) -> Request:
        """Decodes a matvec request transcript (JSON text, or its UTF-8 bytes
        as they arrive) into a Request on a resident ciphertext.  The
        payload is decoded by the C library's base64 decoder straight into a
        pinned byte buffer from a pool, and a numpy payload is uploaded from
        where it lands; any other payload (torch.save bytes, Fortran order)
        is copied into a pinned buffer first.  The buffers return to their
        pools when the request completes.  Safe to call from several
        threads at once."""
        from .runtime import loads
        torch = self.torch
        handed = []

        def sink(nbytes):
            buf = self._take(self.pinned_bytes, nbytes,
                             lambda: torch.empty(nbytes, dtype=torch.uint8, pin_memory=True))
            handed.append(buf)
            return buf.numpy()

        try:
            name, d, diag = parse_matvec_transcript(loads(text, sink=sink))
            try:
                tag, n, l, c = name.split("/")
                n, l, c = int(n), int(l), int(c)
                assert tag == "ct" and (n, l) in self.ct and 0 <= c < len(self.ct[(n, l)])
            except (ValueError, AssertionError):
                raise ValueError(f"no resident ciphertext named {name!r}") from None
            if d not in self.ds or n % d or tuple(diag.shape) != (d, 1, 1, d, l):
                raise ValueError(f"request of d = {d} on {name} does not fit the server")
        except BaseException:
            for buf in handed:
                self._give(self.pinned_bytes, buf.numel(), buf)
            raise
        owner = None
        if isinstance(diag, np.ndarray) and diag.dtype == np.int64 and diag.flags.c_contiguous:
            ptr = diag.ctypes.data
            owner = next((b for b in handed if b.data_ptr() <= ptr and ptr + diag.nbytes <= b.data_ptr() + b.numel()),
                         None)
        for buf in handed:
            if buf is not owner:
                self._give(self.pinned_bytes, buf.numel(), buf)
        if owner is not None:
            return Request(rid, arrival, n, l, d, c, -1, host_diag=torch.from_numpy(diag), host_buf=owner)
        src = torch.as_tensor(diag, dtype=torch.int64)
        host = self._take(self.pinned, tuple(src.shape),
                          lambda: torch.empty(tuple(src.shape), dtype=torch.int64, pin_memory=True))
        host.copy_(src)
        return Request(rid, arrival, n, l, d, c, -1, host_diag=host)

    def alone(self, req: Request) -> np.ndarray:
        """The request run by itself (one stream, nothing else in flight)."""
        req.fused = self.fused
        off = self.arena.alloc(req.footprint())
        if off is None:
            raise MemoryError("arena full")
        try:
            ev, res = self.enqueue(req, off, self.streams[0])
            ev.synchronize()
            return res.numpy().copy()
        finally:
            self.arena.free(off)

    def warm(self):
        """One request of every (n, l, d) shape, so that every table the
        calls derive is cached before timing."""
        rid = -1
        for n in self.ns:
            for l in range(self.lmin, self.lmax + 1):
                for d in self.ds:
                    self.alone(Request(rid, 0.0, n, l, d, 0, 0))
        self.torch.cuda.synchronize()

    def run(self, requests, keep=(), timeout: float | None = 60.0, transcripts=None, intake_threads: int = 0):
        """Serves `requests`; a request still unfinished `timeout` seconds
        after its admission (admitted requests take milliseconds) raises
        TimeoutError.  With `transcripts` ({rid: JSON text or bytes}), a
        request whose rid has one arrives as that transcript and is decoded
        on arrival: on the loop's thread, or with `intake_threads` > 0 on
        that many worker threads while the loop keeps admitting and
        completing requests (the base64 decoding runs in the C library
        without the interpreter lock)."""
        for r in requests:
            r.fused = self.fused
        self.keep = set(keep)
        self.out_host = {}
        if not transcripts:
            return serve(requests, self.arena, self.issue, timeout=timeout)

        def decode(r):
            q = self.from_transcript(transcripts[r.rid], r.rid, r.arrival)
            q.fused = self.fused
            return q

        if intake_threads <= 0:
            return serve(requests, self.arena, self.issue, timeout=timeout,
                         intake=lambda r: decode(r) if r.rid in transcripts else r)
        with cf.ThreadPoolExecutor(max_workers=intake_threads) as pool:
            # the polling loop yields the interpreter lock whenever it has nothing to do
            return serve(requests, self.arena, self.issue, timeout=timeout, idle=lambda: time.sleep(0),
                         intake=lambda r: pool.submit(decode, r) if r.rid in transcripts else r)

    @staticmethod
    def bytes_moved(req: Request) -> int:
        """Algorithmic bytes of one request, copies to and from the host
        included.  Three calls: permute writes the stack (the ciphertext is
        read once per rotation, from L2), modmul reads it and writes it,
        axis_modsum reads it and writes the output.  Fused: the rotation
        table (d x N indices), the ciphertext and the diagonals are read once
        and the output written once."""
        n, l, d = req.n, req.l, req.d
        io = 2 * diag_bytes(l, d) + 2 * out_bytes(n, l)   # H2D + its read, D2H + its write
        if req.fused:
            return d * n * 8 + out_bytes(n, l) + out_bytes(n, l) + io
        return 4 * stack_bytes(n, l, d) + io
