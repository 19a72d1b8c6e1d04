"""The NTT register kernel's shared-tile addressing, restated from
heal_gb300/csrc/heal_ntt_kernels.cuh (point_of, swz_of, tidx) and checked on
the CPU for every tile size, points per thread, tile width and step the
kernels instantiate:
  - in every step, the (thread, register) -> point map covers the tile's
    points exactly once (the exchanges lose and duplicate nothing);
  - every butterfly of a step pairs two points held by the same thread;
  - a point's tile word is the thread's base word XOR a per-register
    constant (the kernel's exchange addressing);
  - shared-memory bank conflicts of each step's access pattern: none where
    the points of one wavefront lie at stride 1, or at stride 16 and number
    at most 16 (the strided and blocked patterns the 4-bit swizzle was made
    for); at most 4-way anywhere."""
import pytest


def point_of(inv, logp, klpt, step, r, e):
    """heal_ntt_kernels.cuh point_of<INV, LOGP, kLPT>(step, r, e)."""
    st0 = klpt * step
    q = min(logp - st0, klpt)
    jj = e & ((1 << q) - 1)
    ident = (r << (klpt - q)) + (e >> q)
    if not inv:
        ld = logp - st0 - q
        hi, lo = ident >> ld, ident & ((1 << ld) - 1)
        return (hi << (ld + q)) + lo + (jj << ld)
    hi, lo = ident >> st0, ident & ((1 << st0) - 1)
    return (hi << (st0 + q)) + lo + (jj << st0)


def swz(s):
    """heal_ntt_kernels.cuh swz_of."""
    return s ^ ((s >> 4) & 15)


def tidx(s, c, logc):
    return (swz(s) << logc) + c


# (direction, log2 points per thread, shared word bytes) of the instantiated
# register kernels: 64-bit words hold 8 points per thread, and 16 in the
# 256-point forward passes of the plain 64-bit transform; the forward
# canonical 32-bit mode holds 16; the other 32-bit modes hold 8
KINDS = [(False, 3, 8), (True, 3, 8), (False, 4, 8), (False, 4, 4), (False, 3, 4), (True, 3, 4)]
SHAPES = [(inv, klpt, wb, logp, logc) for inv, klpt, wb in KINDS for logp in range(4, 13) for logc in range(5)
          if ((1 << logp) >> klpt) << logc <= 512]


@pytest.mark.parametrize("inv,klpt,wb,logp,logc", SHAPES)
def test_register_kernel_addressing(inv, klpt, wb, logp, logc):
    P, kpt, C = 1 << logp, 1 << klpt, 1 << logc
    threads = (P >> klpt) * C
    nstep = (logp + klpt - 1) // klpt
    lanes = 32 if wb == 4 else 16          # lanes served by one shared-memory wavefront
    for step in range(nstep):
        pts = [[point_of(inv, logp, klpt, step, r, e) for e in range(kpt)] for r in range(P >> klpt)]
        assert sorted(p for row in pts for p in row) == list(range(P)), step
        # butterfly partners of the step's stages stay in the thread
        st0 = klpt * step
        for st in range(st0, min(st0 + klpt, logp)):
            dist = (P >> (st + 1)) if not inv else (1 << st)
            for row in pts:
                held = set(row)
                assert all((p ^ dist) in held for p in row), (step, st)
        # base XOR constant equals the direct tile index
        for r, row in enumerate(pts):
            base = tidx(point_of(inv, logp, klpt, step, r, 0), 0, logc)
            for e, p in enumerate(row):
                assert tidx(p, 0, logc) == base ^ (swz(point_of(inv, logp, klpt, step, 0, e)) << logc)
        # bank conflicts of this step's layout
        for e in range(kpt):
            words = [tidx(pts[t >> logc][e], t & (C - 1), logc) for t in range(threads)]
            for w0 in range(0, threads, lanes):
                grp = words[w0:w0 + lanes]
                banks = [(w * wb // 4) % 32 for w in grp]
                ways = max(banks.count(b) for b in set(banks))
                pts_grp = sorted({pts[(w0 + i) >> logc][e] for i in range(len(grp))})
                strides = {b - a for a, b in zip(pts_grp, pts_grp[1:])}
                if strides <= {1} or (strides <= {16} and len(pts_grp) <= 16):
                    assert ways == 1, (step, e, w0, pts_grp)
                assert ways <= 4, (step, e, w0)


def test_headline_shapes_conflict_profile():
    """Worst ways per step layout for the chain's transforms (P = 256 points,
    4 limbs per tile, 64-bit words, 8 points per thread): the forward
    transform's short last step and the inverse's first and last steps have
    2-way conflicts; the other layouts have none."""
    def profile(inv):
        out = []
        for step in range(3):
            worst = 1
            for e in range(8):
                words = [tidx(point_of(inv, 8, 3, step, t >> 2, e), t & 3, 2) for t in range(128)]
                for w0 in range(0, 128, 16):
                    banks = [(w * 2) % 32 for w in words[w0:w0 + 16]]
                    worst = max(worst, max(banks.count(b) for b in set(banks)))
            out.append(worst)
        return out
    assert profile(False) == [1, 1, 2]
    assert profile(True) == [2, 1, 2]


def _swizzles():
    """s ^ ((s >> k1) & m1) [^ ((s >> k2) & m2)]: XOR-linear, invertible on
    every tile (each term moves bits only downward)."""
    out = []
    for k1 in range(1, 9):
        for m1 in (1, 3, 7, 15):
            out.append(lambda s, k1=k1, m1=m1: s ^ ((s >> k1) & m1))
    for k1 in range(1, 9):
        for k2 in range(k1 + 1, 9):
            for m1 in (3, 7, 15):
                for m2 in (1, 3, 7, 15):
                    out.append(lambda s, a=k1, b=k2, x=m1, y=m2: s ^ ((s >> a) & x) ^ ((s >> b) & y))
    return out


def _conflict_free(f, patterns):
    """No wavefront of any pattern has two distinct words in one bank."""
    for pts, logc, wb in patterns:
        C, lanes = 1 << logc, (32 if wb == 4 else 16)
        words = [(f(p) << logc) + (i & (C - 1)) for i, p in enumerate(pts)]
        for w0 in range(0, len(words), lanes):
            by_bank = {}
            for w in words[w0:w0 + lanes]:
                by_bank.setdefault((w * wb // 4) % 32, set()).add(w)
            if any(len(v) > 1 for v in by_bank.values()):
                return False
    return True


@pytest.mark.parametrize("inv", [False, True])
def test_each_64bit_exchange_has_a_conflict_free_swizzle(inv):
    """The next step the 2-way conflicts call for: every exchange of the
    64-bit modes (the keyswitch chain's transforms), taken on its own, has an
    XOR swizzle of one or two shifted terms that is conflict-free for both
    its write pattern (the previous step's layout) and its read pattern, for
    every tile size and width."""
    fams = _swizzles()
    for logp in range(4, 13):
        for x in range(1, (logp + 2) // 3):
            pats = []
            for logc in range(5):
                threads = ((1 << logp) >> 3) << logc
                if threads > 512:
                    continue
                for st in (x - 1, x):
                    for e in range(8):
                        pats.append(([point_of(inv, logp, 3, st, t >> logc, e) for t in range(threads)], logc, 8))
            assert any(_conflict_free(f, pats) for f in fams), (inv, logp, x)
