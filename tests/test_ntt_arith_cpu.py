"""The 64-bit NTT kernels' arithmetic restated in Python integers (CPU only):
the three-multiply high product of the Shoup quotient (mulhi64_3 in
heal_gb300/csrc/heal_ntt_kernels.cuh), the range of the Shoup product built on
it (mulw_grow), and the growing-range headroom that the host's mode choice
(heal_ntt.cu: forward q < 2^56, an inverse pass of P stages q < 2^(62 - P))
relies on.  The GPU tests check the kernels' results bit for bit; this file
checks the bounds those results depend on, including the extreme inputs."""
import random

import pytest

M64 = (1 << 64) - 1


def mulhi64_3(a, b):
    """floor(a * b / 2^64) without the low-by-low partial product and the low
    words of the two cross products, as the kernel forms it."""
    al, ah, bl, bh = a & 0xFFFFFFFF, a >> 32, b & 0xFFFFFFFF, b >> 32
    return (ah * bh + ((ah * bl) >> 32) + ((al * bh) >> 32)) & M64


def mulw_grow(y, w, wp, q):
    return (y * w - mulhi64_3(y, wp) * q) & M64


def edge_words():
    return [0, 1, 2, 0xFFFFFFFF, 1 << 32, (1 << 32) + 1, (1 << 63) - 1, 1 << 63, M64, M64 - 1,
            0xFFFFFFFF00000000, 0x00000000FFFFFFFF | (1 << 40)]


def test_three_multiply_high_product_is_at_most_two_low():
    rng = random.Random(1)
    pairs = [(a, b) for a in edge_words() for b in edge_words()]
    pairs += [(rng.getrandbits(64), rng.getrandbits(64)) for _ in range(100000)]
    # low words all ones: the dropped parts are largest
    pairs += [(rng.getrandbits(32) << 32 | 0xFFFFFFFF, rng.getrandbits(32) << 32 | 0xFFFFFFFF) for _ in range(20000)]
    worst = 0
    for a, b in pairs:
        e = ((a * b) >> 64) - mulhi64_3(a, b)
        assert 0 <= e <= 2, (a, b)
        worst = max(worst, e)
    assert worst == 2  # the bound is reached


@pytest.mark.parametrize("bits", [30, 40, 50, 55])
def test_shoup_product_with_the_short_quotient_is_below_4q(bits):
    rng = random.Random(bits)
    q = (1 << bits) - rng.randrange(1 << 20) * 2 - 1
    for _ in range(20000):
        w = rng.randrange(q)
        wp = (w << 64) // q                       # the companion the derived tables hold
        y = rng.getrandbits(63) if rng.random() < 0.5 else rng.randrange(97 * q)
        r = mulw_grow(y, w, wp, q)
        assert r < 4 * q and r % q == (y * w) % q
    for y in (0, 1, q - 1, q, 97 * q - 1, (1 << 63) - 1):
        w = q - 1
        r = mulw_grow(y, w, (w << 64) // q, q)
        assert r < 4 * q and r % q == (y * w) % q


def test_forward_growing_range_headroom():
    """A canonical input grows by at most 4q per stage (u + t and u - t + 4q
    with t < 4q): below (1 + 4 log2 m) q after all stages, which must stay
    below 2^63 (the unreduced values of a first pass are stored as int64)."""
    for logm in range(1, 25):
        q = (1 << 56) - 1                          # the largest modulus the forward mode takes
        assert (1 + 4 * logm) * q < 1 << 63, logm
    assert (1 + 4 * 24) * (1 << 57) >= 1 << 63    # why 2^57 no longer qualifies


def test_forward_stage_bound_by_simulation():
    """The worst case of one stage, iterated: u < Bq, t < 4q gives u + t and
    u - t + 4q in [0, (B + 4) q)."""
    q = (1 << 50) - 27
    B = 1
    for _ in range(16):
        hi = (B - 1) * q + (q - 1) + (4 * q - 1)   # the largest u + t
        lo = 0 - (4 * q - 1) + 4 * q                # the smallest u - t + 4q
        assert lo >= 0 and hi < (B + 4) * q
        B += 4
    assert B * q < 1 << 63


@pytest.mark.parametrize("P", [6, 7, 8, 12])
def test_inverse_growing_range_headroom(P):
    """Values entering stage s are below 2^(s+1) q (below q at s = 0): the
    difference a - b + 2^(s+1) q is non-negative, the sum stays below
    2^(s+2) q and the product below 4q; a pass of P stages ends below
    2^(P+1) q, which must stay below 2^63 for q < 2^(62 - P)."""
    q = (1 << (62 - P)) - 1
    bound = q                                    # entering stage 0
    for s in range(P):
        qs = q << (s + 1)
        assert bound <= qs                       # a - b + qs >= 0
        nxt = max(2 * bound, 4 * q)              # the sum, the product
        assert nxt <= q << (s + 2)
        bound = nxt
    assert bound <= q << (P + 1) and (q << (P + 1)) < 1 << 63
