"""heal_modmul_axis_sum (the fused op behind DeviceDispatcher.modmul_axis_sum)
equals the composition of HEAL's own ops, computed by the oracle:
axis_modsum(modmul(a', b, p), axis), a' = a or permute(a, perms, axis,
perm_axis); broadcasting, both word sizes, canonical and non-canonical
inputs (the term-by-term fallback), and the argument errors."""
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


def fused(a, b, p, axis, perms=None, perm_axis=0, out_shape=None):
    shape = np.broadcast_shapes(a.shape, b.shape)
    out_shape = out_shape or tuple(d for i, d in enumerate(shape) if i != axis)
    out = capi.DeviceArray.empty(out_shape, a.dtype)
    capi.call("heal_modmul_axis_sum", up(a), up(b), up(p), None if perms is None else up(perms), perm_axis, out, axis)
    return out.numpy()


def composed(a, b, p, axis, perms=None, perm_axis=0):
    shape = np.broadcast_shapes(a.shape, b.shape)
    a_full = np.ascontiguousarray(np.broadcast_to(a, shape))
    if perms is not None:
        a_full = O.permute(a_full, perms.astype(a.dtype), axis, perm_axis)
    prod = O.modmul(a_full, np.ascontiguousarray(np.broadcast_to(b, shape)), p, out_shape=shape)
    return O.axis_modsum(prod, p, axis)


def moduli(dt, k, rng):
    top = (1 << 31) - 1 if dt == np.int32 else (1 << 62)
    qs = [top, 3, 65537][:k] + [int(rng.integers(2, top)) for _ in range(max(0, k - 3))]
    return np.array(qs[:k], dtype=dt)


@pytest.mark.parametrize("dt", [np.int32, np.int64])
@pytest.mark.parametrize("shapes,axis", [
    (((5, 3, 4), (5, 3, 4)), 0),
    (((5, 3, 4), (1, 3, 4)), 0),
    (((6, 7, 2, 4), (6, 1, 1, 4)), 1),
    (((9, 4), (9, 4)), 0),
    (((2, 300, 3), (300, 3)), 1),
])
def test_matches_composition_canonical(dt, shapes, axis):
    rng = np.random.default_rng(1)
    sa, sb = shapes
    p = moduli(dt, sa[-1], rng)
    a = (rng.integers(0, 1 << 62, size=sa) % p.astype(np.int64)).astype(dt)
    b = (rng.integers(0, 1 << 62, size=sb) % p.astype(np.int64)).astype(dt)
    assert np.array_equal(fused(a, b, p, axis), composed(a, b, p, axis))


@pytest.mark.parametrize("dt", [np.int32, np.int64])
def test_matches_composition_non_canonical(dt):
    rng = np.random.default_rng(2)
    p = np.array([97, 65521, 7], dtype=dt)
    a = rng.integers(-1000, 100000, size=(11, 5, 3)).astype(dt)
    b = rng.integers(-500, 3000, size=(11, 5, 3)).astype(dt)
    a[3, 2, 1] = -7
    for axis in (0, 1):
        assert np.array_equal(fused(a, b, p, axis), composed(a, b, p, axis)), axis


@pytest.mark.parametrize("bits", [40, 61, 62, 63])
def test_non_negative_terms_above_q(bits):
    """Terms in [q, 2^bitlen(q)) (non-canonical, non-negative) and terms
    above that, against the composition."""
    rng = np.random.default_rng(bits)
    p = np.array([(1 << (bits - 1)) + 12345, (1 << (bits - 1)) + 3], np.int64)
    lo, hi = int(p.min()), (1 << bits) - 1
    a = rng.integers(lo, hi, size=(37, 6, 2), dtype=np.int64)
    b = rng.integers(lo, hi, size=(37, 6, 2), dtype=np.int64)
    assert np.array_equal(fused(a, b, p, 0), composed(a, b, p, 0))
    b[5, 3, 1] = np.int64((1 << 62) + 5)                       # one term far above
    assert np.array_equal(fused(a, b, p, 0), composed(a, b, p, 0))


def test_rotation_sum_matches_permute_modmul_axis_modsum():
    rng = np.random.default_rng(3)
    d, n, l = 8, 256, 3
    qs = P.ntt_primes(1 << 40, n, l)
    p = np.array(qs, np.int64)
    ct = P.residues(4, (2, n, l), qs)
    perms = np.stack([P.galois_perm(n, pow(5, i, 2 * n)) for i in range(d)]).astype(np.int64)
    diag = P.residues(5, (d, 1, n, l), qs)
    a = np.broadcast_to(ct[None], (d, 2, n, l))
    want = composed(a, diag, p, 0, perms, 2)
    assert np.array_equal(fused(a, diag, p, 0, perms, 2), want)
    # the serving layout: polynomials next to each other, out viewed [n, 2, l]
    a2 = np.broadcast_to(np.moveaxis(ct, 0, 1)[None], (d, n, 2, l))
    got = fused(a2, diag.reshape(d, n, 1, l), p, 0, perms, 1)
    assert np.array_equal(np.moveaxis(got, 1, 0), want)


def test_rotation_sum_over_flattened_slot_pair():
    """The serving layout: S = [d, N/d, d, 2, L], slot j = u * d + s; the
    diagonals enter as [d, 1, d, 1, L] and the rotation gathers over (u, s)."""
    d, n, l = 8, 256, 3
    qs = P.ntt_primes(1 << 40, n, l)
    p = np.array(qs, np.int64)
    ct = P.residues(6, (2, n, l), qs)
    perms = np.stack([P.galois_perm(n, pow(5, i, 2 * n)) for i in range(d)]).astype(np.int64)
    diag = P.residues(7, (d, d, l), qs)                       # diag[i, s, t]
    tiled = np.broadcast_to(diag[:, None, :, :], (d, n // d, d, l)).reshape(d, 1, n, l)
    want = composed(np.broadcast_to(ct[None], (d, 2, n, l)), tiled, p, 0, perms, 2)   # [2, n, l]
    dct, dperm = up(ct), up(perms)
    A = capi.DeviceArray(dct.buf, np.int64, (d, n // d, d, 2, l), (0, d * l, l, n * l, 1))
    B = capi.DeviceArray(up(diag).buf, np.int64, (d, 1, d, 1, l), (d * l, 0, l, 0, 1))
    P3 = capi.DeviceArray(dperm.buf, np.int64, (d, n // d, d), (n, d, 1))
    out = capi.DeviceArray.empty((2, n, l), np.int64)
    O4 = capi.DeviceArray(out.buf, np.int64, (n // d, d, 2, l), (d * l, l, n * l, 1))
    capi.call("heal_modmul_axis_sum", A, B, up(p), P3, 1, O4, 0)
    assert np.array_equal(out.numpy(), want)
    # a gather pair that a does not walk linearly, perms that are not linear, the reduced axis inside the pair
    A_bad = capi.DeviceArray(dct.buf, np.int64, (d, n // d, d, 2, l), (0, l, l, n * l, 1))
    P3_bad = capi.DeviceArray(up(np.zeros((d, n // d, 2 * d), np.int64)).buf, np.int64, (d, n // d, d),
                              (n * 2, 2 * d, 1))
    for args in ((A_bad, B, up(p), P3, 1, O4, 0), (A, B, up(p), P3_bad, 1, O4, 0)):
        with pytest.raises(ValueError):
            capi.call("heal_modmul_axis_sum", *args)
    with pytest.raises(ValueError):
        capi.call("heal_modmul_axis_sum", A, B, up(p), capi.DeviceArray(dperm.buf, np.int64, (n // d, d, 2),
                                                                         (d, 1, 0)), 0, O4, 1)


def test_argument_errors():
    a = np.zeros((4, 5, 3), np.int64)
    p = np.array([7, 11, 13], np.int64)
    perms = np.zeros((4, 5), np.int64)
    out = capi.DeviceArray.empty((5, 3), np.int64)
    da, dp = up(a), up(p)
    bad = [
        ((da, up(np.zeros((4, 6, 3), np.int64)), dp, None, 0, out, 0), ValueError),     # not broadcastable
        ((da, da, dp, None, 0, out, 2), ValueError),                                    # reduce the last axis
        ((da, da, up(np.array([7, 11], np.int64)), None, 0, out, 0), ValueError),        # p length
        ((da, da, dp, None, 0, capi.DeviceArray.empty((4, 3), np.int64), 0), ValueError),  # result shape
        ((da, da, dp, up(np.zeros((4, 4), np.int64)), 1, out, 0), ValueError),            # perms shape
        ((da, da, dp, up(perms), 0, out, 0), ValueError),                                 # perm_axis == axis
        ((da, da, dp, up(np.full((4, 5), 5, np.int64)), 1, out, 0), IndexError),           # index out of range
    ]
    for args, exc in bad:
        with pytest.raises(exc):
            capi.call("heal_modmul_axis_sum", *args)
