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


# ------------------------------------------- heal_modmul_axis_sum_permute
def fused_post(a, b, p, axis, perms, ew, pa, out=None):
    shape = np.broadcast_shapes(a.shape, b.shape)
    out_shape = tuple(d for i, d in enumerate(shape) if i != axis)
    o = out if out is not None else capi.DeviceArray.empty(out_shape, a.dtype)
    capi.call("heal_modmul_axis_sum_permute", a if isinstance(a, capi.DeviceArray) else up(a),
              b if isinstance(b, capi.DeviceArray) else up(b), up(p), axis, up(perms), ew, pa, o)
    return o.numpy()


def composed_post(a, b, p, axis, perms, ew, pa):
    shape = np.broadcast_shapes(a.shape, b.shape)
    prod = O.modmul(np.ascontiguousarray(np.broadcast_to(a, shape)),
                    np.ascontiguousarray(np.broadcast_to(b, shape)), p, out_shape=shape)
    return O.permute(O.axis_modsum(prod, p, axis), perms.astype(a.dtype), ew, pa)


def random_perms(rng, rows, m, dt):
    return np.stack([rng.permutation(m) for _ in range(rows)]).astype(dt)


@pytest.mark.parametrize("dt", [np.int32, np.int64])
@pytest.mark.parametrize("shapes,axis,ew,pa", [
    (((2, 64, 1, 3, 5), (2, 64, 1, 3, 5)), 3, 2, 1),     # keyswitch tail: digits reduced, rows gathered
    (((2, 64, 1, 3, 5), (1, 64, 1, 3, 5)), 3, 0, 1),     # b broadcast over the components
    (((7, 33, 4), (7, 33, 4)), 0, 1, 0),                 # gathered axis after the reduced one
    (((5, 9, 6, 4), (9, 1, 4)), 2, 0, 1),                # broadcast b, reduced axis after the gathered one
    (((3, 50, 2), (3, 50, 2)), 0, 1, 0),
    (((2, 64, 1, 3, 6), (2, 64, 1, 3, 6)), 3, 2, 1),     # an even limb count
])
def test_post_permute_matches_composition(dt, shapes, axis, ew, pa):
    rng = np.random.default_rng(31)
    sa, sb = shapes
    p = moduli(dt, sa[-1], rng)
    a = (rng.integers(0, 1 << 62, size=sa) % p.astype(np.int64)).astype(dt)
    b = (rng.integers(0, 1 << 62, size=sb) % p.astype(np.int64)).astype(dt)
    shape = np.broadcast_shapes(sa, sb)
    rshape = tuple(d for i, d in enumerate(shape) if i != axis)
    perms = random_perms(rng, rshape[ew], rshape[pa], np.int64)
    assert np.array_equal(fused_post(a, b, p, axis, perms, ew, pa), composed_post(a, b, p, axis, perms, ew, pa))


@pytest.mark.parametrize("dt", [np.int32, np.int64])
@pytest.mark.parametrize("k", [3, 4])
def test_post_permute_non_canonical_and_duplicate_rows(dt, k):
    rng = np.random.default_rng(32)
    p = np.array([97, 65521, 7, 40009][:k], dtype=dt)
    a = rng.integers(-1000, 100000, size=(2, 40, 1, 3, k)).astype(dt)
    b = rng.integers(-500, 3000, size=(2, 40, 1, 3, k)).astype(dt)
    perms = random_perms(rng, 1, 40, np.int32)
    perms[0, 7] = perms[0, 8]                          # two results read one row
    assert np.array_equal(fused_post(a, b, p, 3, perms, 2, 1), composed_post(a, b, p, 3, perms, 2, 1))


def test_post_permute_is_the_keyswitch_tail():
    from heal_gb300.chain import KeyswitchChain
    ch = KeyswitchChain(n=1024, limbs=4, digits=3, base_bits=17, bound_bits=50)
    ct = capi.DeviceArray.from_numpy(P.residues(41, ch.shape(), ch.qs))
    want = capi.DeviceArray.empty(ch.shape(), np.int64)
    got = capi.DeviceArray.empty(ch.shape(), np.int64)
    ch.run(ct, want)
    for _ in range(2):
        ch.run_fused(ct, got)
        assert np.array_equal(got.numpy(), want.numpy())


def test_post_permute_errors():
    p = np.array([97, 89], np.int64)
    a = np.zeros((3, 4, 2), np.int64)
    out = capi.DeviceArray.empty((4, 2), np.int64)           # result of a [3, 4, 2] reduced over axis 0
    L = capi.lib()
    ok = up(np.tile(np.arange(4), (2, 1)).astype(np.int64))     # [result.dims[ew = 1], result.dims[pa = 0]]
    wrong = up(np.tile(np.arange(4), (3, 1)).astype(np.int64))  # wrong shape: [3, 4]
    oob_h = np.tile(np.arange(4), (2, 1)).astype(np.int64)
    oob_h[1, 3] = 4
    oob = up(oob_h)
    da, dp = up(a), up(p)                                       # every operand kept alive across the calls
    call = lambda perms, ew, pa: L.heal_modmul_axis_sum_permute(
        capi._arg(da), capi._arg(da), capi._arg(dp), 0, capi._arg(perms), ew, pa, capi._arg(out))
    assert call(ok, 1, 0) == 0
    for ew, pa in [(0, 0), (2, 0), (1, 5)]:
        assert call(ok, ew, pa) == 1
    assert call(wrong, 1, 0) == 1
    before = out.numpy().copy()
    assert call(oob, 1, 0) == 2
    assert np.array_equal(out.numpy(), before)                  # nothing written
    assert call(None, 1, 0) == 1


def test_post_permute_through_lattica_hw():
    """The same op through the `lattica_hw` module and the transcript dispatcher."""
    import torch
    import heal_gb300
    from heal_gb300.runtime.dispatcher import GB300Dispatcher
    hw = heal_gb300.lattica_hw()
    rng = np.random.default_rng(33)
    p = np.array([65537, 97, 257], np.int64)
    a = (rng.integers(0, 1 << 40, size=(2, 16, 1, 3, 3)) % p).astype(np.int64)
    b = (rng.integers(0, 1 << 40, size=(2, 16, 1, 3, 3)) % p).astype(np.int64)
    perms = random_perms(rng, 1, 16, np.int64)
    want = composed_post(a, b, p, 3, perms, 2, 1)
    H = lambda x: hw.host_to_device_64(torch.from_numpy(np.ascontiguousarray(x)))
    out = hw.allocate_on_hardware_64([2, 16, 1, 3])
    hw.modmul_axis_sum_permute_64(H(a), H(b), H(p), 3, H(perms), 2, 1, out)
    assert np.array_equal(hw.device_to_host_64(out).numpy(), want)
    out2 = hw.allocate_on_hardware_64([2, 16, 1, 3])
    GB300Dispatcher().modmul_axis_sum_permute(H(a), H(b), H(p), 3, H(perms), 2, 1, out2)
    assert np.array_equal(hw.device_to_host_64(out2).numpy(), want)


# ------------------------------------------------ heal_g_decomposition_ntt
def gdec_ntt(a, power, bits, p_t, perm, tw_t):
    l, m, r, k = a.shape
    out = capi.DeviceArray.empty((l, m, r, k * power), a.dtype)
    capi.call("heal_g_decomposition_ntt", up(a), power, bits, up(p_t), up(perm), up(tw_t), out)
    return out.numpy()


def gdec_then_ntt(a, power, bits, p_t, perm, tw_t):
    wide = lambda v: np.asarray(v).astype(np.int64)
    dig, _ = O.g_decomposition(a, power, bits)
    l, m, r, k = a.shape
    flat = np.ascontiguousarray(dig.reshape(l, m, r, k * power))
    return O.ntt(wide(flat), wide(p_t), wide(perm), wide(tw_t)).astype(a.dtype)


@pytest.mark.parametrize("dt,bound,m,power,bits", [
    (np.int64, 2**50, 1 << 16, 3, 17),    # the keyswitch digits: two passes
    (np.int64, 2**50, 2048, 3, 17),       # one pass
    (np.int64, 2**40, 8192, 4, 10),
    (np.int32, 2**30, 4096, 2, 15),
    (np.int32, 2**31, 1 << 14, 3, 11),
    (np.int64, 2**62, 512, 2, 31),        # lazy 64-bit ranges
    (np.int64, 2**50, 2, 3, 17),          # the small kernel
])
def test_gdec_ntt_matches_composition(dt, bound, m, power, bits):
    k = 3
    qs = P.ntt_primes(bound, max(m, 2), k)
    p, perm, tw, itw, minv = P.ntt_tables(qs, m, dt)
    p_t, tw_t = np.repeat(p, power), np.repeat(tw, power, axis=0)
    a = P.residues(m + power, (2, m, 1, k), qs, dt)
    assert np.array_equal(gdec_ntt(a, power, bits, p_t, perm, tw_t), gdec_then_ntt(a, power, bits, p_t, perm, tw_t))


def test_gdec_ntt_negative_values_general_perm_and_warnings(capfd):
    m, k, power, bits = 8192, 2, 3, 17
    qs = P.ntt_primes(2**50, m, k)
    p, _, tw, itw, minv = P.ntt_tables(qs, m)
    perm = np.argsort(P.splitmix64(3, m)).astype(np.int64)
    p_t, tw_t = np.repeat(p, power), np.repeat(tw, power, axis=0)
    a = P.residues(8, (1, m, 1, k), qs)
    a[0, 3, 0, 1] = -5                      # digits of the uint64 image, reduced on load
    a[0, 77, 0, 0] = (1 << 60) + 9          # above power * bits: a capacity warning
    capi.synchronize()
    capfd.readouterr()
    got = gdec_ntt(a, power, bits, p_t, perm, tw_t)
    capi.synchronize()
    err_fused = capfd.readouterr().err
    assert np.array_equal(got, gdec_then_ntt(a, power, bits, p_t, perm, tw_t))
    assert "exceeds capacity with base_bits=17 and power=3" in err_fused
    dig = capi.DeviceArray.empty((1, m, 1, k, power), np.int64)
    capi.call("heal_g_decomposition", up(a), dig, power, bits)
    capi.synchronize()
    err_sep = capfd.readouterr().err
    assert err_fused.count("exceeds") == err_sep.count("exceeds") == 2


def test_gdec_ntt_errors():
    qs = P.ntt_primes(2**40, 64, 2)
    p, perm, tw, _, _ = P.ntt_tables(qs, 64)
    a = up(P.residues(1, (1, 64, 1, 2), qs))
    L = capi.lib()
    dperm = up(perm)
    dpt, dtwt, dp = up(np.repeat(p, 3)), up(np.repeat(tw, 3, axis=0)), up(p)   # kept alive across the calls
    good = capi.DeviceArray.empty((1, 64, 1, 6), np.int64)
    bad_shape = capi.DeviceArray.empty((1, 64, 1, 5), np.int64)
    call = lambda out, power, bits, pt: L.heal_g_decomposition_ntt(
        capi._arg(a), power, bits, capi._arg(pt), capi._arg(dperm), capi._arg(dtwt), capi._arg(out))
    assert call(good, 3, 14, dpt) == 0
    assert call(bad_shape, 3, 14, dpt) == 1
    assert call(good, 3, 64, dpt) == 1
    assert call(good, 0, 14, dpt) == 1
    assert call(good, 3, 14, dp) == 1      # p must have k * power moduli


def test_gdec_ntt_through_lattica_hw():
    import torch
    import heal_gb300
    from heal_gb300.runtime.dispatcher import GB300Dispatcher
    hw = heal_gb300.lattica_hw()
    m, k, power, bits = 1024, 2, 3, 17
    qs = P.ntt_primes(2**50, m, k)
    p, perm, tw, _, _ = P.ntt_tables(qs, m)
    p_t, tw_t = np.repeat(p, power), np.repeat(tw, power, axis=0)
    a = P.residues(9, (2, m, 1, k), qs)
    want = gdec_then_ntt(a, power, bits, p_t, perm, tw_t)
    H = lambda x: hw.host_to_device_64(torch.from_numpy(np.ascontiguousarray(x)))
    out = hw.allocate_on_hardware_64([2, m, 1, k * power])
    hw.g_decomposition_ntt_64(H(a), power, bits, H(p_t), H(perm), H(tw_t), out)
    assert np.array_equal(hw.device_to_host_64(out).numpy(), want)
    out2 = hw.allocate_on_hardware_64([2, m, 1, k * power])
    GB300Dispatcher().g_decomposition_ntt(H(a), power, bits, H(p_t), H(perm), H(tw_t), out2)
    assert np.array_equal(hw.device_to_host_64(out2).numpy(), want)


def test_keyswitch_batch_equals_single_chains():
    from heal_gb300.chain import KeyswitchChain
    ch = KeyswitchChain(n=1024, limbs=4, digits=3, base_bits=17, bound_bits=50)
    count = 3
    host = [P.residues(50 + i, ch.shape(), ch.qs) for i in range(count)]
    want = []
    for h in host:
        out = capi.DeviceArray.empty(ch.shape(), np.int64)
        ch.run(capi.DeviceArray.from_numpy(h), out)
        want.append(out.numpy())
    kb = ch.batched(count)
    cts = capi.DeviceArray.from_numpy(np.concatenate(host, axis=0))
    out = capi.DeviceArray.empty(kb.shape(), np.int64)
    kb.run(cts, out)
    got = out.numpy()
    for i in range(count):
        assert np.array_equal(got[2 * i:2 * i + 2], want[i]), i
