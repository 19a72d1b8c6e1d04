"""Bit-exact parity of the GPU backend with HEAL's sample implementation,
through the C ABI: every golden array the reference itself produced
(tests/golden/), and the CPU oracle on seeded inputs across sizes, element
types, modulus widths, strides and permutations."""
import hashlib

import numpy as np
import pytest

from heal_gb300 import capi
from heal_gb300 import params as P
from oracle import oracle as O
from _gpu import intt, ntt, ready, run, up

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def gpu():
    return ready()


def sha(x):
    return hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest()


# ============================================================ golden vectors
def test_ntt_pin(golden):
    g = golden("ntt_pin")
    fw = ntt(g["a"], g["p"], g["perm"], g["tw"])
    assert np.array_equal(fw, g["ntt"])
    assert np.array_equal(intt(fw, g["p"], g["perm"], g["itw"], g["minv"]), g["a"])


@pytest.mark.parametrize("case", ["ntt_i64", "ntt_i64_m1", "ntt_i64_m2", "ntt_i64_m4096", "ntt_i32", "ntt_neg"])
def test_ntt_golden(golden, case):
    g = golden(case)
    assert np.array_equal(ntt(g["a"], g["p"], g["perm"], g["tw"]), g["ntt"])
    src = g["ntt"] if "intt_a" in g else g["a"]
    got = intt(src, g["p"], g["perm"], g["itw"], g["minv"])
    assert np.array_equal(got, O.intt(src, g["p"], g["perm"], g["itw"], g["minv"], exact=1))
    width = 31 if g["a"].dtype == np.int32 else 63
    if int(g["p"].max()) ** 2 < 2 ** width:   # where the reference's m_inv product cannot wrap
        assert np.array_equal(got, g["intt"])
    if "intt_a" in g:
        assert np.array_equal(got, g["a"])


def test_ntt_negative_twiddles(golden):
    g = golden("ntt_negtw")
    assert np.array_equal(ntt(g["a"], g["p"], g["perm"], g["tw"]), g["ntt"])


def test_ntt_general_and_duplicate_perm(golden):
    g = golden("ntt_perm")
    assert np.array_equal(ntt(g["a"], g["p"], g["perm"], g["tw"]), g["ntt"])
    assert np.array_equal(intt(g["a"], g["p"], g["perm"], g["itw"], g["minv"]), g["intt"])
    assert np.array_equal(ntt(g["a"], g["p"], g["dup"], g["tw"]), g["ntt_dup"])
    assert np.array_equal(intt(g["a"], g["p"], g["dup"], g["itw"], g["minv"]), g["intt_dup"])


def test_keyswitch_n256_chain_golden(golden):
    g = golden("keyswitch_n256")
    p, perm, tw = g["p"], g["perm"], g["tw"]
    assert np.array_equal(ntt(g["ct"], p, perm, tw), g["ntt_ct"])
    x = intt(g["ct"], p, perm, g["itw"], g["minv"])
    assert np.array_equal(x, O.intt(g["ct"], p, perm, g["itw"], g["minv"], exact=1))
    dig = run("heal_g_decomposition", g["coef"], 3, 17, out_shape=g["digits"].shape, dtype=np.int64)
    assert np.array_equal(dig, g["digits"])
    L = len(p)
    p_t = np.repeat(p, 3)
    dn = ntt(g["digits"].reshape(2, -1, 1, L * 3), p_t, perm, np.repeat(tw, 3, axis=0))
    assert np.array_equal(dn, g["dn"])
    prod = run("heal_modmul_ttt", g["dn"], g["key"], p_t, out_shape=g["dn"].shape, dtype=np.int64)
    assert np.array_equal(prod, g["prod"])
    moved = up(g["prod"]).reshape((2, g["prod"].shape[1], 1, L, 3)).moveaxis(4, 3)
    acc = run("heal_axis_modsum", moved, p, 3, out_shape=g["acc"].shape, dtype=np.int64)
    assert np.array_equal(acc, g["acc"])
    rot = run("heal_permute", g["acc"], g["gal"], 2, 1, out_shape=g["acc"].shape, dtype=np.int64)
    assert np.array_equal(rot, g["rot"])


@pytest.mark.parametrize("tag,dt", [("32", np.int32), ("64", np.int64)])
@pytest.mark.parametrize("op", ["modmul", "modsum"])
def test_modops_golden(golden, tag, dt, op):
    g = golden(f"{op}_{tag}")
    f = f"heal_{op}"
    assert np.array_equal(run(f + "_ttt", g["a"], g["b"], g["p"], out_shape=g["a"].shape, dtype=dt), g["ttt"])
    assert np.array_equal(run(f + "_ttt", g["an"], g["bn"], g["pn"], out_shape=g["an"].shape, dtype=dt), g["ttt_neg"])
    assert np.array_equal(run(f + "_ttt", g["at"], g["at"], g["p"], out_shape=g["at"].shape, dtype=dt),
                          g["ttt_strided"])
    assert np.array_equal(run(f + "_ttt", g["col"], g["row"], g["prow"], out_shape=(2, 3), dtype=dt), g["ttt_bcast"])
    assert np.array_equal(run(f + "_ttc", g["an"], g["bn"], 1000003, out_shape=g["an"].shape, dtype=dt), g["ttc"])
    assert np.array_equal(run(f + "_tct", g["an"], -12345, g["pn"], out_shape=g["an"].shape, dtype=dt), g["tct"])
    assert np.array_equal(run(f + "_tcc", g["an"], 98765, 4099, out_shape=g["an"].shape, dtype=dt), g["tcc"])


@pytest.mark.parametrize("tag", ["32", "64"])
def test_axis_modsum_golden(golden, tag):
    g = golden(f"axis_modsum_{tag}")
    a = g["a"]
    for ax in (0, 1, 2):
        shape = tuple(d for i, d in enumerate(a.shape) if i != ax)
        assert np.array_equal(run("heal_axis_modsum", a, g["p"], ax, out_shape=shape, dtype=a.dtype), g[f"ax{ax}"])
    seq = run("heal_axis_modsum", np.array([[5], [5], [-8]], a.dtype), np.array([7], a.dtype), 0,
              out_shape=(1,), dtype=a.dtype)
    assert np.array_equal(seq, g["seq"])


@pytest.mark.parametrize("tag", ["32", "64"])
def test_g_decomposition_golden(golden, tag):
    g = golden(f"gdec_{tag}")
    a = g["a"]
    for key, (pw, bits) in {"b3p4": (4, 3), "b17p3": (3, 17), "b1p40": (40, 1)}.items():
        got = run("heal_g_decomposition", a, pw, bits, out_shape=a.shape + (pw,), dtype=a.dtype)
        assert np.array_equal(got, g[key]), key
    capi.synchronize()


@pytest.mark.parametrize("tag", ["32", "64"])
def test_permute_golden(golden, tag):
    g = golden(f"permute_{tag}")
    a = g["a"]
    assert np.array_equal(run("heal_permute", a, g["perms_a"], 1, 2, out_shape=a.shape, dtype=a.dtype), g["r12"])
    assert np.array_equal(run("heal_permute", a, g["perms_b"], 0, 3, out_shape=a.shape, dtype=a.dtype), g["r03"])


def test_roundtrip_full_size_hashes(golden_hash):
    # [8, 4096, 1, 4] int64 with the four largest 30-bit NTT primes, checked
    # against the reference's own outputs by SHA-256
    h = golden_hash["roundtrip_n4096"]
    qs = P.ntt_primes(h["bound"], h["N"], h["L"])
    p, perm, tw, itw, minv = P.ntt_tables(qs, h["N"])
    A = P.residues(h["seeds"][0], h["shape"], qs)
    B = P.residues(h["seeds"][1], h["shape"], qs)
    NA, NB = ntt(A, p, perm, tw), ntt(B, p, perm, tw)
    assert sha(NA) == h["ntt_a"] and sha(NB) == h["ntt_b"]
    assert sha(intt(NA, p, perm, itw, minv)) == h["intt_ntt_a"]
    PR = run("heal_modmul_ttt", NA, NB, p, out_shape=NA.shape, dtype=np.int64)
    assert sha(PR) == h["modmul"]
    AS = run("heal_axis_modsum", PR, p, 0, out_shape=PR.shape[1:], dtype=np.int64)
    assert sha(AS) == h["axis_modsum"]


def test_n65536_hash(golden_hash):
    h = golden_hash["n65536_i64"]
    qs = P.ntt_primes(h["bound"], h["N"], h["L"])
    p, perm, tw, itw, minv = P.ntt_tables(qs, h["N"])
    X = P.residues(h["seed"], h["shape"], qs)
    fw = ntt(X, p, perm, tw)
    assert sha(fw) == h["ntt"]
    assert np.array_equal(intt(fw, p, perm, itw, minv), X)


# ============================================================ oracle sweeps
NTT_CASES = [
    # (shape [l, m, r, k], dtype, prime bound)
    ((3, 2, 1, 2), np.int64, 2**30),
    ((2, 8, 2, 3), np.int64, 2**50),
    ((1, 64, 1, 5), np.int32, 2**30),
    ((2, 256, 3, 8), np.int64, 2**62),
    ((1, 1024, 1, 9), np.int32, 2**31),
    ((2, 2048, 1, 4), np.int64, 2**40),
    ((1, 8192, 1, 3), np.int64, 2**50),   # two passes (64 x 128)
    ((2, 8192, 1, 2), np.int32, 2**30),
    ((1, 16384, 2, 3), np.int64, 2**31),
]


@pytest.mark.parametrize("shape,dt,bound", NTT_CASES)
def test_ntt_intt_vs_oracle(shape, dt, bound):
    l, m, r, k = shape
    qs = P.ntt_primes(bound, max(m, 2), k)
    p, perm, tw, itw, minv = P.ntt_tables(qs, m, dt)
    a = P.residues(hash(shape) & 0xFFFF, shape, qs, dt)
    fw = ntt(a, p, perm, tw)
    assert np.array_equal(fw, O.ntt(a, p, perm, tw))
    back = intt(fw, p, perm, itw, minv)
    assert np.array_equal(back, a)
    assert np.array_equal(intt(a, p, perm, itw, minv), O.intt(a, p, perm, itw, minv, exact=1))


@pytest.mark.parametrize("m", [8192, 65536])
def test_two_pass_general_and_duplicate_perm(m):
    qs = P.ntt_primes(2**40, m, 2)
    p, _, tw, itw, minv = P.ntt_tables(qs, m)
    perm = np.argsort(P.splitmix64(m, m)).astype(np.int64)
    a = P.residues(5, (1, m, 1, 2), qs)
    assert np.array_equal(ntt(a, p, perm, tw), O.ntt(a, p, perm, tw))
    assert np.array_equal(intt(a, p, perm, itw, minv), O.intt(a, p, perm, itw, minv))
    dup = perm.copy()
    dup[5] = dup[11]
    prior = P.residues(6, (1, m, 1, 2), qs)
    assert np.array_equal(ntt(a, p, dup, tw), O.ntt(a, p, dup, tw))
    assert np.array_equal(intt(a, p, dup, itw, minv, prior=prior),
                          O.intt(a, p, dup, itw, minv, result=prior))


@pytest.mark.parametrize("m", [64, 8192])
def test_ntt_non_canonical_inputs(m):
    # values >= q and negative values take the reference's own arithmetic
    qs = P.ntt_primes(2**30, m, 2)
    p, perm, tw, itw, minv = P.ntt_tables(qs, m)
    a = P.uniform(9, (1, m, 1, 2), -(2**40), 2**40)
    b = P.uniform(10, (1, m, 1, 2), 0, 2**40)
    for x in (a, b):
        assert np.array_equal(ntt(x, p, perm, tw), O.ntt(x, p, perm, tw))
        assert np.array_equal(intt(x, p, perm, itw, minv), O.intt(x, p, perm, itw, minv))


def test_ntt_strided_input_and_in_place():
    m, k = 4096, 6
    qs = P.ntt_primes(2**50, m, k)
    p, perm, tw, itw, minv = P.ntt_tables(qs, m)
    limb_major = np.ascontiguousarray(np.moveaxis(P.residues(11, (2, m, k), qs), 2, 1))  # [2, k, m]
    view = np.moveaxis(limb_major, 1, 2)[:, :, None, :]                                 # [2, m, 1, k]
    assert not view.flags.c_contiguous
    want = O.ntt(np.ascontiguousarray(view), p, perm, tw)
    assert np.array_equal(ntt(view, p, perm, tw), want)
    # in place: result aliases a
    d = up(np.ascontiguousarray(view))
    capi.call("heal_ntt", d, up(p), up(perm), up(tw), None, None, d)
    assert np.array_equal(d.numpy(), want)
    capi.call("heal_intt", d, up(p), up(perm), up(itw), up(minv), None, None, d)
    assert np.array_equal(d.numpy(), view)


def test_ntt_errors():
    qs = P.ntt_primes(2**30, 8, 2)
    p, perm, tw, itw, minv = P.ntt_tables(qs, 8)
    a = P.residues(1, (1, 8, 1, 2), qs)
    with pytest.raises(ValueError):
        ntt(a.reshape(8, 2), p, perm, tw)
    with pytest.raises(ValueError):
        ntt(a, p[:1], perm, tw)
    with pytest.raises(ValueError):
        ntt(a, p, perm[:4], tw)
    with pytest.raises(ValueError):
        ntt(a, p, perm, tw[:, :4])
    bad = perm.copy()
    bad[3] = 8
    with pytest.raises(IndexError):
        ntt(a, p, bad, tw)
    with pytest.raises(IndexError):
        intt(a, p, perm, itw, minv[:1])


@pytest.mark.parametrize("dt", [np.int32, np.int64])
def test_modops_vs_oracle_random(dt):
    big = 2**31 if dt == np.int32 else 2**63
    shape = (3, 5, 7, 16)
    qs = np.array(P.ntt_primes(2**30 if dt == np.int32 else 2**62, 8, 16), dt)
    a = P.uniform(1, shape, 0, int(qs.min()), dt)
    b = P.uniform(2, shape, 0, int(qs.min()), dt)
    for f, o in [("heal_modmul_ttt", O.modmul), ("heal_modsum_ttt", O.modsum)]:
        assert np.array_equal(run(f, a, b, qs, out_shape=shape, dtype=dt), o(a, b, qs))
    an = P.uniform(3, shape, -big // 2, big // 2, dt)
    bn = P.uniform(4, (7, 1), -big // 2, big // 2, dt)
    for f, o in [("heal_modmul_ttt", O.modmul), ("heal_modsum_ttt", O.modsum)]:
        assert np.array_equal(run(f, an, bn, qs, out_shape=shape, dtype=dt), o(an, bn, qs, out_shape=shape))
    assert np.array_equal(run("heal_modneg_tt", an, qs, out_shape=shape, dtype=dt), O.modneg(an, qs))
    assert np.array_equal(run("heal_modneg_tc", a, 65537, out_shape=shape, dtype=dt), O.modneg(a, 65537))
    den = P.uniform(14, shape, -1000, 1000, dt)
    den[den == 0] = 3
    assert np.array_equal(run("heal_mod_tt", an, den, out_shape=shape, dtype=dt), O.mod(an, den))
    assert np.array_equal(run("heal_mod_tc", an, 97, out_shape=shape, dtype=dt), O.mod(an, 97))
    # odd sizes: a tail that is not a multiple of the 16-byte vector
    odd = P.uniform(5, (3, 7), 0, 1000, dt)
    assert np.array_equal(run("heal_modmul_ttc", odd, odd, 997, out_shape=odd.shape, dtype=dt),
                          O.modmul(odd, odd, 997))


def test_zero_size_and_aliasing():
    z = np.zeros((0, 4), np.int64)
    assert run("heal_modmul_ttt", z, z, np.array([7, 7, 7, 7]), out_shape=(0, 4), dtype=np.int64).shape == (0, 4)
    # result overlapping an input in another layout
    x = P.uniform(7, (4, 4), 0, 100)
    d = up(x)
    t = capi.DeviceArray(d.buf, np.int64, (4, 4), (1, 4))   # transposed view of the same buffer
    capi.call("heal_modsum_tcc", t, 1, 1000, d)
    assert np.array_equal(d.numpy(), (x.T + 1) % 1000)


def test_permute_and_axis_modsum_vs_oracle():
    for dt in (np.int32, np.int64):
        a = P.uniform(12, (2, 1024, 1, 24), 0, 2**30, dt)
        gal = P.galois_perm(1024, 5).reshape(1, 1024).astype(dt)
        assert np.array_equal(run("heal_permute", a, gal, 2, 1, out_shape=a.shape, dtype=dt), O.permute(a, gal, 2, 1))
        moved = np.moveaxis(P.uniform(13, (2, 64, 1, 5, 3), -2**20, 2**30, dt), 4, 3)
        p = np.array(P.ntt_primes(2**30, 8, 5), dt)
        got = run("heal_axis_modsum", up(np.ascontiguousarray(np.moveaxis(moved, 3, 4))).moveaxis(4, 3), p, 3,
                  out_shape=(2, 64, 1, 5), dtype=dt)
        assert np.array_equal(got, O.axis_modsum(moved, p, 3))


@pytest.mark.parametrize("m", [256, 8192])
def test_twiddle_rows_shared_only_when_equal(m):
    # rows 0, 1, 3 equal; row 2 equal to row 0 except one element; row 4 has
    # row 0's twiddles but another modulus: only truly equal rows may share
    q0, q1 = P.ntt_primes(2**50, m, 2)
    _, perm, tw, _, _ = P.ntt_tables([q0, q1], m)
    base = tw[0]
    rows = np.stack([base, base, base.copy(), base, base])
    rows[2, m // 3] = (rows[2, m // 3] + 1) % q0
    p = np.array([q0, q0, q0, q0, q1])
    a = P.residues(31, (2, m, 1, 5), p)
    assert np.array_equal(ntt(a, p, perm, rows), O.ntt(a, p, perm, rows))


@pytest.mark.parametrize("dt,bits,power", [(np.int32, 40, 2), (np.int32, 32, 3), (np.int32, 7, 5),
                                           (np.int64, 17, 3), (np.int64, 63, 2), (np.int64, 0, 2),
                                           (np.int64, 9, 12)])
def test_g_decomposition_vs_oracle(dt, bits, power):
    lim = 2**31 if dt == np.int32 else 2**63
    a = P.uniform(41, (3, 64, 1, 8), -lim // 2, lim // 2, dt)
    a.flat[:4] = [0, -1, 1, -lim // 2]
    want, _ = O.g_decomposition(a, power, bits)
    got = run("heal_g_decomposition", a, power, bits, out_shape=a.shape + (power,), dtype=dt)
    assert np.array_equal(got, want)
    # a strided input takes the general kernel
    v = np.ascontiguousarray(a.transpose(1, 0, 2, 3)).transpose(1, 0, 2, 3)
    got = run("heal_g_decomposition", v, power, bits, out_shape=a.shape + (power,), dtype=dt)
    assert np.array_equal(got, want)
    capi.synchronize()


def test_int32_31bit_columns_vs_oracle():
    # int32 residues under 31-bit primes: the reference's int32 NTT overflows
    # u + q - v here, so the oracle runs in its exact mode (double width)
    m, k = 65536, 4
    qs = P.ntt_primes(2**31, m, k)
    p, perm, tw, itw, minv = P.ntt_tables(qs, m, np.int32)
    a = P.residues(77, (2, m, 1, k), qs, np.int32)
    fw = ntt(a, p, perm, tw)
    assert np.array_equal(fw, O.ntt(a, p, perm, tw, exact=1))
    assert np.array_equal(intt(fw, p, perm, itw, minv), a)


@pytest.mark.parametrize("dt", [np.int32, np.int64])
@pytest.mark.parametrize("D", [2, 3, 4, 5])
def test_axis_modsum_over_innermost_digits(dt, D):
    """The digit axis of a [.., L, D] tensor moved before L: each output sums
    D adjacent values (the contiguous-block path for D <= 4), including
    negative and out-of-range values."""
    rng = np.random.default_rng(D)
    n, L = 64, 6
    p = np.array([97, 65521, 7, 3, 1 << 20 | 7, 2 ** 30 - 35][:L], dtype=dt)
    a = rng.integers(-50, 2 ** 30, size=(2, n, 1, L, D)).astype(dt)
    a[0, 3, 0, 2, :] = -9
    moved = np.moveaxis(a, 4, 3)                            # [2, n, 1, D, L], digits innermost in memory
    dev = capi.DeviceArray.from_numpy(a).reshape((2, n, 1, L, D)).moveaxis(4, 3)
    out = capi.DeviceArray.empty((2, n, 1, L), dt)
    capi.call("heal_axis_modsum", dev, up(p), out, 3)
    assert np.array_equal(out.numpy(), O.axis_modsum(np.ascontiguousarray(moved), p, 3))


@pytest.mark.parametrize("dt", [np.int32, np.int64])
@pytest.mark.parametrize("shape,ew,pa", [
    ((2, 64, 1, 24), 2, 1),      # the keyswitch chain's Galois permutation: whole rows
    ((3, 32, 8), 0, 1),          # elementwise axis before the permuted one
    ((16, 4, 6), 1, 0),          # elementwise axis inside the gathered rows
    ((5, 32, 3), 0, 1),          # rows of 3 elements: not whole 16-byte vectors
])
def test_permute_row_gathers(dt, shape, ew, pa):
    rng = np.random.default_rng(len(shape) + ew)
    a = rng.integers(-1000, 1 << 30, size=shape).astype(dt)
    l, m = shape[ew], shape[pa]
    perms = np.stack([rng.permutation(m) for _ in range(l)]).astype(dt)
    out = capi.DeviceArray.empty(shape, dt)
    capi.call("heal_permute", up(a), up(perms), out, ew, pa)
    assert np.array_equal(out.numpy(), O.permute(a, perms, ew, pa))


@pytest.mark.parametrize("dt", [np.int32, np.int64])
@pytest.mark.parametrize("n,in_place", [(1 << 18, False), ((1 << 18) + 24, True), ((1 << 20) + 8, False)])
def test_large_dense_modops_vs_oracle(dt, n, in_place):
    """Large dense operands (many grid-stride iterations, a length that is
    not a multiple of the grid), in place and out of place, with moduli on
    the last axis and signed values."""
    rng = np.random.default_rng(n + in_place)
    k = 24
    p = np.array([97, 65521, 2 ** 30 - 35, 7, 3, 2 ** 31 - 1] * 4, dtype=dt)[:k]
    shape = (n // k, k)
    a = rng.integers(-2 ** 20, 2 ** 31 - 1, size=shape).astype(dt)
    b = rng.integers(0, 2 ** 31 - 1, size=shape).astype(dt)
    for name, op in (("heal_modmul_ttt", O.modmul), ("heal_modsum_ttt", O.modsum)):
        da, db = up(a), up(b)
        out = da if in_place else capi.DeviceArray.empty(shape, dt)
        capi.call(name, da, db, up(p), out)
        assert np.array_equal(out.numpy(), op(a, b, p)), name
    capi.synchronize()


@pytest.mark.parametrize("m", [16, 4096, 1 << 14])
def test_ntt_permutation_one_swap_from_bit_reversal(m):
    """A permutation that differs from bit reversal in two entries must not be
    taken for it (the kernels compute bit reversal instead of loading it)."""
    k = 3
    qs = P.ntt_primes(1 << 50, m, k)
    p, perm, tw, itw, minv = P.ntt_tables(qs, m)
    swapped = perm.copy()
    swapped[[1, m - 2]] = swapped[[m - 2, 1]]
    x = P.residues(m, (2, m, 1, k), qs)
    for pm in (perm, swapped):
        assert np.array_equal(ntt(x, p, pm, tw), O.ntt(x, p, pm, tw))
        y = O.ntt(x, p, pm, tw)
        assert np.array_equal(intt(y, p, pm, itw, minv), O.intt(y, p, pm, itw, minv))


@pytest.mark.parametrize("dt", [np.int32, np.int64])
def test_broadcast_and_strided_modops_in_vector_units(dt):
    """Results contiguous on their innermost axis with operands contiguous or
    broadcast there (moved 16 bytes at a time), beside the cases that must
    stay element by element: an operand at an odd element offset, an odd
    innermost length, a strided innermost axis."""
    rng = np.random.default_rng(7 if dt == np.int32 else 8)
    hi = 2 ** 30 if dt == np.int32 else 2 ** 62
    L, N = 16, 256
    qs = np.array(P.ntt_primes(hi, 8, L), dt)
    lo = int(qs.min())
    ct = rng.integers(0, lo, size=(2, N, 1, L)).astype(dt)
    pt = rng.integers(0, lo, size=(N, 1, L)).astype(dt)
    for f, o in [("heal_modmul_ttt", O.modmul), ("heal_modsum_ttt", O.modsum)]:
        # plaintext broadcast over the two polynomials, and the reverse roles
        assert np.array_equal(run(f, ct, pt, qs, out_shape=ct.shape, dtype=dt), o(ct, pt, qs, out_shape=ct.shape)), f
        assert np.array_equal(run(f, pt, ct, qs, out_shape=ct.shape, dtype=dt), o(pt, ct, qs, out_shape=ct.shape)), f
    # a stack of rotations times its diagonals: [d, 2, N/d, d, L] x [d, 1, 1, d, L]
    d = 4
    stack = rng.integers(0, lo, size=(d, 2, N // d, d, L)).astype(dt)
    diag = rng.integers(0, lo, size=(d, 1, 1, d, L)).astype(dt)
    want = O.modmul(stack, diag, qs, out_shape=stack.shape)
    assert np.array_equal(run("heal_modmul_ttt", stack, diag, qs, out_shape=stack.shape, dtype=dt), want)
    ds = up(stack)  # in place, as the three-call product runs
    capi.call("heal_modmul_ttt", ds, up(diag), up(qs), ds)
    assert np.array_equal(ds.numpy(), want)
    # a transposed operand (outer axes swapped, limbs still contiguous), a scalar b, negation
    x = rng.integers(-hi, hi, size=(N, 2, L)).astype(dt)
    xt = up(x).moveaxis(1, 0)
    xn = np.ascontiguousarray(np.moveaxis(x, 1, 0))
    assert np.array_equal(run("heal_modmul_ttt", xt, up(ct.reshape(2, N, L)), up(qs), out_shape=(2, N, L), dtype=dt),
                          O.modmul(xn, ct.reshape(2, N, L), qs))
    assert np.array_equal(run("heal_modmul_tct", xt, 12345, up(qs), out_shape=(2, N, L), dtype=dt),
                          O.modmul(xn, 12345, qs))
    assert np.array_equal(run("heal_modneg_tt", xt, up(qs), out_shape=(2, N, L), dtype=dt), O.modneg(xn, qs))
    den = rng.integers(1, 1000, size=(2, N, L)).astype(dt)
    assert np.array_equal(run("heal_mod_tt", xt, up(den), out_shape=(2, N, L), dtype=dt), O.mod(xn, den))
    # moduli per row and limb ([N, L] broadcast over the polynomials), and one modulus broadcast along the limbs
    prow = rng.integers(lo // 2, lo, size=(N, 1, L)).astype(dt)
    assert np.array_equal(run("heal_modmul_ttt", ct, pt, prow, out_shape=ct.shape, dtype=dt),
                          O.modmul(ct, pt, prow, out_shape=ct.shape))
    p1 = qs[:1].copy()
    assert np.array_equal(run("heal_modsum_ttt", ct, pt, p1, out_shape=ct.shape, dtype=dt),
                          O.modsum(ct, pt, p1, out_shape=ct.shape))
    # one element off the 16-byte grid: the element-wise kernel
    buf = up(np.concatenate([np.zeros(1, dt), pt.ravel()]))
    off = capi.DeviceArray(buf.buf, dt, (N, 1, L), None, np.dtype(dt).itemsize)
    assert np.array_equal(run("heal_modmul_ttt", up(ct), off, up(qs), out_shape=ct.shape, dtype=dt),
                          O.modmul(ct, pt, qs, out_shape=ct.shape))
    # an odd number of limbs, and limbs taken every other element
    q3 = qs[:3].copy()
    c3 = np.ascontiguousarray(ct[..., :3])
    p3 = np.ascontiguousarray(pt[..., :3])
    assert np.array_equal(run("heal_modmul_ttt", c3, p3, q3, out_shape=c3.shape, dtype=dt),
                          O.modmul(c3, p3, q3, out_shape=c3.shape))
    wide = up(np.repeat(pt, 2, axis=2))
    half = capi.DeviceArray(wide.buf, dt, (N, 1, L), (2 * L, 2 * L, 2))
    assert np.array_equal(run("heal_modmul_ttt", up(ct), half, up(qs), out_shape=ct.shape, dtype=dt),
                          O.modmul(ct, pt, qs, out_shape=ct.shape))


@pytest.mark.parametrize("dt", [np.int32, np.int64])
def test_permute_strided_sources_in_vector_units(dt):
    """A ciphertext expanded over a stack of rotations (stride 0 on the
    elementwise axis) and a transposed source: limbs move 16 bytes at a time.
    An odd element offset stays element by element."""
    rng = np.random.default_rng(11)
    d, N, L = 8, 512, 16
    ct = rng.integers(-1000, 1 << 30, size=(2, N, L)).astype(dt)
    perms = np.stack([rng.permutation(N) for _ in range(d)]).astype(dt)
    src = up(ct).reshape((1, 2, N, L)).expand(0, d)
    want = O.permute(np.ascontiguousarray(np.broadcast_to(ct[None], (d, 2, N, L))), perms, 0, 2)
    assert np.array_equal(run("heal_permute", src, up(perms), 0, 2, out_shape=(d, 2, N, L), dtype=dt), want)
    x = rng.integers(0, 1 << 30, size=(N, 2, L)).astype(dt)
    p2 = np.stack([rng.permutation(N) for _ in range(2)]).astype(dt)
    xt = up(x).moveaxis(1, 0)
    assert np.array_equal(run("heal_permute", xt, up(p2), 0, 1, out_shape=(2, N, L), dtype=dt),
                          O.permute(np.ascontiguousarray(np.moveaxis(x, 1, 0)), p2, 0, 1))
    buf = up(np.concatenate([np.zeros(1, dt), x.ravel()]))
    off = capi.DeviceArray(buf.buf, dt, (N, 2, L), None, np.dtype(dt).itemsize).moveaxis(1, 0)
    assert np.array_equal(run("heal_permute", off, up(p2), 0, 1, out_shape=(2, N, L), dtype=dt),
                          O.permute(np.ascontiguousarray(np.moveaxis(x, 1, 0)), p2, 0, 1))


# ------------------------------------------- 64-bit growing-range boundaries
# The 64-bit transforms skip per-butterfly reductions while the modulus leaves
# headroom: forward for q < 2^56 (values stay below (1 + 4 log2 m) q), an
# inverse pass of P stages for q < 2^(62 - P) (values below 2^(P+1) q).
# Primes just below and just above each threshold, with pass splits that move
# the inverse's pass lengths across them.
GROW_CASES = [
    # (m, prime bound, first-pass log2 per call: 0 = one pass)
    (1 << 16, 2**57, (8, 4, 12)),    # above the forward's threshold: lazy ranges in both directions
    (1 << 16, 2**56, (8, 4, 12)),    # forward grows to 65q < 2^62.1; inverse passes: lazy ranges
    (1 << 16, 2**54, (8, 4, 12)),    # 8-stage inverse passes grow; 12-stage ones do not
    (1 << 16, 2**55, (8, 4, 12)),    # 8-stage inverse passes just above their threshold
    (1 << 16, 2**50, (8, 4, 12)),    # every pass grows
    (4096, 2**50, (0, 6)),           # one 12-stage pass at its inverse threshold
    (4096, 2**51, (0, 6)),
    (1 << 20, 2**56, (10, 8)),       # the forward's longest tested chain: 81q < 2^62.4
]


@pytest.mark.parametrize("m,bound,splits", GROW_CASES)
def test_ntt_growing_range_thresholds(m, bound, splits):
    k = 2
    qs = P.ntt_primes(bound, m, k)
    qs[1] = P.ntt_primes(2**40, m, 1)[0]        # mixed widths: the largest modulus picks the mode
    p, perm, tw, itw, minv = P.ntt_tables(qs, m)
    a = P.residues(m ^ bound.bit_length(), (1, m, 1, k), qs)
    want = O.ntt(a, p, perm, tw)
    code = capi.DTYPES[np.dtype(np.int64)]
    dx, dp, dperm, dtw, ditw, dminv, dwant = (up(v) for v in (a, p, perm, tw, itw, minv, want))
    out = capi.DeviceArray.empty(a.shape, np.int64)
    try:
        for s in splits:
            for inv in (0, 1):
                capi.check(capi.lib().heal_ntt_set_plan(code, inv, m, k, 4, s))
            capi.call("heal_ntt", dx, dp, dperm, dtw, None, None, out)
            assert np.array_equal(out.numpy(), want), s
            capi.call("heal_intt", dwant, dp, dperm, ditw, dminv, None, None, out)
            assert np.array_equal(out.numpy(), a), s
    finally:
        capi.check(capi.lib().heal_ntt_clear_plans())


@pytest.mark.parametrize("m", [8192, 1 << 16])
def test_two_pass_negative_values_beside_unreduced_tiles(m):
    # a few negative inputs send some first-pass tiles to the reference's
    # arithmetic while their neighbours hand unreduced values to the second pass
    qs = P.ntt_primes(2**50, m, 3)
    p, perm, tw, itw, minv = P.ntt_tables(qs, m)
    a = P.residues(21, (2, m, 1, 3), qs)
    a[0, 5, 0, 1] = -7
    a[1, m // 2 + 3, 0, 2] = -(2**45)
    a[1, 17, 0, 0] = 2**55                      # non-negative, above q: reduced on load
    assert np.array_equal(ntt(a, p, perm, tw), O.ntt(a, p, perm, tw))
    assert np.array_equal(intt(a, p, perm, itw, minv), O.intt(a, p, perm, itw, minv, exact=1))


def test_butterfly_peak_diagnostic():
    import ctypes
    rate = ctypes.c_double()
    L = capi.lib()
    capi.check(L.heal_ntt_butterfly_peak(16, ctypes.byref(rate)))
    assert 1e10 < rate.value < 1e14              # butterflies per second on one GPU
    assert L.heal_ntt_butterfly_peak(0, ctypes.byref(rate)) == 1
    assert L.heal_ntt_butterfly_peak(16, None) == 1


@pytest.mark.parametrize("m", [8192, 1 << 16])
@pytest.mark.parametrize("bounds", [(2**32,), (2**32 + 2**26,), (2**32 + 2**26, 2**32)],
                         ids=["below_2_32", "above_2_32", "mixed"])
def test_growing_range_reduction_around_2_32(m, bounds):
    """Each growing-range pass that reduces ends with a Shoup product by 1;
    when every modulus is above 2^32 its companion floor(2^64 / q) fits in
    32 bits and the high product is the short one.  Moduli just below 2^32
    (the long product), just above (the short one), and both in one call
    (the long one for all) against the oracle, both directions."""
    qs = np.concatenate([np.asarray(P.ntt_primes(b, m, 2), np.int64) for b in bounds])
    assert (qs > 2**31).all() and (qs < 2**33).all()
    p, perm, tw, itw, minv = P.ntt_tables(qs, m)
    a = P.residues(m + len(bounds), (2, m, 1, len(qs)), qs)
    fw = ntt(a, p, perm, tw)
    assert np.array_equal(fw, O.ntt(a, p, perm, tw))
    assert np.array_equal(intt(fw, p, perm, itw, minv), a)
    assert np.array_equal(intt(a, p, perm, itw, minv), O.intt(a, p, perm, itw, minv, exact=1))
