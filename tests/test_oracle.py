"""Pins the CPU oracle (oracle/heal_oracle.c) to HEAL's own sample
implementation: every golden array was produced by the reference's
example_impl (tests/golden/make_golden.py), plus the literal tables of the
reference's GoogleTest suite.  No GPU needed."""
import hashlib

import numpy as np
import pytest

from heal_gb300 import params as P
from oracle import oracle as O


def sha(x):
    return hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest()


@pytest.mark.parametrize("exact", [0, 1])
def test_ntt_pin_tables(golden, exact):
    # tests/test_ntt.cpp:9-28 — round trip with p = {17, 257}
    g = golden("ntt_pin")
    fw = O.ntt(g["a"], g["p"], g["perm"], g["tw"], exact=exact)
    assert np.array_equal(fw, g["ntt"])
    back = O.intt(fw, g["p"], g["perm"], g["itw"], g["minv"], exact=exact)
    assert np.array_equal(back, g["intt"]) and np.array_equal(back, g["a"])


@pytest.mark.parametrize("case", ["ntt_i64", "ntt_i64_m1", "ntt_i64_m2", "ntt_i64_m4096", "ntt_i32",
                                  "ntt_neg"])
@pytest.mark.parametrize("exact", [0, 1])
def test_ntt_intt_vs_reference(golden, case, exact):
    g = golden(case)
    assert np.array_equal(O.ntt(g["a"], g["p"], g["perm"], g["tw"], exact=exact), g["ntt"])
    src = g["ntt"] if "intt_a" in g else g["a"]
    got = O.intt(src, g["p"], g["perm"], g["itw"], g["minv"], exact=exact)
    width = 31 if g["a"].dtype == np.int32 else 63
    # the reference scales by m_inv in the element type (ntt_impl.cpp:165);
    # it is exact only while q^2 < 2^(width)
    if not exact or int(g["p"].max()) ** 2 < 2 ** width:
        assert np.array_equal(got, g["intt"])
    if "intt_a" in g:
        if not exact or int(g["p"].max()) ** 2 < 2 ** width:
            assert np.array_equal(O.intt(g["a"], g["p"], g["perm"], g["itw"], g["minv"], exact=exact), g["intt_a"])
        if exact:
            assert np.array_equal(got, g["a"])   # exact INTT inverts the reference's NTT


def test_ntt_negative_twiddles(golden):
    g = golden("ntt_negtw")
    for exact in (0, 1):
        assert np.array_equal(O.ntt(g["a"], g["p"], g["perm"], g["tw"], exact=exact), g["ntt"])


def test_ntt_general_and_duplicate_perm(golden):
    g = golden("ntt_perm")
    assert np.array_equal(O.ntt(g["a"], g["p"], g["perm"], g["tw"]), g["ntt"])
    assert np.array_equal(O.intt(g["a"], g["p"], g["perm"], g["itw"], g["minv"]), g["intt"])
    assert np.array_equal(O.ntt(g["a"], g["p"], g["dup"], g["tw"]), g["ntt_dup"])
    # the scatter leaves the result's previous contents (zeros) where no index lands
    assert np.array_equal(O.intt(g["a"], g["p"], g["dup"], g["itw"], g["minv"]), g["intt_dup"])


def test_keyswitch_n256_chain(golden):
    g = golden("keyswitch_n256")
    p, perm, tw, itw, minv = g["p"], g["perm"], g["tw"], g["itw"], g["minv"]
    assert np.array_equal(O.ntt(g["ct"], p, perm, tw), g["ntt_ct"])
    # the reference's single-width m_inv scaling overflows at 50-bit q: the
    # literal mode reproduces it, the exact mode does not
    lit = O.intt(g["ct"], p, perm, itw, minv, exact=0)
    assert np.array_equal(lit, g["intt_ct_literal"])
    ex = O.intt(g["ct"], p, perm, itw, minv, exact=1)
    assert not np.array_equal(ex, lit)
    assert np.array_equal(O.ntt(ex, p, perm, tw), g["ct"])      # exact INTT inverts NTT
    assert ((ex >= 0) & (ex < p)).all()
    d, warns = O.g_decomposition(g["coef"], 3, 17)
    assert np.array_equal(d, g["digits"]) and warns == 0
    L, D = len(p), 3
    qs_t = np.repeat(p, D)
    dn = O.ntt(g["digits"].reshape(2, -1, 1, L * D), qs_t, perm, np.repeat(tw, D, axis=0))
    assert np.array_equal(dn, g["dn"])
    prod = O.modmul(dn, g["key"], qs_t)
    assert np.array_equal(prod, g["prod"])
    acc = O.axis_modsum(np.moveaxis(prod.reshape(2, -1, 1, L, D), 4, 3), p, 3)
    assert np.array_equal(acc, g["acc"])
    assert np.array_equal(O.permute(acc, g["gal"], 2, 1), g["rot"])


@pytest.mark.parametrize("tag,dt", [("32", np.int32), ("64", np.int64)])
@pytest.mark.parametrize("op", ["modmul", "modsum"])
def test_modops_vs_reference(golden, tag, dt, op):
    g = golden(f"{op}_{tag}")
    f = O.modmul if op == "modmul" else O.modsum
    assert np.array_equal(f(g["a"], g["b"], g["p"]), g["ttt"])
    assert np.array_equal(f(g["an"], g["bn"], g["pn"]), g["ttt_neg"])
    assert np.array_equal(f(g["at"], g["at"], g["p"]), g["ttt_strided"])
    assert np.array_equal(f(g["col"], g["row"], g["prow"], out_shape=(2, 3)), g["ttt_bcast"])
    assert np.array_equal(f(g["an"], g["bn"], 1000003), g["ttc"])
    assert np.array_equal(f(g["an"], -12345, g["pn"]), g["tct"])
    assert np.array_equal(f(g["an"], 98765, 4099), g["tcc"])


@pytest.mark.parametrize("tag", ["32", "64"])
def test_axis_modsum_vs_reference(golden, tag):
    g = golden(f"axis_modsum_{tag}")
    for ax in (0, 1, 2):
        assert np.array_equal(O.axis_modsum(g["a"], g["p"], ax, exact=0), g[f"ax{ax}"])
    dt = g["a"].dtype
    # sequential truncating reduction: (5 + 5) % 7 = 3, (3 - 8) % 7 = -5
    seq = O.axis_modsum(np.array([[5], [5], [-8]], dt), np.array([7], dt), 0)
    assert np.array_equal(seq, g["seq"]) and seq.tolist() == [-5]


@pytest.mark.parametrize("tag", ["32", "64"])
def test_g_decomposition_vs_reference(golden, tag):
    g = golden(f"gdec_{tag}")
    for key, (pw, bits) in {"b3p4": (4, 3), "b17p3": (3, 17), "b1p40": (40, 1)}.items():
        d, _ = O.g_decomposition(g["a"], pw, bits)
        assert np.array_equal(d, g[key]), key


@pytest.mark.parametrize("tag", ["32", "64"])
def test_permute_vs_reference(golden, tag):
    g = golden(f"permute_{tag}")
    assert np.array_equal(O.permute(g["a"], g["perms_a"], 1, 2), g["r12"])
    assert np.array_equal(O.permute(g["a"], g["perms_b"], 0, 3), g["r03"])


def test_roundtrip_full_size_hashes(golden_hash):
    h = golden_hash["roundtrip_n4096"]
    qs = P.ntt_primes(h["bound"], h["N"], h["L"])
    p, perm, tw, itw, minv = P.ntt_tables(qs, h["N"])
    A = P.residues(h["seeds"][0], h["shape"], qs)
    B = P.residues(h["seeds"][1], h["shape"], qs)
    NA = O.ntt(A, p, perm, tw)
    assert sha(NA) == h["ntt_a"]
    NB = O.ntt(B, p, perm, tw)
    assert sha(NB) == h["ntt_b"]
    assert sha(O.intt(NA, p, perm, itw, minv)) == h["intt_ntt_a"]
    PR = O.modmul(NA, NB, p)
    assert sha(PR) == h["modmul"]
    assert sha(O.axis_modsum(PR, p, 0)) == h["axis_modsum"]


# ---- literal tables of the reference's GoogleTest suite ----

def test_g_decomposition_literal_tables():
    # tests/test_g_decomposition.cpp:16-21 and :47-56
    d, _ = O.g_decomposition(np.array([0, 1, 2, 3], np.int32), 2, 1)
    assert d.tolist() == [[0, 0], [1, 0], [0, 1], [1, 1]]
    a = np.array([[[5, 12], [3, 1]], [[8, 7], [9, 2]]], np.int32)
    d, _ = O.g_decomposition(a, 3, 2)
    assert d.tolist() == [[[[1, 1, 0], [0, 3, 0]], [[3, 0, 0], [1, 0, 0]]],
                          [[[0, 2, 0], [3, 1, 0]], [[1, 2, 0], [2, 0, 0]]]]
    d, w = O.g_decomposition(np.array([255], np.int32), 3, 3)
    assert w == 0 and d.tolist() == [[7, 7, 3]]


def test_decomp_reconstruct_round_trip():
    # tests/test_decomp_reconstruct.cpp:7-38
    a = np.array([51, 29, 63], np.int32)
    d, _ = O.g_decomposition(a, 6, 1)
    d = O.modmul(d, np.array([1, 2, 4, 8, 16, 32], np.int32), np.array([1024] * 6, np.int32))
    r = O.axis_modsum(d.reshape(3, 6, 1), np.array([1024], np.int32), 1)
    assert r.reshape(3).tolist() == a.tolist()


def test_modop_literal_cases():
    # tests/test_modop.cpp:102-188
    a = np.array([[1, 2], [3, 4]], np.int32)
    assert O.modsum(a, 5, 6).tolist() == ((a + 5) % 6).tolist()
    assert O.modmul(a, 5, np.array([6, 7], np.int32)).tolist() == ((a * 5) % np.array([6, 7])).tolist()
    assert O.modsum(np.array([[10, 20]], np.int32), 3, np.array([4, 5], np.int32)).tolist() == [[1, 3]]
    r = O.modmul(np.array([[1], [2]], np.int32), np.array([10, 20, 30], np.int32), np.array([11, 17, 23], np.int32),
                 out_shape=(2, 3))
    assert r.tolist() == [[10, 3, 7], [9, 6, 14]]
    with pytest.raises(ValueError):
        O.modsum(np.zeros((2, 3), np.int32), np.zeros((2, 4), np.int32), np.arange(3, dtype=np.int32))
    with pytest.raises(ValueError):
        O.modsum(np.zeros((2, 3), np.int32), np.zeros((2, 3), np.int32), np.zeros((4, 1), np.int32))


def test_mod_literal_cases():
    # tests/test_modop.cpp:224-486
    a = np.array([[5, 7, 9], [10, 12, 14]], np.int64)
    b = np.array([[3, 5, 7], [4, 6, 8]], np.int64)
    assert O.mod(a, b).tolist() == (a % b).tolist()
    assert O.mod(a, 6).tolist() == (a % 6).tolist()
    assert O.mod(6, b).tolist() == (6 % b).tolist()
    assert O.mod(0, np.array([[1, 2], [3, 4]], np.int64)).tolist() == [[0, 0], [0, 0]]
    with pytest.raises(ValueError):
        O.mod(np.zeros((2, 3), np.int64), np.zeros((2, 2), np.int64))
    # C's truncating remainder, not Python's floor remainder
    assert O.mod(np.array([-7], np.int64), 3).tolist() == [-1]


def test_axis_modsum_literal_cases():
    # tests/test_axis_modsum.cpp:7-85
    a = np.arange(1, 25, dtype=np.int32).reshape(2, 3, 4)
    p = np.array([11, 13, 17, 19], np.int32)
    assert O.axis_modsum(a, p, 1).tolist() == (a.sum(1) % p).tolist()
    with pytest.raises(ValueError):
        O.axis_modsum(np.zeros((2, 2, 2), np.int32), np.array([7, 11], np.int32), -1)
    with pytest.raises(ValueError):
        O.axis_modsum(np.zeros((2, 2, 2), np.int32), np.array([7, 11], np.int32), 3)
    with pytest.raises(ValueError):
        O.axis_modsum(np.zeros((2, 2, 2), np.int32), np.array([7, 11, 13], np.int32), 2)


def test_permute_errors():
    # tests/test_permute.cpp:64-84
    a = np.zeros((2, 3, 4), np.int32)
    perms = np.zeros((2, 3), np.int32)
    for ew, pa in [(3, 1), (1, 1), (0, 3)]:
        with pytest.raises(ValueError):
            O.permute(a, perms, ew, pa)
    with pytest.raises(IndexError):
        O.permute(a, np.array([[0, 1, 3], [1, 2, 0]], np.int32), 0, 1)


def test_oracle_matches_reference_on_seeded_random_cases():
    """oracle/crosscheck_ref.py: the oracle's literal mode against HEAL's own
    example_impl (compiled from its sources into oracle/_ref/) on seeded
    random shapes, tables and signed inputs of every op. The reference's
    pybind module runs in its own process: it registers DeviceTensor types
    under the same names as this backend's module."""
    import glob
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if not glob.glob(os.path.join(root, "oracle", "_ref", "lattica_hw*.so")):
        pytest.skip("the reference's sample implementation is not built here (oracle/build_ref.sh)")
    p = subprocess.run([sys.executable, os.path.join(root, "oracle", "crosscheck_ref.py"), "24"],
                       capture_output=True, text=True, cwd=root)
    assert p.returncode == 0, p.stdout[-2000:] + p.stderr[-2000:]
    assert "bit-exact against the reference" in p.stdout


@pytest.mark.parametrize("dt,bits,m", [(np.int64, 50, 64), (np.int64, 50, 256), (np.int64, 62, 32),
                                       (np.int32, 31, 64), (np.int32, 31, 256)])
def test_exact_mode_is_the_negacyclic_transform(dt, bits, m):
    """The exact mode (the GPU's contract) checked without the reference, in
    Python integers: where the reference overflows (50-bit INTT, 31-bit int32
    NTT and INTT) the forward transform is the natural-order negacyclic DFT
    out[i] = sum_j a[j] psi^((2i+1) j) mod q, and intt(ntt(a)) = a."""
    k = 2
    qs = P.ntt_primes(1 << bits, m, k)
    p, perm, tw, itw, minv = P.ntt_tables(qs, m, dtype=dt)
    a = P.residues(31 + m, (1, m, 1, k), qs, dt)
    fwd = O.ntt(a, p, perm, tw, exact=True)
    for t, q in enumerate(qs):
        psi = P.psi(q, m)
        x = [int(v) for v in a[0, :, 0, t]]
        want = [sum(x[j] * pow(psi, (2 * i + 1) * j, q) for j in range(m)) % q for i in range(m)]
        assert [int(v) for v in fwd[0, :, 0, t]] == want, (q, t)
    assert np.array_equal(O.intt(fwd, p, perm, itw, minv, exact=True), a)


@pytest.mark.parametrize("dt,bits", [(np.int32, 31), (np.int64, 62)])
def test_exact_axis_modsum_in_python_integers(dt, bits):
    """axis_modsum's exact mode: the reference's running truncated sum
    sum = (sum + a_r) % q, taken in Python integers (no wraparound), for
    moduli whose 2q exceeds the element type (31-bit int32, 62-bit int64)."""
    k = 3
    qs = P.ntt_primes(1 << bits, 8, k)
    a = P.residues(7, (5, 4, k), qs, dt)
    a[1] -= np.asarray(qs, dt)      # some negative terms: the truncated % keeps their sign
    got = O.axis_modsum(a, np.asarray(qs, dt), 0, exact=True)

    def trunc_mod(x, q):
        r = abs(x) % q
        return r if x >= 0 else -r

    for i in range(4):
        for t, q in enumerate(qs):
            s = 0
            for r in range(5):
                s = trunc_mod(s + int(a[r, i, t]), q)
            assert int(got[i, t]) == s, (i, t)


def test_wraparound_cases_pin_the_literal_mode(golden):
    """The reference's own outputs where its element-type sums wrap: the int32
    NTT / INTT at 31-bit moduli (ntt_impl.cpp:106-107,155-157,165) and
    axis_modsum's running sum at moduli near 2^31 and 2^63
    (axis_modsum_impl.cpp:70).  The literal mode reproduces them; the exact
    mode does not."""
    g = golden("ntt_i32_q31")
    args = (g["p"], g["perm"], g["itw"], g["minv"])
    assert np.array_equal(O.ntt(g["a"], g["p"], g["perm"], g["tw"], exact=False), g["ntt"])
    assert np.array_equal(O.intt(g["ntt"], *args, exact=False), g["intt"])
    assert np.array_equal(O.intt(g["a"], *args, exact=False), g["intt_a"])
    assert not np.array_equal(O.ntt(g["a"], g["p"], g["perm"], g["tw"], exact=True), g["ntt"])
    for tag in ("32", "64"):
        g = golden(f"axis_modsum_wrap_{tag}")
        for ax in (0, 1):
            assert np.array_equal(O.axis_modsum(g["a"], g["p"], ax, exact=False), g[f"ax{ax}"])
            assert not np.array_equal(O.axis_modsum(g["a"], g["p"], ax, exact=True), g[f"ax{ax}"])
