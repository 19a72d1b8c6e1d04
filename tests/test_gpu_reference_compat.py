"""Reference-compatibility mode (heal_set_reference_compat).  With it on, the
GPU reproduces the sample implementation's wraparound in the element type:
the INTT's single-width m^-1 scaling (ntt_impl.cpp:165, every int64 modulus
above about 2^31.5), the int32 butterflies at moduli of 2^30 and above
(ntt_impl.cpp:106-107,155-157) and axis_modsum's running sum
(axis_modsum_impl.cpp:70).  Its outputs then equal the reference's own
outputs (tests/golden/, written by the compiled example_impl) and the
oracle's literal mode bit for bit, also where the exact results differ;
with it off the exact results return."""
import numpy as np
import pytest

from heal_gb300 import capi
from heal_gb300 import params as P
from oracle import oracle as O
from _gpu import intt, ntt, ready, run

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def gpu():
    return ready()


@pytest.fixture
def compat():
    lib = capi.lib()
    capi.check(lib.heal_set_reference_compat(1))
    assert lib.heal_get_reference_compat() == 1
    try:
        yield
    finally:
        capi.check(lib.heal_set_reference_compat(0))


@pytest.mark.parametrize("case", ["ntt_i64", "ntt_i64_m1", "ntt_i64_m2", "ntt_i64_m4096", "ntt_i32", "ntt_i32_q31",
                                  "ntt_neg", "ntt_pin"])
def test_golden_transforms_equal_the_reference_outputs(golden, compat, case):
    """Every golden transform, the INTTs whose 40-bit scaling overflows in
    the reference included (the exact mode skips those)."""
    g = golden(case)
    assert np.array_equal(ntt(g["a"], g["p"], g["perm"], g["tw"]), g["ntt"])
    # the stored intt is of the NTT output where intt_a is stored too, and for the
    # round-trip pin (tests/test_ntt.cpp); of `a` otherwise
    src = g["ntt"] if "intt_a" in g or case == "ntt_pin" else g["a"]
    assert np.array_equal(intt(src, g["p"], g["perm"], g["itw"], g["minv"]), g["intt"])
    if "intt_a" in g:
        assert np.array_equal(intt(g["a"], g["p"], g["perm"], g["itw"], g["minv"]), g["intt_a"])


@pytest.mark.parametrize("tag,dt", [("32", np.int32), ("64", np.int64)])
def test_golden_axis_modsum_wrap_equals_the_reference(golden, compat, tag, dt):
    g = golden(f"axis_modsum_wrap_{tag}")
    for ax in (0, 1):
        shape = tuple(d for i, d in enumerate(g["a"].shape) if i != ax)
        assert np.array_equal(run("heal_axis_modsum", g["a"], g["p"], ax, out_shape=shape, dtype=dt), g[f"ax{ax}"])


def test_keyswitch_intt_overflow_equals_the_reference(golden, compat):
    g = golden("keyswitch_n256")
    got = intt(g["ct"], g["p"], g["perm"], g["itw"], g["minv"])
    assert np.array_equal(got, g["intt_ct_literal"])
    assert (got < 0).any()  # the reference's wrapped scaling leaves negative residues


def test_off_restores_the_exact_results(golden):
    g = golden("keyswitch_n256")
    capi.check(capi.lib().heal_set_reference_compat(0))
    got = intt(g["ct"], g["p"], g["perm"], g["itw"], g["minv"])
    assert np.array_equal(got, O.intt(g["ct"], g["p"], g["perm"], g["itw"], g["minv"], exact=True))
    assert not np.array_equal(got, g["intt_ct_literal"])


# (shape [l, m, r, k], dtype, prime bound): 31-bit int32 moduli wrap the butterflies' sums; 50-bit and
# near-2^63 int64 moduli wrap the INTT scaling (and, near 2^63, the sums); one and two passes
LITERAL_CASES = [
    ((2, 1024, 1, 3), np.int32, 2**31),
    ((1, 8192, 1, 2), np.int32, 2**31),
    ((2, 4096, 1, 3), np.int64, 2**50),
    ((1, 8192, 1, 2), np.int64, 2**50),
    ((2, 256, 1, 2), np.int64, 2**63),
    ((1, 1 << 16, 1, 2), np.int32, 2**31),   # two 256-point passes: the staged int32 kernel's exact path
]


@pytest.mark.parametrize("shape,dt,bound", LITERAL_CASES)
def test_transforms_equal_the_oracle_literal_mode(compat, shape, dt, bound):
    l, m, r, k = shape
    qs = P.ntt_primes(bound, m, k)
    p, perm, tw, itw, minv = P.ntt_tables(qs, m, dt)
    a = P.residues(m + k, shape, qs, dt)
    want = O.ntt(a, p, perm, tw, exact=False)
    fw = ntt(a, p, perm, tw)
    assert np.array_equal(fw, want)
    assert np.array_equal(intt(a, p, perm, itw, minv), O.intt(a, p, perm, itw, minv, exact=False))
    assert np.array_equal(intt(fw, p, perm, itw, minv), O.intt(want, p, perm, itw, minv, exact=False))
    # the case is one where the reference overflows somewhere
    assert not (np.array_equal(want, O.ntt(a, p, perm, tw, exact=True)) and
                np.array_equal(O.intt(want, p, perm, itw, minv, exact=False),
                               O.intt(want, p, perm, itw, minv, exact=True)))


@pytest.mark.parametrize("dt,bound", [(np.int32, 2**31), (np.int64, 2**63)])
def test_axis_modsum_running_sum_wraps_like_the_reference(compat, dt, bound):
    qs = np.asarray(P.ntt_primes(bound, 8, 3), dt)
    a = P.residues(7, (6, 40, 3), qs, dt)
    for axis in (0, 1):
        shape = tuple(d for i, d in enumerate(a.shape) if i != axis)
        want = O.axis_modsum(a, qs, axis, exact=False)
        assert not np.array_equal(want, O.axis_modsum(a, qs, axis, exact=True))
        assert np.array_equal(run("heal_axis_modsum", a, qs, axis, out_shape=shape, dtype=dt), want)


def test_keyswitch_batch_equals_the_calls_in_compat_mode(compat):
    """The persistent keyswitch batch takes the same literal arithmetic as the
    calls it replaces (its INTT stage scales in the element type too)."""
    from heal_gb300.configs import RaggedKeyswitch
    rk = RaggedKeyswitch(count=4, logns=(12, 13), lmin=2, lmax=4, seed=17)
    want = []
    for i in range(len(rk.specs)):
        rk.run_calls(i)
        want.append(rk.outs[i].numpy())
    for o in rk.outs:
        capi.call("heal_copy_strided", capi.DeviceArray.from_numpy(np.zeros(o.shape, np.int64)), o)
    rk.run_batched()
    for i, w in enumerate(want):
        assert np.array_equal(rk.outs[i].numpy(), w), i
    # on these 50-bit moduli the literal INTT leaves negative residues in x
    assert any((j["x"].numpy() < 0).any() for j in rk.jobs)
