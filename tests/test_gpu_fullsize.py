"""The benchmarked configurations at their full sizes against the oracle.

- The keyswitch chain at N = 2^16, L = 24 limbs of 50-bit primes, D = 3: the
  GPU runs the whole chain (the INTT over k = 24 limbs, the digit NTT over
  k = 72, 4-limb tiles, 64-bit growing ranges in two 256-point passes), per
  call and fused; the oracle computes a few output limbs (each output limb
  depends only on its own input limb and key columns), and those limbs of the
  INTT, of the digit transforms and of the result must be bit-identical.
- The int32 NTT at N = 2^16 over 32 limbs of 31-bit primes (the
  [64, 65536, 1, 32] workload's shape with 2 batch rows): forward and inverse
  against the oracle's 64-bit transform of the same residues widened to int64,
  which is exact for q < 2^31 (the reference's own int32 transform overflows
  u + q - v there, ntt_impl.cpp:106-107).
"""
import numpy as np
import pytest

from heal_gb300 import capi
from heal_gb300 import params as P
from oracle import oracle as O
from oracle.chain import oracle_chain
from _gpu import ready

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def gpu():
    return ready()


@pytest.fixture(scope="module")
def chain():
    from heal_gb300.chain import KeyswitchChain
    return KeyswitchChain(n=1 << 16, limbs=24, digits=3, base_bits=17, bound_bits=50)


LIMBS = [0, 5, 13, 23]   # first and last tile, both ends of a 4-limb tile, a tile in the middle


def oracle_parts(ch, ct, li):
    """The oracle's INTT limbs, the digit-transform columns times the key (the
    chain multiplies them in place) and the output limbs, for limbs `li`."""
    h = ch.host
    li = np.asarray(li)
    x = O.intt(np.ascontiguousarray(ct[..., li]), h["p"][li], h["perm"], h["itw"][li], h["minv"][li])
    dig, warns = O.g_decomposition(x, ch.D, ch.bits)
    assert warns == 0
    n, k = ct.shape[1], len(li)
    p_t = np.repeat(h["p"][li], ch.D)
    dn = O.ntt(dig.reshape(2, n, 1, k * ch.D), p_t, h["perm"], np.repeat(h["tw"][li], ch.D, axis=0))
    cols = (li[:, None] * ch.D + np.arange(ch.D)[None, :]).reshape(-1)
    prod = O.modmul(dn, np.ascontiguousarray(h["key"][..., cols]), p_t)
    out = oracle_chain(h, ct, ch.D, ch.bits, limb_idx=li)
    return x, prod, out


def test_keyswitch_chain_full_shape_vs_oracle(chain):
    ch = chain
    ct = P.residues(2024, ch.shape(), ch.qs)
    dct = capi.DeviceArray.from_numpy(ct)
    out = capi.DeviceArray.empty(ch.shape(), np.int64)
    ch.run(dct, out)
    x_want, prod_want, out_want = oracle_parts(ch, ct, LIMBS)
    cols = (np.asarray(LIMBS)[:, None] * ch.D + np.arange(ch.D)[None, :]).reshape(-1)
    assert np.array_equal(ch.x.numpy()[..., LIMBS], x_want), "INTT of [2, 65536, 1, 24] differs"
    assert np.array_equal(ch.dn.numpy()[..., cols], prod_want), "digit NTT x key of [2, 65536, 1, 72] differs"
    got = out.numpy()
    assert np.array_equal(got[..., LIMBS], out_want), "keyswitch chain output differs"
    # the fused three-call form of the same chain
    out2 = capi.DeviceArray.empty(ch.shape(), np.int64)
    ch.run_fused(dct, out2)
    assert np.array_equal(out2.numpy(), got)


def test_keyswitch_chain_full_shape_other_limbs(chain):
    """A second ciphertext through the fused chain, on other limbs: across
    the two tests every 4-limb tile of the INTT holds a checked limb."""
    ch = chain
    ct = P.residues(77, ch.shape(), ch.qs)
    out = capi.DeviceArray.empty(ch.shape(), np.int64)
    ch.run_fused(capi.DeviceArray.from_numpy(ct), out)
    li = [2, 7, 8, 11, 14, 19, 22]
    want = oracle_chain(ch.host, ct, ch.D, ch.bits, limb_idx=li)
    assert np.array_equal(out.numpy()[..., li], want)


def test_int32_ntt_full_shape_vs_oracle():
    from heal_gb300.configs import Int32Ntt
    c4 = Int32Ntt(batch=2)
    c4.ntt()
    c4.intt()
    t = {k: np.asarray(v, np.int64) for k, v in c4.host_tables.items()}
    x = np.asarray(c4.host_x, np.int64)
    want = O.ntt(x, t["p"], t["perm"], t["tw"])
    assert np.array_equal(c4.Y.numpy().astype(np.int64), want), "int32 NTT [2, 65536, 1, 32] differs"
    back = O.intt(want, t["p"], t["perm"], t["itw"], t["minv"])
    assert np.array_equal(back, x)
    assert np.array_equal(c4.Z.numpy(), c4.host_x), "int32 INTT [2, 65536, 1, 32] differs"
