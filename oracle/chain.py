"""The keyswitch-shaped chain on the CPU oracle (test infrastructure only).

INTT -> g_decomposition -> NTT of the digit limbs -> modmul by the key ->
axis_modsum over the digits -> permute, each step the oracle's restatement of
HEAL's example_impl call (ntt_impl.cpp:69-170, g_decomposition_impl.cpp:10-67,
modop_impl.cpp:44-80, axis_modsum_impl.cpp:12-76, permute_impl.cpp:8-65).
Used by tests/, __graft_entry__.smoke() and bench.py's CPU leg as the checker.
"""
import numpy as np

from . import oracle as O


def oracle_chain(ch_host: dict, ct: np.ndarray, digits: int, base_bits: int, limb_idx=None):
    """The keyswitch chain of heal_gb300.chain.KeyswitchChain on the oracle.  With
    `limb_idx`, only those limbs are computed: every output limb depends only
    on its own input limb and key columns."""
    h = ch_host
    p, perm, tw, itw, minv = h["p"], h["perm"], h["tw"], h["itw"], h["minv"]
    key = h["key"]
    L = len(p)
    if limb_idx is not None:
        li = np.asarray(limb_idx)
        cols = (li[:, None] * digits + np.arange(digits)[None, :]).reshape(-1)
        p, tw, itw, minv = p[li], tw[li], itw[li], minv[li]
        key = key[..., cols]
        ct = ct[..., li]
        L = len(li)
    x = O.intt(np.ascontiguousarray(ct), p, perm, itw, minv)
    dig, _ = O.g_decomposition(x, digits, base_bits)
    n = ct.shape[1]
    p_t = np.repeat(p, digits)
    dn = O.ntt(dig.reshape(2, n, 1, L * digits), p_t, perm, np.repeat(tw, digits, axis=0))
    prod = O.modmul(dn, np.ascontiguousarray(key), p_t)
    acc = O.axis_modsum(np.moveaxis(prod.reshape(2, n, 1, L, digits), 4, 3), p, 3)
    return O.permute(acc, h["gal"], 2, 1)


def oracle_roundtrip(A, B, p, perm, tw, itw, minv):
    """The round-trip step of heal_gb300.configs.RoundTripChain on the oracle:
    ntt(A), ntt(B), intt(ntt(A)), modmul of the two transforms, axis_modsum
    over axis 0.  Returns (NA, NB, RA, PR, AS)."""
    NA = O.ntt(A, p, perm, tw)
    NB = O.ntt(B, p, perm, tw)
    RA = O.intt(NA, p, perm, itw, minv)
    PR = O.modmul(NA, NB, p)
    AS = O.axis_modsum(PR, p, 0)
    return NA, NB, RA, PR, AS


def oracle_matvec(ct, perms, diag, p):
    """One matrix-vector request of heal_gb300.serving.MatVecServer on the
    oracle, as the three HEAL calls compute it: ct [2, N, L] expanded over the
    d rotations and permuted by perms [d, N] (elementwise axis 0, permuted
    axis 2), times the diagonals [d, 1, 1, d, L] on the [d, 2, N/d, d, L]
    view, summed over the rotations."""
    d = perms.shape[0]
    _, n, l = ct.shape
    stack = O.permute(np.ascontiguousarray(np.broadcast_to(ct[None], (d, 2, n, l))), perms, 0, 2)
    prod = O.modmul(stack.reshape(d, 2, n // d, d, l), diag, p)
    return O.axis_modsum(prod.reshape(d, 2, n, l), p, 0)
