"""Writes the synthetic verify-transcripts under tests/golden/transcripts/.

HEAL's example transcript is not distributed with its sources, so these are
recorded here with heal_gb300.runtime.TranscriptBuilder, in HEAL's transcript
JSON format, with every device_to_host carrying the expected tensor computed
by the CPU oracle (a restatement of example_impl).  Run from the repository
root:  python tests/golden/make_transcripts.py
"""
import os
import sys

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from heal_gb300 import params as P                      # noqa: E402
from heal_gb300.runtime import TranscriptBuilder, save_transcript_to_json   # noqa: E402
from oracle import build as ob                          # noqa: E402
from oracle import oracle as O                          # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden", "transcripts")
I64 = torch.int64
T = lambda a: torch.from_numpy(np.ascontiguousarray(a))


def keyswitch(n=256, L=4, D=3, bits=17, bound=50):
    """The keyswitch-shaped chain: intt, digits, ntt of the digits, key
    product, sum over the digits, Galois permutation X -> X^5."""
    qs = P.ntt_primes(1 << bound, n, L)
    p, perm, tw, itw, minv = P.ntt_tables(qs, n)
    p_t, tw_t = np.repeat(p, D), np.repeat(tw, D, axis=0)
    key = P.residues(7, (2, n, 1, L * D), p_t)
    gal = P.galois_perm(n, 5).reshape(1, n).astype(np.int64)
    ct = P.residues(1000, (2, n, 1, L), qs)
    # expected, step by step on the oracle
    x = O.intt(ct, p, perm, itw, minv)
    dig, _ = O.g_decomposition(x, D, bits)
    dn = O.ntt(dig.reshape(2, n, 1, L * D), p_t, perm, tw_t)
    prod = O.modmul(dn, key, p_t)
    acc = O.axis_modsum(np.moveaxis(prod.reshape(2, n, 1, L, D), 4, 3), p, 3)
    out = O.permute(acc, gal, 2, 1)

    b = TranscriptBuilder()
    b.segment("keyswitch")
    d = {k: b.host_to_device(T(v)) for k, v in
         {"ct": ct, "p": p, "perm": perm, "itw": itw, "minv": minv, "p_t": p_t, "tw_t": tw_t, "key": key,
          "gal": gal}.items()}
    xd = b.op("empty", (2, n, 1, L), I64, dtype=I64)
    xd = b.op("intt", d["ct"], d["perm"], None, d["p"], None, None, d["itw"], d["minv"], xd, 0, 0, dtype=I64)
    b.device_to_host(xd, T(x))
    dg = b.op("empty", (2, n, 1, L, D), I64, dtype=I64)
    dg = b.op("apply_g_decomp", xd, D, bits, dg, dtype=I64)
    dgf = b.op("reshape", dg, (2, n, 1, L * D), dtype=I64)
    nd = b.op("empty", (2, n, 1, L * D), I64, dtype=I64)
    nd = b.op("ntt", dgf, d["perm"], None, d["p_t"], None, None, d["tw_t"], nd, 0, 0, dtype=I64)
    b.device_to_host(nd, T(dn))
    nd = b.op("_modmul_ttt", nd, d["key"], d["p_t"], nd, dtype=I64)
    pm = b.op("reshape", nd, (2, n, 1, L, D), dtype=I64)
    pm = b.op("moveaxis", pm, 4, 3, dtype=I64)
    ac = b.op("empty", (2, n, 1, L), I64, dtype=I64)
    ac = b.op("axis_modsum", pm, 3, d["p"], ac, dtype=I64)
    od = b.op("empty", (2, n, 1, L), I64, dtype=I64)
    od = b.op("take_along_axis", ac, d["gal"], 2, 1, od, dtype=I64)
    b.device_to_host(od, T(out))
    b.free(*d.values(), xd, dg, dgf, nd, pm, ac, od)
    b.end_segment()
    return b.transcript()


def roundtrip_ops(n=256, L=4, batch=2, bound=30):
    """The round-trip chain (ntt, intt, modmul, axis_modsum over the batch) and the
    remaining elementwise and view ops of the dispatcher."""
    qs = P.ntt_primes(1 << bound, n, L)
    p, perm, tw, itw, minv = P.ntt_tables(qs, n)
    A = P.residues(101, (batch, n, 1, L), qs)
    B = P.residues(102, (batch, n, 1, L), qs)
    NA, NB = O.ntt(A, p, perm, tw), O.ntt(B, p, perm, tw)
    RA = O.intt(NA, p, perm, itw, minv)
    PR = O.modmul(NA, NB, p)
    AS = O.axis_modsum(PR, p, 0)
    SUM = O.modsum(NA, NB, p)
    NEG = O.modneg(NA, p)
    MODC = O.mod(NA, 1000003)
    MULC = O.modmul(NA, 12345, p)
    sl = np.ascontiguousarray(NA[1, 16:48:2, 0, :])          # get_slice(a, 1, slice(16, 48, 2), 0, ...)

    b = TranscriptBuilder()
    b.segment("roundtrip")
    d = {k: b.host_to_device(T(v)) for k, v in {"A": A, "B": B, "p": p, "perm": perm, "tw": tw, "itw": itw,
                                               "minv": minv}.items()}
    shape = (batch, n, 1, L)
    na = b.op("ntt", d["A"], d["perm"], None, d["p"], None, None, d["tw"], b.op("empty", shape, I64, dtype=I64),
              0, 0, dtype=I64)
    nb = b.op("ntt", d["B"], d["perm"], None, d["p"], None, None, d["tw"], b.op("zeros", shape, I64, dtype=I64),
              0, 0, dtype=I64)
    ra = b.op("intt", na, d["perm"], None, d["p"], None, None, d["itw"], d["minv"],
              b.op("empty", shape, I64, dtype=I64), 0, 0, dtype=I64)
    pr = b.op("_modmul_ttt", na, nb, d["p"], b.op("empty", shape, I64, dtype=I64), dtype=I64)
    asum = b.op("axis_modsum", pr, 0, d["p"], b.op("empty", shape[1:], I64, dtype=I64), dtype=I64)
    for ptr, want in ((na, NA), (ra, RA), (pr, PR), (asum, AS)):
        b.device_to_host(ptr, T(want))
    b.end_segment()
    b.segment("elementwise")
    s = b.op("_modsum_ttt", na, nb, d["p"], b.op("empty", shape, I64, dtype=I64), dtype=I64)
    g = b.op("_modneg_tt", na, d["p"], b.op("empty", shape, I64, dtype=I64), dtype=I64)
    m = b.op("_mod_tc", na, 1000003, b.op("empty", shape, I64, dtype=I64), dtype=I64)
    c = b.op("_modmul_tct", na, 12345, d["p"], b.op("empty", shape, I64, dtype=I64), dtype=I64)
    for ptr, want in ((s, SUM), (g, NEG), (m, MODC), (c, MULC)):
        b.device_to_host(ptr, T(want))
    b.end_segment()
    b.segment("views")
    v = b.op("get_slice", na, 1, slice(16, 48, 2), 0, Ellipsis, dtype=I64)
    b.device_to_host(v, T(sl))
    cv = b.op("contiguous", v, dtype=I64)
    fl = b.op("flatten", cv, dtype=I64)
    b.device_to_host(fl, T(sl.reshape(-1)))
    u = b.op("unsqueeze", b.op("new_reference", asum, dtype=I64), 0, dtype=I64)
    e = b.op("expand", u, 3, 0, dtype=I64)
    b.device_to_host(e, T(np.broadcast_to(AS[None], (3,) + AS.shape)))
    b.end_segment()
    return b.transcript()


def matvec(n=256, d=4, L=3, bound=40):
    """One matrix-vector request: the sum over d Galois rotations of
    rot_i(ct) * diag_i, as take_along_axis + modmul + axis_modsum and as one
    modmul_axis_sum."""
    qs = P.ntt_primes(1 << bound, n, L)
    p = np.array(qs, np.int64)
    ct = P.residues(4, (2, n, L), qs)
    perms = np.stack([P.galois_perm(n, pow(5, i, 2 * n)) for i in range(d)]).astype(np.int64)
    diag = P.residues(5, (d, 1, n, L), qs)
    stack = O.permute(np.ascontiguousarray(np.broadcast_to(ct[None], (d, 2, n, L))), perms, 0, 2)
    want = O.axis_modsum(O.modmul(stack, np.ascontiguousarray(np.broadcast_to(diag, (d, 2, n, L))), p,
                                  out_shape=(d, 2, n, L)), p, 0)

    b = TranscriptBuilder()
    b.segment("matvec")
    dc, dp, dd, dpm = (b.host_to_device(T(v)) for v in (ct, p, diag, perms))
    a = b.op("expand", b.op("unsqueeze", dc, 0, dtype=I64), d, 0, dtype=I64)     # [d, 2, n, L], stride 0
    st = b.op("take_along_axis", a, dpm, 0, 2, b.op("empty", (d, 2, n, L), I64, dtype=I64), dtype=I64)
    st = b.op("_modmul_ttt", st, dd, dp, st, dtype=I64)
    o3 = b.op("axis_modsum", st, 0, dp, b.op("empty", (2, n, L), I64, dtype=I64), dtype=I64)
    b.device_to_host(o3, T(want))
    of = b.op("modmul_axis_sum", a, dd, dp, 0, b.op("empty", (2, n, L), I64, dtype=I64), dpm, 2, dtype=I64)
    b.device_to_host(of, T(want))
    b.end_segment()
    return b.transcript()


def main():
    ob.build()
    os.makedirs(OUT, exist_ok=True)
    for name, fn in (("keyswitch_n256.json", keyswitch), ("roundtrip_ops_n256.json", roundtrip_ops),
                     ("matvec_n256.json", matvec)):
        path = os.path.join(OUT, name)
        save_transcript_to_json(fn(), path)
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
