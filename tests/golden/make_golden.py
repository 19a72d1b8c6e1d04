"""Writes the golden fixtures of tests/golden/ from HEAL's own sample
implementation (example_impl), compiled from the reference sources by
oracle/build_ref.sh into oracle/_ref/.

Run in a container that has the reference sources:
    python tests/golden/make_golden.py
Outputs:
    tests/golden/golden_small.npz  full input/output arrays of small cases
    tests/golden/golden_hash.json  SHA-256 of outputs of full-size cases
                                    (their inputs are regenerated from seeds)
The GPU tests and the oracle tests only read these files; nothing at test
time needs the reference sources.
"""
import glob
import warnings
import hashlib
import importlib.util
import json
import os
import subprocess
import sys

import numpy as np
import torch

warnings.filterwarnings("ignore", message="The given NumPy array is not writable")

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)
from heal_gb300 import params as P  # noqa: E402


def load_reference():
    hits = glob.glob(os.path.join(ROOT, "oracle", "_ref", "lattica_hw*.so"))
    if not hits:
        subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
        hits = glob.glob(os.path.join(ROOT, "oracle", "_ref", "lattica_hw*.so"))
    spec = importlib.util.spec_from_file_location("lattica_hw", hits[0])
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


R = load_reference()
SUF = {np.dtype(np.int32): "32", np.dtype(np.int64): "64"}


def fn(name, dt):
    return getattr(R, f"{name}_{SUF[np.dtype(dt)]}")


def H(x):
    """host_to_device of a numpy array; torch.from_numpy keeps its strides."""
    return fn("host_to_device", x.dtype)(torch.from_numpy(x))


def dh(dt_, dev):
    return fn("device_to_host", dt_)(dev).numpy()


def alloc(shape, dt):
    return fn("allocate_on_hardware", dt)(list(shape))


def ref_ntt(a, p, perm, tw):
    out = alloc(a.shape, a.dtype)
    fn("ntt", a.dtype)(H(a), H(p), H(perm), H(tw), None, None, out)
    return dh(a.dtype, out)


def ref_intt(a, p, perm, itw, minv):
    out = alloc(a.shape, a.dtype)
    fn("intt", a.dtype)(H(a), H(p), H(perm), H(itw), H(minv), None, None, out)
    return dh(a.dtype, out)


def ref_modop(op, kind, a, b, p, out_shape):
    out = alloc(out_shape, a.dtype)
    f = fn(f"{op}_{kind}", a.dtype)
    bb = H(b) if kind[1] == "t" else int(b)
    pp = H(p) if kind[2] == "t" else int(p)
    f(H(a), bb, pp, out)
    return dh(a.dtype, out)


def ref_axis_modsum(a, p, axis):
    shape = [d for i, d in enumerate(a.shape) if i != axis]
    out = alloc(shape, a.dtype)
    fn("axis_modsum", a.dtype)(H(a), H(p), out, axis)
    return dh(a.dtype, out)


def ref_gdec(a, power, bits):
    out = alloc(list(a.shape) + [power], a.dtype)
    fn("g_decomposition", a.dtype)(H(a), out, power, bits)
    return dh(a.dtype, out)


def ref_permute(a, perms, ew, pa):
    out = alloc(a.shape, a.dtype)
    fn("permute", a.dtype)(H(a), H(perms), out, ew, pa)
    return dh(a.dtype, out)


def sha(x):
    return hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest()


small = {}
hashes = {}


def put(case, **arrays):
    for k, v in arrays.items():
        small[f"{case}__{k}"] = np.asarray(v)


# ---- 1. the pins of tests/test_ntt.cpp (int32, p = {17, 257})
a = np.array([1, 2, 3, 4, 5, 6, 7, 8], np.int32).reshape(1, 4, 1, 2)
p = np.array([17, 257], np.int32)
perm = np.array([0, 2, 1, 3], np.int32)
tw = np.array([[1, 4, 2, 8], [1, 16, 4, 64]], np.int32)
itw = np.array([[1, 13, 9, 15], [1, 241, 193, 253]], np.int32)
minv = np.array([13, 193], np.int32)
fw = ref_ntt(a, p, perm, tw)
put("ntt_pin", a=a, p=p, perm=perm, tw=tw, itw=itw, minv=minv, ntt=fw, intt=ref_intt(fw, p, perm, itw, minv))

# ---- 2. small NTT / INTT cases, int64 and int32, canonical and negative
for case, dt, shape, bound, seed in [("ntt_i64", np.int64, (2, 64, 3, 3), 2**40, 11),
                                    ("ntt_i64_m1", np.int64, (2, 1, 2, 3), 2**40, 12),
                                    ("ntt_i64_m2", np.int64, (3, 2, 1, 2), 2**40, 13),
                                    ("ntt_i64_m4096", np.int64, (1, 4096, 1, 2), 2**40, 19),
                                    ("ntt_i32", np.int32, (3, 32, 1, 2), 2**14, 14),
                                    # 31-bit moduli: the reference's int32 sums wrap (ntt_impl.cpp:106-107)
                                    ("ntt_i32_q31", np.int32, (2, 64, 1, 3), 2**31, 15)]:
    n = shape[1]
    qs = P.ntt_primes(bound, max(n, 2), shape[3])
    p, perm, tw, itw, minv = P.ntt_tables(qs, n, dt)
    x = P.residues(seed, shape, qs, dt)
    fw = ref_ntt(x, p, perm, tw)
    put(case, a=x, p=p, perm=perm, tw=tw, itw=itw, minv=minv, ntt=fw, intt=ref_intt(fw, p, perm, itw, minv),
        intt_a=ref_intt(x, p, perm, itw, minv))

# negative and over-range inputs (C truncating semantics all the way through)
qs = P.ntt_primes(2**20, 16, 2)
p, perm, tw, itw, minv = P.ntt_tables(qs, 16, np.int64)
x = P.uniform(21, (2, 16, 1, 2), -(2**21), 2**21)
put("ntt_neg", a=x, p=p, perm=perm, tw=tw, itw=itw, minv=minv, ntt=ref_ntt(x, p, perm, tw),
    intt=ref_intt(x, p, perm, itw, minv))
# negative twiddles
twn = tw.copy()
twn[:, 1::3] -= p[:, None]
put("ntt_negtw", a=P.residues(22, (1, 16, 2, 2), qs), p=p, perm=perm, tw=twn,
    ntt=ref_ntt(P.residues(22, (1, 16, 2, 2), qs), p, perm, twn))
# arbitrary (non bit-reversal) permutation; non-bijective one for the INTT scatter
rp = np.argsort(P.splitmix64(23, 16)).astype(np.int64)
dup = rp.copy()
dup[3] = dup[7]
xx = P.residues(24, (2, 16, 1, 2), qs)
put("ntt_perm", a=xx, p=p, perm=rp, dup=dup, tw=tw, itw=itw, minv=minv, ntt=ref_ntt(xx, p, rp, tw),
    intt=ref_intt(xx, p, rp, itw, minv), ntt_dup=ref_ntt(xx, p, dup, tw), intt_dup=ref_intt(xx, p, dup, itw, minv))

# ---- 3. keyswitch-shaped ops at N = 256, 50-bit primes (reference INTT overflows here:
#         its output pins the oracle's literal mode)
N, L, D, BITS = 256, 4, 3, 17
qs = P.ntt_primes(2**50, N, L)
p, perm, tw, itw, minv = P.ntt_tables(qs, N, np.int64)
ct = P.residues(31, (2, N, 1, L), qs)
coef = P.residues(32, (2, N, 1, L), qs)
digits = ref_gdec(coef, D, BITS)
qs_t = np.repeat(p, D)
tw_t = np.repeat(tw, D, axis=0)
dn = ref_ntt(digits.reshape(2, N, 1, L * D), qs_t, perm, tw_t)
key = P.residues(33, (2, N, 1, L * D), qs_t)
prod = ref_modop("modmul", "ttt", dn, key, qs_t, dn.shape)
moved = np.moveaxis(prod.reshape(2, N, 1, L, D), 4, 3)  # [2, N, 1, D, L] strided view
acc = ref_axis_modsum(moved, p, 3)
gal = P.galois_perm(N, 5).reshape(1, N)
put("keyswitch_n256", ct=ct, coef=coef, p=p, perm=perm, tw=tw, itw=itw, minv=minv, key=key,
    ntt_ct=ref_ntt(ct, p, perm, tw), intt_ct_literal=ref_intt(ct, p, perm, itw, minv),
    digits=digits, dn=dn, prod=prod, acc=acc, gal=gal, rot=ref_permute(acc, gal, 2, 1))

# ---- 4. elementwise modular ops with broadcasting, strides and signs
for dt in (np.int32, np.int64):
    tag = SUF[np.dtype(dt)]
    big = 2**30 if dt == np.int32 else 2**62
    a = P.uniform(41, (2, 3, 4), 0, 200, dt)
    b = P.uniform(42, (1, 3, 4), 0, 200, dt)
    pp = P.uniform(43, (4,), 100, 200, dt)
    an = P.uniform(44, (2, 3, 4), -big, big, dt)
    bn = P.uniform(45, (3, 4), -big, big, dt)
    pn = P.uniform(46, (4,), -big // 4, big // 4, dt)
    pn[pn == 0] = 7
    at = np.ascontiguousarray(P.uniform(47, (4, 3, 2), -1000, 1000, dt)).transpose(2, 1, 0)
    col = P.uniform(48, (2, 1), 0, 50, dt)
    row = P.uniform(49, (3,), 0, 50, dt)
    prow = np.array([11, 17, 23], dt)
    for op in ("modmul", "modsum"):
        put(f"{op}_{tag}", a=a, b=b, p=pp, an=an, bn=bn, pn=pn, at=at, col=col, row=row, prow=prow,
            ttt=ref_modop(op, "ttt", a, b, pp, a.shape),
            ttt_neg=ref_modop(op, "ttt", an, bn, pn, an.shape),
            ttt_strided=ref_modop(op, "ttt", at, at, pp, at.shape),
            ttt_bcast=ref_modop(op, "ttt", col, row, prow, (2, 3)),
            ttc=ref_modop(op, "ttc", an, bn, 1000003, an.shape),
            tct=ref_modop(op, "tct", an, -12345, pn, an.shape),
            tcc=ref_modop(op, "tcc", an, 98765, 4099, an.shape))

# ---- 5. axis_modsum (sequential truncating reduction), g_decomposition, permute
for dt in (np.int32, np.int64):
    tag = SUF[np.dtype(dt)]
    big = 2**29 if dt == np.int32 else 2**61
    x = P.uniform(51, (3, 5, 2, 4), -big, big, dt)
    pp = np.array([7, 1000003, 65537, 97], dt)
    put(f"axis_modsum_{tag}", a=x, p=pp, ax0=ref_axis_modsum(x, pp, 0), ax1=ref_axis_modsum(x, pp, 1),
        ax2=ref_axis_modsum(x, pp, 2), seq=ref_axis_modsum(np.array([[5], [5], [-8]], dt), np.array([7], dt), 0))
    lim = 2**31 if dt == np.int32 else 2**63
    g = P.uniform(52, (4, 6), -lim // 2, lim // 2, dt)
    g.flat[:3] = [0, 1, -1]
    put(f"gdec_{tag}", a=g, b3p4=ref_gdec(g, 4, 3), b17p3=ref_gdec(g, 3, 17), b1p40=ref_gdec(g, 40, 1))
    x = P.uniform(53, (2, 3, 4, 5), 0, 1000, dt)
    perms_a = np.stack([np.argsort(P.splitmix64(54 + i, 4)) for i in range(3)]).astype(dt)
    perms_b = np.stack([np.argsort(P.splitmix64(60 + i, 5)) for i in range(2)]).astype(dt)
    put(f"permute_{tag}", a=x, perms_a=perms_a, perms_b=perms_b,
        r12=ref_permute(x, perms_a, 1, 2), r03=ref_permute(x, perms_b, 0, 3))

# ---- 6. axis_modsum's running sum wrapping in the element type (axis_modsum_impl.cpp:70): canonical
#         residues of moduli near 2^31 (int32) and 2^63 (int64)
for dt, bound in ((np.int32, 2**31), (np.int64, 2**63)):
    tag = SUF[np.dtype(dt)]
    qs = np.asarray(P.ntt_primes(bound, 8, 3), dt)
    x = P.residues(61, (6, 40, 3), qs, dt)
    put(f"axis_modsum_wrap_{tag}", a=x, p=qs, ax0=ref_axis_modsum(x, qs, 0), ax1=ref_axis_modsum(x, qs, 1))

np.savez_compressed(os.path.join(HERE, "golden_small.npz"), **small)

# ---- 6. full-size cases checked by hash (inputs regenerated from seeds)
N, L = 4096, 4
qs = P.ntt_primes(2**30, N, L)
p, perm, tw, itw, minv = P.ntt_tables(qs, N, np.int64)
A = P.residues(101, (8, N, 1, L), qs)
B = P.residues(102, (8, N, 1, L), qs)
NA, NB = ref_ntt(A, p, perm, tw), ref_ntt(B, p, perm, tw)
RT = ref_intt(NA, p, perm, itw, minv)
assert np.array_equal(RT, A)
PR = ref_modop("modmul", "ttt", NA, NB, p, NA.shape)
AS = ref_axis_modsum(PR, p, 0)
hashes["roundtrip_n4096"] = {"N": N, "L": L, "bound": 2**30, "seeds": [101, 102], "shape": [8, N, 1, L],
                  "ntt_a": sha(NA), "ntt_b": sha(NB), "intt_ntt_a": sha(RT), "modmul": sha(PR), "axis_modsum": sha(AS),
                  "ntt_a_head": NA.reshape(-1)[:16].tolist(), "axis_modsum_head": AS.reshape(-1)[:16].tolist()}

N, L = 2**16, 2
qs = P.ntt_primes(2**50, N, L)
p, perm, tw, itw, minv = P.ntt_tables(qs, N, np.int64)
X = P.residues(201, (2, N, 1, L), qs)
hashes["n65536_i64"] = {"N": N, "L": L, "bound": 2**50, "seed": 201, "shape": [2, N, 1, L],
                        "ntt": sha(ref_ntt(X, p, perm, tw))}

with open(os.path.join(HERE, "golden_hash.json"), "w") as f:
    json.dump(hashes, f, indent=1)
print("wrote", len(small), "arrays and", len(hashes), "hash cases")
