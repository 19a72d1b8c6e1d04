"""RNS / NTT parameters and seeded residues for HEAL-layout tensors.

The tables follow the convention HEAL's NTT consumes (include/ntt.h:13-21,
tests/test_ntt.cpp:15-28): for a prime q = 1 (mod 2N) with primitive 2N-th
root psi, twiddles[t, i] = psi^bitrev(i), inv_twiddles[t, i] = psi^-bitrev(i),
perm = bitrev, m_inv = N^-1 (mod q).  With them ntt() returns the negacyclic
evaluations out[i] = sum_j a_j psi^((2i+1) j) in natural order.

Residues come from a counter-based SplitMix64 stream so that the same seed
gives the same tensor on every machine and numpy version.
"""
from __future__ import annotations

import functools

import numpy as np

_MR_BASES = (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37)


def is_prime(n: int) -> bool:
    """Deterministic Miller-Rabin for n < 3.3e24 (covers every 64-bit n)."""
    if n < 2:
        return False
    for p in _MR_BASES:
        if n % p == 0:
            return n == p
    d, s = n - 1, 0
    while d % 2 == 0:
        d //= 2
        s += 1
    for a in _MR_BASES:
        x = pow(a, d, n)
        if x in (1, n - 1):
            continue
        for _ in range(s - 1):
            x = x * x % n
            if x == n - 1:
                break
        else:
            return False
    return True


def ntt_primes(bound: int, n: int, count: int) -> list[int]:
    """The `count` largest primes q < bound with q = 1 (mod 2n), descending."""
    step = 2 * n
    q = ((bound - 2) // step) * step + 1
    out = []
    while len(out) < count and q > step:
        if q < bound and is_prime(q):
            out.append(q)
        q -= step
    if len(out) < count:
        raise ValueError(f"only {len(out)} primes below {bound} are 1 mod {step}")
    return out


def _factor(n: int) -> list[int]:
    fs, d = [], 2
    while d * d <= n:
        if n % d == 0:
            fs.append(d)
            while n % d == 0:
                n //= d
        d += 1 if d == 2 else 2
    if n > 1:
        fs.append(n)
    return fs


@functools.lru_cache(maxsize=None)
def smallest_generator(q: int) -> int:
    """Smallest g generating the multiplicative group mod prime q."""
    fs = _factor(q - 1)
    g = 2
    while any(pow(g, (q - 1) // f, q) == 1 for f in fs):
        g += 1
    return g


def psi(q: int, n: int) -> int:
    """Primitive 2n-th root of unity g^((q-1)/2n) with g the smallest generator."""
    return pow(smallest_generator(q), (q - 1) // (2 * n), q)


def bitrev(n: int) -> np.ndarray:
    """Bit-reversal permutation of range(n), n a power of two."""
    bits = max(n.bit_length() - 1, 0)
    idx = np.arange(n, dtype=np.int64)
    out = np.zeros(n, dtype=np.int64)
    for b in range(bits):
        out |= ((idx >> b) & 1) << (bits - 1 - b)
    return out


def _powers(base: int, n: int, q: int) -> np.ndarray:
    """base^0 .. base^(n-1) mod q as int64 (exact for q < 2^63)."""
    out = np.empty(n, dtype=np.int64)
    if q < (1 << 31):
        # doubling with int64 products (no overflow below 2^62)
        out[0] = 1
        filled, cur = 1, base % q
        while filled < n:
            take = min(filled, n - filled)
            out[filled:filled + take] = (out[:take] * cur) % q
            filled += take
            cur = cur * cur % q
        return out
    v = 1
    for i in range(n):
        out[i] = v
        v = v * base % q
    return out


@functools.lru_cache(maxsize=64)
def _tables_one(q: int, n: int):
    br = bitrev(n)
    ps = psi(q, n)
    pw = _powers(ps, n, q)
    ipw = _powers(pow(ps, -1, q), n, q)
    return pw[br], ipw[br], pow(n, -1, q)


def ntt_tables(qs, n: int, dtype=np.int64):
    """(p[k], perm[n], twiddles[k, n], inv_twiddles[k, n], m_inv[k]) for moduli qs."""
    tw = np.stack([_tables_one(int(q), n)[0] for q in qs]).astype(dtype)
    itw = np.stack([_tables_one(int(q), n)[1] for q in qs]).astype(dtype)
    minv = np.array([_tables_one(int(q), n)[2] for q in qs], dtype=dtype)
    return (np.array(qs, dtype=dtype), bitrev(n).astype(dtype), tw, itw, minv)


def galois_perm(n: int, elt: int) -> np.ndarray:
    """Index map of the automorphism X -> X^elt on natural-order negacyclic
    evaluations: out[i] takes the evaluation at psi^(elt*(2i+1))."""
    i = np.arange(n, dtype=np.int64)
    return (((elt * (2 * i + 1)) % (2 * n)) - 1) // 2


_M1, _M2, _G = np.uint64(0xBF58476D1CE4E5B9), np.uint64(0x94D049BB133111EB), np.uint64(0x9E3779B97F4A7C15)


def splitmix64(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """SplitMix64 outputs for counters offset .. offset+count-1 of `seed`."""
    with np.errstate(over="ignore"):
        x = (np.arange(offset, offset + count, dtype=np.uint64) + np.uint64(1)) * _G
        x = x + np.uint64(seed & 0xFFFFFFFFFFFFFFFF) * _M2
        x = (x ^ (x >> np.uint64(30))) * _M1
        x = (x ^ (x >> np.uint64(27))) * _M2
        return x ^ (x >> np.uint64(31))


def residues(seed: int, shape, qs, dtype=np.int64) -> np.ndarray:
    """Tensor of `shape` whose last axis runs over the moduli qs, each entry
    in [0, q_t) (SplitMix64 reduced mod q_t)."""
    shape = tuple(int(s) for s in shape)
    qs = np.asarray(qs, dtype=np.uint64)
    if shape[-1] != len(qs):
        raise ValueError("last axis must equal the number of moduli")
    n = int(np.prod(shape))
    r = splitmix64(seed, n).reshape(shape) % qs
    return r.astype(dtype)


def uniform(seed: int, shape, low: int, high: int, dtype=np.int64) -> np.ndarray:
    """Integers in [low, high) from the SplitMix64 stream of `seed`."""
    shape = tuple(int(s) for s in shape)
    n = int(np.prod(shape)) if shape else 1
    span = np.uint64(high - low)
    r = (splitmix64(seed, n) % span).astype(np.int64) + low
    return r.reshape(shape).astype(dtype)
