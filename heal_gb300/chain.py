"""The keyswitch-shaped chain as a sequence of HEAL calls on the GPU.

One step, on a ciphertext tensor ct[2, N, 1, L] (HEAL's [l, m, r, k] with
the 2 ciphertext components as l and the L RNS limbs as k):

  x     = intt(ct)                                   [2, N, 1, L]
  dig   = g_decomposition(x, D, base_bits)           [2, N, 1, L, D]
  dn    = ntt(dig viewed [2, N, 1, L*D], moduli tiled D times)
  prod  = modmul_ttt(dn, key[2, N, 1, L*D], moduli tiled)
  acc   = axis_modsum(prod viewed [2, N, 1, D, L], p, axis=3)
  out   = permute(acc, galois[1, N], elementwise_axis=2, perm_axis=1)

(run_fused makes 3 calls: intt, heal_g_decomposition_ntt, heal_modmul_axis_sum_permute.)
Every step is one C-ABI call (include/heal_gb300.h); the reshape and the
digit-axis move are stride-only views.  The moduli are the L largest primes
q < 2^bound_bits with q = 1 (mod 2N); the key is seeded uniform residues; the
Galois map is X -> X^(5^r mod 2N).
"""
from __future__ import annotations

import numpy as np

from . import capi
from . import params as P


class KeyswitchChain:
    def __init__(self, n: int = 1 << 16, limbs: int = 24, digits: int = 3, base_bits: int = 17,
                 bound_bits: int = 50, rot: int = 1, key_seed: int = 7, dtype=np.int64):
        self.n, self.L, self.D, self.bits = n, limbs, digits, base_bits
        self.dtype = np.dtype(dtype)
        qs = P.ntt_primes(1 << bound_bits, n, limbs)
        self.qs = qs
        p, perm, tw, itw, minv = P.ntt_tables(qs, n, self.dtype)
        self.host = {"p": p, "perm": perm, "tw": tw, "itw": itw, "minv": minv}
        self.host["p_t"] = np.repeat(p, digits)
        self.host["tw_t"] = np.repeat(tw, digits, axis=0)
        self.host["key"] = P.residues(key_seed, (2, n, 1, limbs * digits), self.host["p_t"], self.dtype)
        elt = pow(5, rot, 2 * n)
        self.host["gal"] = P.galois_perm(n, elt).reshape(1, n).astype(self.dtype)
        D = capi.DeviceArray.from_numpy
        self.dev = {k: D(v) for k, v in self.host.items()}
        E = capi.DeviceArray.empty
        self.x = E((2, n, 1, limbs), self.dtype, zero=False)
        self.dig = E((2, n, 1, limbs, digits), self.dtype, zero=False)
        self.dn = E((2, n, 1, limbs * digits), self.dtype, zero=False)
        self.acc = E((2, n, 1, limbs), self.dtype, zero=False)
        self.dig_flat = self.dig.reshape((2, n, 1, limbs * digits))
        self.prod_moved = self.dn.reshape((2, n, 1, limbs, digits)).moveaxis(4, 3)
        self.key_moved = self.dev["key"].reshape((2, n, 1, limbs, digits)).moveaxis(4, 3)

    def shape(self):
        return (2, self.n, 1, self.L)

    def twin(self) -> "KeyswitchChain":
        """A chain on the same resident tables and key with its own
        intermediate tensors, so that two chains can run on two streams."""
        t = object.__new__(KeyswitchChain)
        t.__dict__.update(self.__dict__)
        E = capi.DeviceArray.empty
        n, L, D = self.n, self.L, self.D
        t.x = E((2, n, 1, L), self.dtype, zero=False)
        t.dig = E((2, n, 1, L, D), self.dtype, zero=False)
        t.dn = E((2, n, 1, L * D), self.dtype, zero=False)
        t.acc = E((2, n, 1, L), self.dtype, zero=False)
        t.dig_flat = t.dig.reshape((2, n, 1, L * D))
        t.prod_moved = t.dn.reshape((2, n, 1, L, D)).moveaxis(4, 3)
        return t

    def tune(self, ct: capi.DeviceArray, reps: int = 5) -> dict:
        """Runs the NTT autotuner on the chain's two transform shapes (the
        INTT of the ciphertext, the NTT of the digits) and keeps the fastest
        plans for every later call; returns them.  Overwrites the chain's
        intermediate tensors only."""
        d = self.dev
        inv = capi.autotune_ntt(True, ct, d["p"], d["perm"], d["itw"], d["minv"], self.x, reps)
        capi.call("heal_g_decomposition", self.x, self.dig, self.D, self.bits)
        fwd = capi.autotune_ntt(False, self.dig_flat, d["p_t"], d["perm"], d["tw_t"], None, self.dn, reps)
        return {"intt": {"tile_limbs": inv[0], "first_pass_log2": inv[1]},
                "ntt": {"tile_limbs": fwd[0], "first_pass_log2": fwd[1]}}

    def run(self, ct: capi.DeviceArray, out: capi.DeviceArray):
        """Enqueues one chain step (6 HEAL calls) on the library stream."""
        d = self.dev
        capi.call("heal_intt", ct, d["p"], d["perm"], d["itw"], d["minv"], None, None, self.x)
        capi.call("heal_g_decomposition", self.x, self.dig, self.D, self.bits)
        capi.call("heal_ntt", self.dig_flat, d["p_t"], d["perm"], d["tw_t"], None, None, self.dn)
        capi.call("heal_modmul_ttt", self.dn, d["key"], d["p_t"], self.dn)
        capi.call("heal_axis_modsum", self.prod_moved, d["p"], self.acc, 3)
        capi.call("heal_permute", self.acc, d["gal"], out, 2, 1)

    def run_fused(self, ct: capi.DeviceArray, out: capi.DeviceArray):
        """The same step in 3 HEAL-level calls: the INTT, then
        heal_g_decomposition_ntt (the digit NTT extracts the digits as it
        loads x, so the digit tensor is never written), then
        heal_modmul_axis_sum_permute (modmul, axis_modsum and permute in one
        pass).  Bit-identical to run()."""
        d = self.dev
        capi.call("heal_intt", ct, d["p"], d["perm"], d["itw"], d["minv"], None, None, self.x)
        capi.call("heal_g_decomposition_ntt", self.x, self.D, self.bits, d["p_t"], d["perm"], d["tw_t"], self.dn)
        capi.call("heal_modmul_axis_sum_permute", self.prod_moved, self.key_moved, d["p"], 3, d["gal"], 2, 1, out)

    def job(self, ct: capi.DeviceArray, out: capi.DeviceArray) -> dict:
        """run_fused's three calls as one heal_keyswitch_batch job (fields of
        capi.KeyswitchJob), on this chain's tables, key and intermediates."""
        d = self.dev
        return {"ct": ct, "p": d["p"], "perm": d["perm"], "inv_twiddles": d["itw"], "m_inv": d["minv"], "x": self.x,
                "power": self.D, "base_bits": self.bits, "p_digits": d["p_t"], "twiddles_digits": d["tw_t"],
                "digits": self.dn, "tail_a": self.prod_moved, "tail_b": self.key_moved, "tail_axis": 3,
                "galois": d["gal"], "elementwise_axis": 2, "perm_axis": 1, "result": out}

    def bytes_per_chain_fused(self) -> int:
        """Algorithmic bytes of run_fused: the INTT's read and write, the
        digit NTT's read of x and write of the digit transforms, and one read
        of those and the key and one write of the result."""
        e = self.dtype.itemsize
        ct = 2 * self.n * self.L * e
        dg = ct * self.D
        return (2 * ct) + (ct + dg) + (2 * dg + ct)

    def batched(self, count: int) -> "KeyswitchBatch":
        """A fused chain over `count` ciphertexts at once (same tables and key)."""
        return KeyswitchBatch(self, count)

    # ---- algorithmic bytes (reads + writes of the six calls, tables excluded)
    def bytes_per_chain(self) -> int:
        e = self.dtype.itemsize
        ct = 2 * self.n * self.L * e
        dg = ct * self.D
        return (2 * ct) + (ct + dg) + (2 * dg) + (3 * dg) + (dg + ct) + (2 * ct)

    def ntt_limbs_per_chain(self) -> int:
        return 2 * self.L + 2 * self.L * self.D


class KeyswitchBatch:
    """The fused chain (KeyswitchChain.run_fused) on `count` ciphertexts in the
    same three calls: the ciphertexts are one tensor [2 * count, N, 1, L]
    (ciphertext-major), the key [2, N, 1, L * D] is broadcast over them in
    the tail, and every kernel runs count times the tiles.  Each output
    [2, N, 1, L] slice equals the single chain's output for its ciphertext."""

    def __init__(self, chain: KeyswitchChain, count: int):
        self.ch, self.count = chain, count
        n, L, D = chain.n, chain.L, chain.D
        E = capi.DeviceArray.empty
        B = 2 * count
        self.x = E((B, n, 1, L), chain.dtype, zero=False)
        self.dn = E((B, n, 1, L * D), chain.dtype, zero=False)
        # [count, 2, N, 1, D, L] views of the digit transforms and of the key
        self.dn_moved = self.dn.reshape((count, 2, n, 1, L, D)).moveaxis(5, 4)
        self.key_moved = chain.dev["key"].reshape((1, 2, n, 1, L, D)).moveaxis(5, 4)
        # the Galois rows per ciphertext component: the permutation's elementwise
        # axis is the component axis (2 rows, the same map), so the result view
        # merges to 4 axes
        self.gal2 = capi.DeviceArray.from_numpy(np.repeat(chain.host["gal"], 2, axis=0))

    def shape(self):
        return (2 * self.count, self.ch.n, 1, self.ch.L)

    def run(self, cts: capi.DeviceArray, out: capi.DeviceArray):
        """cts and out: [2 * count, N, 1, L]."""
        ch, d = self.ch, self.ch.dev
        capi.call("heal_intt", cts, d["p"], d["perm"], d["itw"], d["minv"], None, None, self.x)
        capi.call("heal_g_decomposition_ntt", self.x, ch.D, ch.bits, d["p_t"], d["perm"], d["tw_t"], self.dn)
        o = out.reshape((self.count, 2, ch.n, 1, ch.L))
        capi.call("heal_modmul_axis_sum_permute", self.dn_moved, self.key_moved, d["p"], 4, self.gal2, 1, 2, o)

