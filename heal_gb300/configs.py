"""Workloads of the benchmark configurations, built through the C ABI.

cfg1  plain batched NTT -> INTT round trip: N = 2^12, the 4 largest primes
      q < 2^30 with q = 1 (mod 2N), a batch of 8 polynomials [8, N, 1, 4]
      int64; then modmul of two NTT-domain tensors and axis_modsum over the
      batch axis.  Five HEAL calls per step, small enough that launch latency
      dominates, so it also runs as one captured CUDA graph.
cfg4  batched NTT at N = 2^16 over 32 limbs of 31-bit primes (the largest
      q < 2^31 with q = 1 (mod 2N)), batch 64, int32 residues: [64, N, 1, 32],
      512 MiB per tensor.
"""
from __future__ import annotations

import numpy as np

from . import capi
from . import params as P


class Cfg1:
    N, L, BATCH, BOUND = 4096, 4, 8, 1 << 30

    def __init__(self, seeds=(101, 102)):
        qs = P.ntt_primes(self.BOUND, self.N, self.L)
        self.qs = qs
        p, perm, tw, itw, minv = P.ntt_tables(qs, self.N)
        shape = (self.BATCH, self.N, 1, self.L)
        self.host = {"A": P.residues(seeds[0], shape, qs), "B": P.residues(seeds[1], shape, qs)}
        D = capi.DeviceArray.from_numpy
        self.t = {k: D(v) for k, v in {"p": p, "perm": perm, "tw": tw, "itw": itw, "minv": minv}.items()}
        self.A, self.B = D(self.host["A"]), D(self.host["B"])
        E = capi.DeviceArray.empty
        self.NA, self.NB, self.RA, self.PR = (E(shape, np.int64, zero=False) for _ in range(4))
        self.AS = E(shape[1:], np.int64, zero=False)

    def run(self):
        t = self.t
        capi.call("heal_ntt", self.A, t["p"], t["perm"], t["tw"], None, None, self.NA)
        capi.call("heal_ntt", self.B, t["p"], t["perm"], t["tw"], None, None, self.NB)
        capi.call("heal_intt", self.NA, t["p"], t["perm"], t["itw"], t["minv"], None, None, self.RA)
        capi.call("heal_modmul_ttt", self.NA, self.NB, t["p"], self.PR)
        capi.call("heal_axis_modsum", self.PR, t["p"], self.AS, 0)

    def transform_limbs(self) -> int:
        return 3 * self.BATCH * self.L   # two NTTs and one INTT of 32 limbs each


class Cfg4:
    N, L, BATCH, BOUND = 1 << 16, 32, 64, 1 << 31

    def __init__(self, batch: int | None = None, seed: int = 404):
        self.batch = batch or self.BATCH
        qs = P.ntt_primes(self.BOUND, self.N, self.L)
        self.qs = qs
        p, perm, tw, itw, minv = P.ntt_tables(qs, self.N, np.int32)
        self.host_tables = {"p": p, "perm": perm, "tw": tw, "itw": itw, "minv": minv}
        self.shape = (self.batch, self.N, 1, self.L)
        D = capi.DeviceArray.from_numpy
        self.t = {k: D(v) for k, v in self.host_tables.items()}
        self.host_x = P.residues(seed, self.shape, qs, np.int32)
        self.X = D(self.host_x)
        self.Y = capi.DeviceArray.empty(self.shape, np.int32, zero=False)
        self.Z = capi.DeviceArray.empty(self.shape, np.int32, zero=False)

    def ntt(self):
        t = self.t
        capi.call("heal_ntt", self.X, t["p"], t["perm"], t["tw"], None, None, self.Y)

    def intt(self):
        t = self.t
        capi.call("heal_intt", self.Y, t["p"], t["perm"], t["itw"], t["minv"], None, None, self.Z)

    def limbs(self) -> int:
        return self.batch * self.L

    def bytes_per_call(self) -> int:
        return 2 * self.batch * self.N * self.L * 4
