"""Workloads of the benchmark configurations, built through the C ABI.

RoundTripChain  plain batched NTT -> INTT round trip: N = 2^12, the 4 largest primes
      q < 2^30 with q = 1 (mod 2N), a batch of 8 polynomials [8, N, 1, 4]
      int64; then modmul of two NTT-domain tensors and axis_modsum over the
      batch axis.  Five HEAL calls per step, small enough that launch latency
      dominates, so it also runs as one captured CUDA graph.
Int32Ntt        batched NTT at N = 2^16 over 32 limbs of 31-bit primes (the
      largest q < 2^31 with q = 1 (mod 2N)), batch 64, int32 residues:
      [64, N, 1, 32], 512 MiB per tensor.
RaggedBatch     256 ciphertexts of mixed ring degree and limb count, each
      through the round-trip chain.
"""
from __future__ import annotations

import numpy as np

from . import capi
from . import params as P


class RoundTripChain:
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

    def bytes_per_step(self) -> int:
        """Algorithmic bytes of one step: three transforms (read + write of a
        [8, 4096, 1, 4] int64 tensor each), modmul (two reads, one write),
        axis_modsum (one read, one write of a [4096, 1, 4] tensor)."""
        t = self.BATCH * self.N * self.L * 8
        return 3 * 2 * t + 3 * t + t + t // self.BATCH


class Int32Ntt:
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


class RaggedBatch:
    """Ragged batch: `count` ciphertexts [2, N_i, 1, L_i] int64 with N_i drawn
    from 2^logns and L_i uniform in 2..32, under the largest 30-bit primes
    q = 1 (mod 2 N_i) (limb t of every ciphertext of ring degree N uses the
    t-th such prime).  Every ciphertext runs the round-trip chain: ntt(A_i),
    ntt(B_i), intt(ntt(A_i)), modmul of the two NTTs, axis_modsum over the
    polynomial axis.  The batch runs as a plain loop of C-ABI calls or as one
    CUDA graph whose branches take the ciphertexts in parallel."""

    COUNT, LOGNS, LMIN, LMAX, BOUND = 256, (12, 13, 14, 15, 16), 2, 32, 1 << 30

    def __init__(self, count: int = COUNT, logns=LOGNS, seed: int = 303):
        idx = P.uniform(seed, (count,), 0, len(logns))
        ls = P.uniform(seed + 1, (count,), self.LMIN, self.LMAX + 1)
        self.specs = [(1 << int(logns[i]), int(l)) for i, l in zip(idx, ls)]
        D, E = capi.DeviceArray.from_numpy, capi.DeviceArray.empty
        self.qs, self.tables = {}, {}
        for n in sorted({n for n, _ in self.specs}):
            qs = P.ntt_primes(self.BOUND, n, self.LMAX)
            p, perm, tw, itw, minv = P.ntt_tables(qs, n)
            self.qs[n] = qs
            self.tables[n] = {"p": D(p), "perm": D(perm), "tw": D(tw), "itw": D(itw), "minv": D(minv)}
        self.A, self.B, self.NA, self.NB, self.RA, self.PR, self.AS, self.views = ([] for _ in range(8))
        for i, (n, l) in enumerate(self.specs):
            shape = (2, n, 1, l)
            self.A.append(D(P.residues(seed * 1000 + 2 * i, shape, self.qs[n][:l])))
            self.B.append(D(P.residues(seed * 1000 + 2 * i + 1, shape, self.qs[n][:l])))
            for lst in (self.NA, self.NB, self.RA, self.PR):
                lst.append(E(shape, np.int64, zero=False))
            self.AS.append(E((n, 1, l), np.int64, zero=False))
            t = self.tables[n]
            self.views.append({
                "p": capi.DeviceArray(t["p"].buf, np.int64, (l,), (1,)),
                "perm": t["perm"],
                "tw": capi.DeviceArray(t["tw"].buf, np.int64, (l, n), (n, 1)),
                "itw": capi.DeviceArray(t["itw"].buf, np.int64, (l, n), (n, 1)),
                "minv": capi.DeviceArray(t["minv"].buf, np.int64, (l,), (1,)),
            })

    # ---- the chain of one ciphertext: five C-ABI calls
    def chain(self, i: int):
        v = self.views[i]
        capi.call("heal_ntt", self.A[i], v["p"], v["perm"], v["tw"], None, None, self.NA[i])
        capi.call("heal_ntt", self.B[i], v["p"], v["perm"], v["tw"], None, None, self.NB[i])
        capi.call("heal_intt", self.NA[i], v["p"], v["perm"], v["itw"], v["minv"], None, None, self.RA[i])
        capi.call("heal_modmul_ttt", self.NA[i], self.NB[i], v["p"], self.PR[i])
        capi.call("heal_axis_modsum", self.PR[i], v["p"], self.AS[i], 0)

    def run(self):
        for i in range(len(self.specs)):
            self.chain(i)

    # ---- the same chain with the transforms of all ciphertexts batched
    def _batch_jobs(self):
        if not hasattr(self, "_jobs"):
            fwd = []
            for i in range(len(self.specs)):
                v = self.views[i]
                fwd.append((self.A[i], v["p"], v["perm"], v["tw"], None, self.NA[i]))
                fwd.append((self.B[i], v["p"], v["perm"], v["tw"], None, self.NB[i]))
            inv = [(self.NA[i], v["p"], v["perm"], v["itw"], v["minv"], self.RA[i])
                   for i, v in enumerate(self.views)]
            self._jobs = (capi.ntt_jobs(fwd), len(fwd), capi.ntt_jobs(inv), len(inv))
        return self._jobs

    def transforms_batched(self):
        """ntt(A_i) and ntt(B_i) of every ciphertext as one heal_ntt_batch,
        then intt(ntt(A_i)) of every ciphertext as another."""
        fwd, nf, inv, ni = self._batch_jobs()
        lib = capi.lib()
        capi.check(lib.heal_ntt_batch(0, fwd, nf))
        capi.check(lib.heal_ntt_batch(1, inv, ni))

    def elementwise(self, i: int):
        v = self.views[i]
        capi.call("heal_modmul_ttt", self.NA[i], self.NB[i], v["p"], self.PR[i])
        capi.call("heal_axis_modsum", self.PR[i], v["p"], self.AS[i], 0)

    def run_batched(self):
        """The chain of every ciphertext with its 768 transforms in two
        batched calls; modmul and axis_modsum per ciphertext.  Bit-identical
        to run()."""
        self.transforms_batched()
        for i in range(len(self.specs)):
            self.elementwise(i)

    def graph_batched(self, branches: int = 8) -> capi.Graph:
        """run_batched as one CUDA graph: the two transform batches, then the
        per-ciphertext modmul and axis_modsum spread over `branches` parallel
        branches (forked after the batches, which they read)."""
        lib = capi.lib()
        plan = self.schedule(branches)

        def rec():
            self.transforms_batched()
            capi.check(lib.heal_graph_fork(branches))
            for b, cts in enumerate(plan):
                capi.check(lib.heal_graph_branch(b))
                for i in cts:
                    self.elementwise(i)
            capi.check(lib.heal_graph_branch(-1))
        return capi.Graph(rec)

    def schedule(self, branches: int) -> list[list[int]]:
        """Ciphertexts per branch: largest first onto the least loaded branch."""
        load, out = [0] * branches, [[] for _ in range(branches)]
        for i in sorted(range(len(self.specs)), key=lambda i: -self.work(i)):
            b = load.index(min(load))
            out[b].append(i)
            load[b] += self.work(i)
        return out

    def record(self, branches: int):
        """Issues the batch for capture: branch b runs its ciphertexts in order."""
        plan = self.schedule(branches)

        def rec(branch):
            for b, cts in enumerate(plan):
                branch(b)
                for i in cts:
                    self.chain(i)
            branch(-1)
        return rec

    def graph(self, branches: int = 8) -> capi.Graph:
        return capi.Graph(self.record(branches), branches=branches)

    def autotune(self, reps: int = 3) -> dict:
        """Tunes the NTT plan of every distinct (N, L) shape of the batch,
        forward and inverse; returns {(N, L): (forward plan, inverse plan)}."""
        done = {}
        for i, (n, l) in enumerate(self.specs):
            if (n, l) in done:
                continue
            v = self.views[i]
            fwd = capi.autotune_ntt(False, self.A[i], v["p"], v["perm"], v["tw"], None, self.NA[i], reps)
            inv = capi.autotune_ntt(True, self.NA[i], v["p"], v["perm"], v["itw"], v["minv"], self.RA[i], reps)
            done[(n, l)] = (fwd, inv)
        return done

    # ---- sizes
    def work(self, i: int) -> int:
        n, l = self.specs[i]
        return n.bit_length() * n * l

    def elements(self) -> int:
        return sum(2 * n * l for n, l in self.specs)

    def transform_limbs(self) -> int:
        return sum(3 * 2 * l for _, l in self.specs)

    def bytes_of(self, i: int) -> int:
        """Algorithmic bytes of ciphertext i's chain: three transforms (read +
        write), modmul (two reads, one write), axis_modsum (read of both
        polynomials, write of one)."""
        n, l = self.specs[i]
        return 2 * n * l * 8 * (2 + 2 + 2 + 3) + (2 * n * l + n * l) * 8

    def bytes_per_step(self) -> int:
        """Algorithmic bytes of one pass over the batch."""
        return sum(self.bytes_of(i) for i in range(len(self.specs)))


class RaggedKeyswitch:
    """Ragged keyswitch batch: `count` ciphertexts [2, N_i, 1, L_i] int64 with
    N_i drawn from 2^logns and L_i uniform in lmin..lmax, under the largest
    50-bit primes q = 1 (mod 2 N_i) (limb t of every ciphertext of ring
    degree N uses the t-th such prime), each through the fused keyswitch step
    of heal_gb300.chain.KeyswitchChain (INTT, g_decomposition into D = 3
    digits of base 2^17 with the NTT of the digits, then modmul by a key,
    axis_modsum over the digits and the Galois permutation X -> X^5).  The
    tables and the key of each ring degree cover lmax limbs; a ciphertext of
    L limbs uses views of their first L limbs.  Runs as the plain loop of
    three C-ABI calls per ciphertext, or as one heal_keyswitch_batch call."""

    COUNT, LOGNS, LMIN, LMAX, D, BITS, BOUND = 256, (12, 13, 14, 15, 16), 2, 32, 3, 17, 1 << 50

    def __init__(self, count: int = COUNT, logns=LOGNS, lmin: int = LMIN, lmax: int = LMAX, seed: int = 707):
        idx = P.uniform(seed, (count,), 0, len(logns))
        ls = P.uniform(seed + 1, (count,), lmin, lmax + 1)
        self.specs = [(1 << int(logns[i]), int(l)) for i, l in zip(idx, ls)]
        self.lmax, D = lmax, self.D
        Dv, E = capi.DeviceArray.from_numpy, capi.DeviceArray.empty
        self.qs, self.tabs = {}, {}
        for n in sorted({n for n, _ in self.specs}):
            qs = P.ntt_primes(self.BOUND, n, lmax)
            p, perm, tw, itw, minv = P.ntt_tables(qs, n)
            self.qs[n] = qs
            host = {"p": p, "perm": perm, "tw": tw, "itw": itw, "minv": minv, "p_t": np.repeat(p, D),
                    "tw_t": np.repeat(tw, D, axis=0),
                    "key": P.residues(seed + n, (2, n, 1, lmax * D), np.repeat(p, D)),
                    "gal": P.galois_perm(n, 5).reshape(1, n)}
            self.tabs[n] = {"host": host, "dev": {k: Dv(v) for k, v in host.items()}}
        self.cts, self.outs, self.jobs, self.host_cts = [], [], [], []
        for i, (n, l) in enumerate(self.specs):
            ct = P.residues(seed * 1000 + i, (2, n, 1, l), self.qs[n][:l])
            self.host_cts.append(ct)
            self.cts.append(Dv(ct))
            self.outs.append(E((2, n, 1, l), np.int64))
            self.jobs.append(self._job(i, E))

    def _job(self, i, E) -> dict:
        n, l = self.specs[i]
        D, L = self.D, self.lmax
        t = self.tabs[n]["dev"]
        V = lambda arr, shape, strides, off=0: capi.DeviceArray(arr.buf, np.int64, shape, strides, arr.offset + off)
        x = E((2, n, 1, l), np.int64, zero=False)
        dn = E((2, n, 1, l * D), np.int64, zero=False)
        key = t["key"]  # [2, n, 1, L * D]: the first l * D columns, viewed [2, n, 1, D, l] as in the chain
        return {"ct": self.cts[i], "p": V(t["p"], (l,), (1,)), "perm": t["perm"],
                "inv_twiddles": V(t["itw"], (l, n), (n, 1)), "m_inv": V(t["minv"], (l,), (1,)), "x": x,
                "power": D, "base_bits": self.BITS, "p_digits": V(t["p_t"], (l * D,), (1,)),
                "twiddles_digits": V(t["tw_t"], (l * D, n), (n, 1)), "digits": dn,
                "tail_a": V(dn, (2, n, 1, D, l), (n * l * D, l * D, l * D, 1, D)),
                "tail_b": V(key, (2, n, 1, D, l), (n * L * D, L * D, L * D, 1, D)),
                "tail_axis": 3, "galois": t["gal"], "elementwise_axis": 2, "perm_axis": 1,
                "result": self.outs[i]}

    def run_calls(self, i: int):
        """Ciphertext i's step as its three C-ABI calls."""
        j = self.jobs[i]
        capi.call("heal_intt", j["ct"], j["p"], j["perm"], j["inv_twiddles"], j["m_inv"], None, None, j["x"])
        capi.call("heal_g_decomposition_ntt", j["x"], j["power"], j["base_bits"], j["p_digits"], j["perm"],
                  j["twiddles_digits"], j["digits"])
        capi.call("heal_modmul_axis_sum_permute", j["tail_a"], j["tail_b"], j["p"], j["tail_axis"], j["galois"],
                  j["elementwise_axis"], j["perm_axis"], j["result"])

    def run(self):
        """The plain loop: three calls per ciphertext."""
        for i in range(len(self.specs)):
            self.run_calls(i)

    def run_batched(self):
        """Every ciphertext's step in one heal_keyswitch_batch call."""
        if not hasattr(self, "_arr"):
            self._arr = capi.keyswitch_jobs(self.jobs)
        capi.check(capi.lib().heal_keyswitch_batch(self._arr, len(self.jobs)))

    def host_tables(self, i: int) -> dict:
        """Ciphertext i's tables and key as numpy arrays (the oracle chain's input)."""
        n, l = self.specs[i]
        h, D, L = self.tabs[n]["host"], self.D, self.lmax
        cols = np.arange(l * D)
        return {"p": h["p"][:l], "perm": h["perm"], "tw": h["tw"][:l], "itw": h["itw"][:l], "minv": h["minv"][:l],
                "key": np.ascontiguousarray(h["key"][..., cols]), "gal": h["gal"]}

    def bytes_per_step(self) -> int:
        """Algorithmic bytes of the fused step over the batch (as
        KeyswitchChain.bytes_per_chain_fused per ciphertext)."""
        tot = 0
        for n, l in self.specs:
            ct = 2 * n * l * 8
            dg = ct * self.D
            tot += 2 * ct + (ct + dg) + (2 * dg + ct)
        return tot
