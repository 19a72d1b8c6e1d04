"""Benchmark of the HEAL hot path on one GB300: the keyswitch-shaped chain.

Workload: a ciphertext ct[2][L=24][N=2^16] of int64 residues under the 24
largest 50-bit primes q = 1 (mod 2N), through INTT, g_decomposition (D = 3
digits of base 2^17), NTT of the 72 digit limbs, modmul against a
key[3][2][24][2^16], axis_modsum over the digits, and the Galois permutation
X -> X^5.  Each HEAL call is one C-ABI call.  One step is a batch of
CHAINS_PER_STEP such chains (ciphertexts rotating through 8 resident inputs),
so that the driver's 20 timed steps span about half a second.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Printed: one JSON line (rank 0).  `value` is chains/s with inputs resident
in HBM, timed with CUDA events, consecutive chains alternating between the
library stream and a second stream (`value_one_stream`: all on one); inputs
rotate through 8 ciphertexts (192 MiB) and 8 outputs, more than the 126 MiB
L2, so no chain reads the previous chain's data from L2.  `e2e` is the same
through the C ABI from pinned host buffers (H2D of ct and D2H of the result of
every chain inside the timed region, on their own streams so that they overlap
the chains of neighbouring steps; `e2e.serial_value` is the same back to
back).  `roofline` covers the batched NTT of the digits.  `cpu_baseline`
times the CPU oracle (a restatement of HEAL's example_impl) on this host, on
SAMPLE_LIMBS of the 24 limbs per run, and compares every limb it computes
with the GPU chain's output for the same ciphertext (`oracle_equal`).

--impl reference times the CPU oracle itself on all host cores, SAMPLE_LIMBS
limbs of one chain per step (every limb is independent), scaled to chains/s.
Under torchrun with N > 1 every rank runs its own chains on its own GPU
(replicas, no collective on the data path); the time is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N, L, D, BITS, BOUND = 1 << 16, 24, 3, 17, 50
METRIC = "batched NTT limbs/s & keyswitch chains/s on 1 GB300, bit-exact, % HBM roofline"
CONFIG = {"workload": "keyswitch chain: ct[2][24][65536] int64, 50-bit NTT primes, INTT -> g_decomposition "
                      "(D=3, base 2^17) -> NTT(72 limbs) -> modmul(key[3][2][24][65536]) -> axis_modsum(digits) "
                      "-> permute(X->X^5); one step = 128 such chains",
          "N": N, "limbs": L, "digits": D, "base_bits": BITS, "prime_bits": BOUND,
          "l2": "inputs rotate through 8 ciphertexts (192 MiB) and 8 outputs, larger than L2",
          "parallelism": "replicas per GPU (limb/ciphertext sharding needs no collective)",
          "streams": "two chains in flight on two CUDA streams (value_one_stream: one stream)",
          "chains_per_step": 128}
CHAINS_PER_STEP = CONFIG["chains_per_step"]
RING = 8
# the workloads reported under "configs" beside the headline (--configs)
WORKLOADS = ("roundtrip", "ragged", "ragged_keyswitch", "int32_ntt", "serving")


def dist_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def max_over_ranks(ms: float, world: int, device) -> float:
    """The slowest rank's time (every rank gets it); a no-op on one rank."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, ms: float) -> float:
    """Units all ranks processed per second, over the slowest rank's time
    (each rank runs its own replicas: weak scaling)."""
    return units_per_rank * world / (ms / 1e3)


class Clocks:
    """Samples SM clocks and clock-event (throttle) reasons while running:
    NVML through ctypes every 2 ms (read-only queries), else nvidia-smi every
    200 ms."""

    # NVML clocks-event reason bits (nvml.h)
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        ids = [x for x in vis.split(",") if x.strip()]
        self.gpu = int(ids[gpu]) if gpu < len(ids) and ids[gpu].strip().isdigit() else gpu
        self.proc = None
        self.path = None
        self.nvml = None
        self.rows = []

    def _nvml_open(self):
        import ctypes
        try:
            lib = ctypes.CDLL("libnvidia-ml.so.1")
        except OSError:
            return None
        h = ctypes.c_void_p()
        if lib.nvmlInit_v2() != 0 or lib.nvmlDeviceGetHandleByIndex_v2(self.gpu, ctypes.byref(h)) != 0:
            return None
        fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons")
        return lib, h, fn

    def _sample_loop(self):
        import ctypes
        lib, h, reasons_fn = self.nvml
        mhz, mx, mw, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx))          # NVML_CLOCK_SM
        while not self.stop.is_set():
            ok = lib.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(mhz)) == 0
            ok = ok and reasons_fn(h, ctypes.byref(rs)) == 0
            p = mw.value if lib.nvmlDeviceGetPowerUsage(h, ctypes.byref(mw)) == 0 else 0
            if ok:
                self.rows.append((mhz.value, mx.value, p / 1000.0, rs.value))
            self.stop.wait(0.002)

    def __enter__(self):
        import threading
        self.nvml = self._nvml_open()
        if self.nvml:
            self.stop = threading.Event()
            self.thread = threading.Thread(target=self._sample_loop, daemon=True)
            self.thread.start()
            return self
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.nvml:
            self.stop.set()
            self.thread.join()
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        if self.nvml:
            if not self.rows:
                return {"sm_mhz": None, "sm_max_mhz": None, "samples": 0, "reasons": ["no NVML samples"],
                        "source": "nvml"}
            reasons = sorted({name for r in self.rows for bit, name in self.REASONS.items() if r[3] & bit})
            return {"sm_mhz": statistics.median(r[0] for r in self.rows), "sm_max_mhz": float(self.rows[0][1]),
                    "power_w": statistics.median(r[2] for r in self.rows), "samples": len(self.rows),
                    "reasons": reasons, "source": "nvml, every 2 ms"}
        rows = []
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9:
                    rows.append(f)
        finally:
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": float(rows[0][2]) if rows[0][2].replace(".", "").isdigit() else None,
                "samples": len(rows), "reasons": reasons, "source": "nvidia-smi, every 200 ms"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_traffic():
    """dram bytes per NTT call from the committed ncu summary, if present."""
    try:
        with open(os.path.join(ROOT, "profiles", "ntt_traffic.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


# ------------------------------------------------------------------- CPU
# limbs per CPU run of the oracle chain: the INTT gets 2 x 8 = 16 columns and the digit NTT 48, so every
# core of a 16-core host has work in each step (4 limbs left half of them idle in the INTT); divides 24
SAMPLE_LIMBS = 8


def sample_limbs(run):
    return [(run * SAMPLE_LIMBS + i) % L for i in range(SAMPLE_LIMBS)]


def cpu_sample(ch_host, ct, seconds=10.0, gpu_out=None):
    """Oracle chain restricted to SAMPLE_LIMBS limbs per run, repeated for
    ~`seconds`; returns (chains/s, threads, runs, check).  With `gpu_out` (the
    GPU chain's output for `ct`), every limb the oracle computes is compared
    with the same limb of it; `check` counts the limbs compared and whether
    all were bit-identical."""
    from oracle import oracle as O
    from oracle.chain import oracle_chain
    threads = O.set_threads(os.cpu_count() or 1)
    runs, t0, el = 0, time.perf_counter(), 0.0
    checked, equal = set(), True
    while True:
        li = sample_limbs(runs)
        t1 = time.perf_counter()
        got = oracle_chain(ch_host, ct, D, BITS, limb_idx=li)
        el += time.perf_counter() - t1
        if gpu_out is not None:
            equal = equal and bool(np.array_equal(got, gpu_out[..., li]))
            checked.update(li)
        runs += 1
        if time.perf_counter() - t0 >= seconds:
            break
    check = None if gpu_out is None else {"oracle_limbs_checked": len(checked), "oracle_equal": equal}
    return runs * SAMPLE_LIMBS / el / L, threads, runs, check


def reference_arm(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    from heal_gb300 import params as P
    from oracle import build as ob
    from oracle import oracle as O
    from oracle.chain import oracle_chain
    ob.build()
    qs = P.ntt_primes(1 << BOUND, N, L)
    p, perm, tw, itw, minv = P.ntt_tables(qs, N)
    host = {"p": p, "perm": perm, "tw": tw, "itw": itw, "minv": minv,
            "key": P.residues(7, (2, N, 1, L * D), np.repeat(p, D)),
            "gal": P.galois_perm(N, 5).reshape(1, N)}
    ct = P.residues(1000, (2, N, 1, L), qs)
    threads = O.set_threads(os.cpu_count() or 1)
    for w in range(args.warmup):
        oracle_chain(host, ct, D, BITS, limb_idx=sample_limbs(w))
    t0 = time.perf_counter()
    for s in range(args.steps):
        oracle_chain(host, ct, D, BITS, limb_idx=sample_limbs(s))
    el = time.perf_counter() - t0
    value = args.steps * SAMPLE_LIMBS / el / L
    sample = (f"{SAMPLE_LIMBS} of the 24 limbs of one chain per step (chain output limbs are independent), "
              f"{args.steps} steps, scaled by {SAMPLE_LIMBS}/24; the oracle restatement of example_impl (the "
              f"reference's own objects are x86 builds of sources the GPU host does not have)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "chains/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64",
            "data": "synthetic", "config": CONFIG,
            "cpu_baseline": {"value": value, "unit": "chains/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "chains/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------- GPU
def our_arm(args):
    import torch
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import heal_gb300
    from heal_gb300 import capi
    from heal_gb300 import params as P
    from heal_gb300.chain import KeyswitchChain
    heal_gb300.build()
    capi.check(capi.lib().heal_init(local))
    stream = torch.cuda.ExternalStream(capi.stream())

    ch = KeyswitchChain(n=N, limbs=L, digits=D, base_bits=BITS, bound_bits=BOUND)
    cts_host = [P.residues(1000 + i, ch.shape(), ch.qs) for i in range(RING)]
    cts = [capi.DeviceArray.from_numpy(c) for c in cts_host]
    outs = [capi.DeviceArray.empty(ch.shape(), np.int64) for _ in range(RING)]

    def barrier():
        torch.cuda.synchronize()
        capi.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # host time to enqueue the first HOST_SAMPLE chains of the last timed
    # loop, while the device's launch queue still has room (later launches
    # wait for queue space, so the loop as a whole advances at the device's
    # pace): the host's own cost per chain, to compare with the device time
    HOST_SAMPLE = 32
    host_ms = {"last": 0.0, "n": 1}

    def enqueue(fn, steps):
        h0 = time.perf_counter()
        for s in range(steps):
            fn(s)
            if s + 1 == min(HOST_SAMPLE, steps):
                host_ms["last"], host_ms["n"] = (time.perf_counter() - h0) * 1e3, s + 1

    def timed(fn, steps):
        barrier()
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = capi.launches()
        start.record(stream)
        enqueue(fn, steps)
        stop.record(stream)
        stop.synchronize()
        barrier()
        ms = max_over_ranks(start.elapsed_time(stop), world, "cuda")
        return ms, capi.launches() - l0

    # ---- NTT plans for the chain's shapes (the autotuner, before any timing)
    plans = ch.tune(cts[0]) if not args.no_tune else None
    ch.run(cts[0], outs[0])
    # two chains in flight: even steps on the library stream, odd steps on a
    # args.inflight chains in flight: step s runs on chain s % K, each chain
    # with its own intermediates (twins share the resident tables and key)
    # and its own stream (chain 0 on the library stream), so that one chain's
    # kernels fill the tails of the others'
    K = max(1, args.inflight)
    chains = [ch] + [ch.twin() for _ in range(K - 1)]
    sides = [torch.cuda.Stream() for _ in range(K - 1)]
    ch2, side = (chains[1], sides[0]) if K > 1 else (ch.twin(), torch.cuda.Stream())  # the e2e pipeline's pair
    lib = capi.lib()

    def on(st):
        capi.check(lib.heal_set_stream(st.cuda_stream if st is not None else None))

    def in_flight(method):
        def step(s):
            c = s % K
            if c:
                on(sides[c - 1])
                getattr(chains[c], method)(cts[s % RING], outs[s % RING])
                on(None)
            else:
                getattr(ch, method)(cts[s % RING], outs[s % RING])
        return step

    chain_step2 = in_flight("run")

    def timed2(fn, steps):
        barrier()
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = capi.launches()
        start.record(stream)
        for sd in sides:
            sd.wait_event(start)
        enqueue(fn, steps)
        for sd in sides:
            joined = torch.cuda.Event()
            joined.record(sd)
            stream.wait_event(joined)
        stop.record(stream)
        stop.synchronize()
        barrier()
        return max_over_ranks(start.elapsed_time(stop), world, "cuda"), capi.launches() - l0

    chain_step = lambda s: ch.run(cts[s % RING], outs[s % RING])
    # one timed step is CHAINS_PER_STEP chains; the timed loops below count chains
    nch = args.steps * CHAINS_PER_STEP
    for w in range(args.warmup * CHAINS_PER_STEP):
        chain_step2(w)
    with Clocks(local) as clk:
        ms, launches = timed2(chain_step2, nch)
    clocks = clk.summary()
    host_us = {"resident": host_ms["last"] * 1e3 / host_ms["n"]}
    value = whole_job_rate(nch, world, ms)
    for w in range(args.warmup):
        chain_step(w)
    ms_one, _ = timed(chain_step, nch)
    value_one = whole_job_rate(nch, world, ms_one)

    # ---- the same chain fused into 3 calls: intt, heal_g_decomposition_ntt,
    # heal_modmul_axis_sum_permute
    want0 = outs[0].numpy()

    fused_step2 = in_flight("run_fused")

    fused_step = lambda s: ch.run_fused(cts[s % RING], outs[s % RING])
    for w in range(args.warmup):
        fused_step2(w)
    ms_f2, launches_f = timed2(fused_step2, nch)
    for w in range(args.warmup):
        fused_step(w)
    ms_f1, _ = timed(fused_step, nch)
    ch.run_fused(cts[0], outs[0])
    assert np.array_equal(outs[0].numpy(), want0), "fused chain differs from the per-call chain"
    tail = lambda s: capi.call("heal_modmul_axis_sum_permute", ch.prod_moved, ch.key_moved, ch.dev["p"], 3,
                               ch.dev["gal"], 2, 1, outs[s % RING])
    for w in range(3):
        tail(w)
    reps = max(200, args.steps)                      # calls per kernel-level timing
    tail_ms, _ = timed(tail, reps)
    value_f = whole_job_rate(nch, world, ms_f2)
    # the fused chain on 8 ciphertexts per call (one [16, N, 1, L] tensor, the key broadcast)
    KB = 8
    kb = ch.batched(KB)
    kcts = [capi.DeviceArray.from_numpy(np.concatenate([cts_host[(j + i) % RING] for i in range(KB)], axis=0))
            for j in range(2)]
    kouts = [capi.DeviceArray.empty(kb.shape(), np.int64) for _ in range(2)]
    kb.run(kcts[0], kouts[0])
    assert np.array_equal(kouts[0].numpy()[:2], want0), "batched fused chain differs from the per-call chain"
    for w in range(args.warmup):
        kb.run(kcts[w % 2], kouts[w % 2])
    ksteps = max(5, nch // KB)
    ms_kb, _ = timed(lambda s: kb.run(kcts[s % 2], kouts[s % 2]), ksteps)
    batched_rate = whole_job_rate(ksteps * KB, world, ms_kb)
    fused_chain = {"value": value_f, "unit": "chains/s", "value_one_stream": whole_job_rate(nch, world, ms_f1),
                   "batched_8_per_call": batched_rate,
                   "vs_per_call": value_f / value, "calls_per_chain": 3, "launches_per_chain": launches_f / nch,
                   "tail_ms_per_call": tail_ms / reps,
                   "tail_achieved_GBps": (2 * 2 * N * L * D + 2 * N * L) * 8 / (tail_ms / reps / 1e3) / 1e9,
                   "hbm_frac": ch.bytes_per_chain_fused() * value_f / world / 1e9 / peaks()[0],
                   "workload": "the same chain in 3 calls: intt; g_decomposition -> ntt as one "
                               "heal_g_decomposition_ntt; modmul(key) -> axis_modsum(digits) -> permute as one "
                               "heal_modmul_axis_sum_permute; bit-identical to the per-call chain (checked)"}

    # ---- batched NTT of the digits (the dominant kernel) and the per-call split
    ntt_step = lambda s: capi.call("heal_ntt", ch.dig_flat, ch.dev["p_t"], ch.dev["perm"], ch.dev["tw_t"],
                                   None, None, ch.dn)
    for w in range(3):
        ntt_step(w)
    ntt_ms, ntt_launches = timed(ntt_step, reps)
    ntt_call_ms = ntt_ms / reps
    limbs_per_call = 2 * L * D
    ntt_bytes = 2 * limbs_per_call * N * 8           # read + write of every limb once
    hbm, peak_kind = peaks()
    achieved = ntt_bytes / (ntt_call_ms / 1e3) / 1e9
    traffic = profile_traffic()
    chain_bytes = ch.bytes_per_chain()
    # the integer-pipe ceiling: the same 64-bit butterfly with its operands in registers
    import ctypes
    peak_bf = ctypes.c_double()
    capi.check(capi.lib().heal_ntt_butterfly_peak(256, ctypes.byref(peak_bf)))
    ntt_bf = limbs_per_call * (N // 2) * int(np.log2(N))
    int_roofline = {"bound": "integer pipes", "kernel": "heal_ntt of the 72 digit limbs ([2, 65536, 1, 72] int64)",
                    "achieved": ntt_bf / (ntt_call_ms / 1e3) / 1e9, "peak": peak_bf.value / 1e9,
                    "unit": "Gbutterfly/s", "frac": ntt_bf / (ntt_call_ms / 1e3) / peak_bf.value,
                    "butterflies_per_call": ntt_bf,
                    "peak_kind": "measured live: the same 64-bit growing-range butterfly with its operands in "
                                 "registers (heal_ntt_butterfly_peak)"}

    # ---- per-call split of one chain step (CUDA events around each HEAL call)
    names = ["intt", "g_decomposition", "ntt", "modmul_ttt", "axis_modsum", "permute"]
    d = ch.dev
    calls = [lambda s: capi.call("heal_intt", cts[s % RING], d["p"], d["perm"], d["itw"], d["minv"], None, None, ch.x),
             lambda s: capi.call("heal_g_decomposition", ch.x, ch.dig, D, BITS),
             lambda s: capi.call("heal_ntt", ch.dig_flat, d["p_t"], d["perm"], d["tw_t"], None, None, ch.dn),
             lambda s: capi.call("heal_modmul_ttt", ch.dn, d["key"], d["p_t"], ch.dn),
             lambda s: capi.call("heal_axis_modsum", ch.prod_moved, d["p"], ch.acc, 3),
             lambda s: capi.call("heal_permute", ch.acc, d["gal"], outs[s % RING], 2, 1)]
    nsplit = 50
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(len(calls) + 1)] for _ in range(nsplit)]
    barrier()
    for s in range(nsplit):
        evs[s][0].record(stream)
        for ci, fn in enumerate(calls):
            fn(s)
            evs[s][ci + 1].record(stream)
    torch.cuda.synchronize()
    split_ms = {n: statistics.median(evs[s][ci].elapsed_time(evs[s][ci + 1]) for s in range(nsplit))
                for ci, n in enumerate(names)}

    # ---- end to end through the C ABI from pinned host memory.  Every step
    # copies its ciphertext in (H2D) and its result out (D2H) inside the timed
    # region.  The copies run on their own streams into a ring of E2E_RING
    # device buffers per direction, so the H2D of the next steps runs ahead
    # while the two chains in flight compute, and the D2H of a finished chain
    # overlaps the chains after it (with two buffers, a chain's input copy
    # could only start once the chain two steps back had finished, and one
    # copy time per pair of chains ran with a single chain in flight).
    E2E_RING = 4
    nbytes = 2 * N * L * 8
    import ctypes
    lib = capi.lib()
    pin_in = ctypes.c_void_p()
    capi.check(lib.heal_host_alloc(nbytes, ctypes.byref(pin_in)))
    pin_out = [ctypes.c_void_p() for _ in range(E2E_RING)]
    for p_ in pin_out:
        capi.check(lib.heal_host_alloc(nbytes, ctypes.byref(p_)))
    ctypes.memmove(pin_in, cts_host[0].ctypes.data, nbytes)
    dev_in = [capi.DeviceArray.empty(ch.shape(), np.int64, zero=False) for _ in range(E2E_RING)]
    dev_out = [capi.DeviceArray.empty(ch.shape(), np.int64, zero=False) for _ in range(E2E_RING)]
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
    ev_in, ev_comp, ev_out = ([torch.cuda.Event() for _ in range(E2E_RING)] for _ in range(3))
    use = lambda st: capi.check(lib.heal_set_stream(st.cuda_stream if st is not None else None))

    def e2e_step(s):
        b = s % E2E_RING
        s_in.wait_event(ev_comp[b])                       # the chain that last read dev_in[b]
        use(s_in)
        capi.check(lib.heal_h2d_async(ctypes.c_void_p(dev_in[b].ptr), pin_in, nbytes))
        ev_in[b].record(s_in)
        cs, chb = (stream, ch) if s % 2 == 0 else (side, ch2)  # two chains in flight, as in the resident run
        cs.wait_event(ev_in[b])
        cs.wait_event(ev_out[b])                          # the copy that last read dev_out[b]
        use(None if cs is stream else side)
        chb.run(dev_in[b], dev_out[b])
        ev_comp[b].record(cs)
        s_out.wait_event(ev_comp[b])
        use(s_out)
        capi.check(lib.heal_d2h_async(pin_out[b], ctypes.c_void_p(dev_out[b].ptr), nbytes))
        ev_out[b].record(s_out)
        use(None)

    def e2e_timed(steps):
        barrier()
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        s_in.wait_event(start)
        side.wait_event(start)
        enqueue(e2e_step, steps)
        for ev in ev_out:
            stream.wait_event(ev)
        stop.record(stream)
        stop.synchronize()
        barrier()
        return max_over_ranks(start.elapsed_time(stop), world, "cuda")

    for w in range(args.warmup):
        e2e_step(w)
    e2e_ms = e2e_timed(nch)
    e2e = whole_job_rate(nch, world, e2e_ms)
    host_us["e2e"] = host_ms["last"] * 1e3 / host_ms["n"]
    torch.cuda.synchronize()
    want = outs[0].numpy()
    for p_ in pin_out:
        got = np.frombuffer((ctypes.c_char * nbytes).from_address(p_.value), dtype=np.int64).reshape(ch.shape())
        assert np.array_equal(got, want), "e2e output differs from the resident run"

    # the same without overlap: H2D, chain, D2H back to back on one stream
    def serial_step(s):
        capi.check(lib.heal_h2d_async(ctypes.c_void_p(dev_in[0].ptr), pin_in, nbytes))
        ch.run(dev_in[0], dev_out[0])
        capi.check(lib.heal_d2h_async(pin_out[0], ctypes.c_void_p(dev_out[0].ptr), nbytes))

    for w in range(args.warmup):
        serial_step(w)
    serial_ms, _ = timed(serial_step, nch)
    e2e_serial = whole_job_rate(nch, world, serial_ms)
    capi.lib().heal_host_free(pin_in)
    for p_ in pin_out:
        capi.lib().heal_host_free(p_)

    # ---- the other configurations (reported beside the headline)
    configs = {}
    if not args.skip_configs:
        configs = other_configs(args, timed, stream)

    # ---- CPU baseline (rank 0, N = 1 only)
    cpu = None
    if world == 1 and not args.skip_cpu:
        v, threads, runs, check = cpu_sample(ch.host, cts_host[0], seconds=args.cpu_seconds, gpu_out=want0)
        cpu = {"value": v, "unit": "chains/s", "cores": threads, "kind": "port",
               "sample": f"CPU oracle chain on {SAMPLE_LIMBS} of the 24 limbs per run ({runs} runs, "
                         f"~{args.cpu_seconds:.0f} s), scaled by {SAMPLE_LIMBS}/24; every limb it computes is "
                         f"compared with the GPU chain's output for the same ciphertext", **check}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "chains/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "int64", "data": "synthetic",
                "config": CONFIG, "chains_in_flight": K, "value_one_stream": value_one,
                "ntt_limbs_per_s": limbs_per_call * reps * world / (ntt_ms / 1e3),
                "chain_hbm_frac": chain_bytes * value / world / 1e9 / hbm,
                "roofline": {"bound": "hbm", "kernel": "heal_ntt of the 72 digit limbs ([2, 65536, 1, 72] int64)",
                             "achieved": achieved, "peak": hbm, "peak_kind": peak_kind, "unit": "GB/s",
                             "frac": achieved / hbm, "algorithmic_bytes": ntt_bytes,
                             "ms_per_call": ntt_call_ms,
                             "traffic": traffic.get("bytes_per_call") if traffic else None},
                "int_roofline": int_roofline,
                "e2e": {"value": e2e, "unit": "chains/s", "h2d_bytes_per_step": nbytes * CHAINS_PER_STEP,
                        "d2h_bytes_per_step": nbytes * CHAINS_PER_STEP,
                        "pipeline": f"H2D and D2H on their own streams into a ring of {E2E_RING} device buffers "
                                    "per direction, consecutive chains alternating between two compute streams",
                        "serial_value": e2e_serial},
                "host_us_per_chain": {k: v for k, v in host_us.items()},
                "device_us_per_chain": {"resident": ms * 1e3 / nch, "e2e": e2e_ms * 1e3 / nch},
                "gpu_launches": launches, "launches_per_step": launches / args.steps,
                "split_ms": split_ms, "ntt_plans": plans, "fused_chain": fused_chain,
                "clocks": clocks, "cpu_baseline": cpu, "configs": configs}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def other_configs(args, timed, stream):
    """The other workloads, timed like the headline: the N = 4096 round-trip
    chain (plain and as one CUDA graph), the int32 NTT of [64, 65536, 1, 32],
    the ragged batch of 256 ciphertexts and the serving loop."""
    out = {}
    want = set(args.configs.split(","))
    if "roundtrip" in want:
        out["roundtrip_n4096"] = roundtrip_config(args, timed)
    if "int32_ntt" in want:
        out["int32_ntt_n65536"] = int32_ntt_config(args, timed)
    if "ragged" in want:
        out["ragged_256"] = ragged_config(args, timed)
    if "ragged_keyswitch" in want:
        out["ragged_keyswitch_256"] = ragged_keyswitch_config(args, timed)
    if "serving" in want:
        out["serving"] = serving_config(args)
    return out


def cpu_run(fn, seconds):
    """Calls fn() until ~`seconds` have passed (at least once); returns
    (seconds per call, calls, threads).  The oracle uses every host core."""
    from oracle import oracle as O
    threads = O.set_threads(os.cpu_count() or 1)
    n, t0 = 0, time.perf_counter()
    while True:
        fn()
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            return el / n, n, threads


def hbm_roofline(nbytes, ms, kernel, note=None):
    """The `roofline` object of a workload timed as a whole: algorithmic bytes
    over its CUDA-event time against the measured HBM copy bandwidth."""
    hbm, kind = peaks()
    achieved = nbytes / (ms / 1e3) / 1e9
    r = {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": hbm, "peak_kind": kind, "unit": "GB/s",
         "frac": achieved / hbm, "algorithmic_bytes": nbytes, "traffic": None}
    if note:
        r["note"] = note
    return r


def roundtrip_config(args, timed):
    import hashlib
    from heal_gb300 import capi
    from heal_gb300.configs import RoundTripChain
    from oracle.chain import oracle_roundtrip
    c1 = RoundTripChain()
    c1.run()
    with open(os.path.join(ROOT, "tests", "golden", "golden_hash.json")) as f:
        gh = json.load(f)["roundtrip_n4096"]
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a.numpy()).tobytes()).hexdigest()
    exact = sha(c1.NA) == gh["ntt_a"] and sha(c1.AS) == gh["axis_modsum"] and sha(c1.RA) == gh["intt_ntt_a"]
    steps = max(args.steps, 200)
    for _ in range(3):
        c1.run()
    ms_plain, l_plain = timed(lambda s: c1.run(), steps)
    graph = capi.Graph(c1.run)
    for _ in range(3):
        graph.launch()
    ms_graph, l_graph = timed(lambda s: graph.launch(), steps)
    exact = exact and sha(c1.AS) == gh["axis_modsum"]
    t = {k: v.numpy() for k, v in c1.t.items()}
    want = oracle_roundtrip(c1.host["A"], c1.host["B"], t["p"], t["perm"], t["tw"], t["itw"], t["minv"])
    oracle_equal = all(np.array_equal(w, g.numpy()) for w, g in zip(want, (c1.NA, c1.NB, c1.RA, c1.PR, c1.AS)))
    cpu_s, runs, threads = cpu_run(lambda: oracle_roundtrip(c1.host["A"], c1.host["B"], t["p"], t["perm"], t["tw"],
                                                            t["itw"], t["minv"]), 3.0)
    step_ms = ms_graph / steps
    return {"workload": "ntt(A), ntt(B), intt(ntt(A)), modmul, axis_modsum over the batch; [8, 4096, 1, 4] "
                        "int64, 30-bit primes", "bit_exact_vs_reference_hashes": exact,
            "oracle_equal": oracle_equal,
            "step_us_plain": ms_plain / steps * 1e3, "step_us_graph": step_ms * 1e3,
            "transform_limbs_per_s_graph": c1.transform_limbs() * steps / (ms_graph / 1e3),
            "launches_per_step": l_graph / steps,
            "roofline": hbm_roofline(c1.bytes_per_step(), step_ms, "the captured step (5 calls)",
                                     "the 10.6 MB step is L2-resident; launch latency bounds it"),
            "cpu_baseline": {"value": c1.transform_limbs() / cpu_s, "unit": "transform limbs/s", "cores": threads,
                             "kind": "port", "step_us": cpu_s * 1e6,
                             "sample": f"the whole step on the oracle, {runs} runs"}}


def int32_ntt_config(args, timed):
    from heal_gb300.configs import Int32Ntt
    from oracle import oracle as O
    c4 = Int32Ntt()
    c4.ntt()
    c4.intt()
    # full-shape parity: two of the 64 batch rows (64 limb-polynomials of 2^16 points) against the oracle's
    # 64-bit transform of the same residues widened to int64 (exact for q < 2^31)
    t = c4.host_tables
    wide = lambda a: np.asarray(a, np.int64)
    x2 = wide(c4.host_x[:2])
    want = O.ntt(x2, wide(t["p"]), wide(t["perm"]), wide(t["tw"]))
    got = c4.Y.numpy()[:2]
    ntt_equal = bool(np.array_equal(got.astype(np.int64), want))
    inv_want = O.intt(want, wide(t["p"]), wide(t["perm"]), wide(t["itw"]), wide(t["minv"]))
    intt_equal = bool(np.array_equal(c4.Z.numpy()[:2].astype(np.int64), inv_want))
    round_trip = bool(np.array_equal(c4.Z.numpy(), c4.host_x))
    st4 = max(20, args.steps)
    ms4, _ = timed(lambda s: c4.ntt(), st4)
    ms4i, _ = timed(lambda s: c4.intt(), st4)
    per = ms4 / st4
    x1 = wide(c4.host_x[:1])
    cpu_s, runs, threads = cpu_run(lambda: O.ntt(x1, wide(t["p"]), wide(t["perm"]), wide(t["tw"])), 5.0)
    return {"workload": "ntt on [64, 65536, 1, 32] int32, 31-bit primes, radix-8 Shoup butterflies on the integer "
                        "pipes", "ntt_ms": per, "intt_ms": ms4i / st4, "limbs_per_s": c4.limbs() / (per / 1e3),
            "oracle_equal": {"ntt_rows_0_1": ntt_equal, "intt_rows_0_1": intt_equal},
            "round_trip_exact": round_trip,
            "roofline": hbm_roofline(c4.bytes_per_call(), per, "heal_ntt of [64, 65536, 1, 32] int32 (two passes)"),
            "cpu_baseline": {"value": c4.L / cpu_s, "unit": "limbs/s", "cores": threads, "kind": "port",
                             "sample": f"the oracle's 64-bit NTT of one batch row (32 limbs) widened to int64, "
                                       f"{runs} runs"},
            "tensor_core_floor": tensor_floor(c4.limbs(), per)}


def tensor_floor(limb_polys: int, cuda_core_ms: float) -> dict:
    """The exact tensor-core alternative for the int32 NTT, bounded from below by the
    GEMM work alone: a four-step 256 x 256 NTT of 31-bit residues whose
    radix-256 DFTs run as byte-plane GEMMs (4 x 4 planes, exact with INT32 or
    FP32 accumulation over K = 256) costs 2 flops x 2 passes x 16 planes x
    256^3 MACs per limb-polynomial.  The dense INT8 rate is measured here with
    torch._int_mm (cuBLASLt) on 8192^3, the bf16 rate with torch.matmul; twiddle
    products, recombination and reduction mod q come on top of the floor."""
    import torch
    ops = 2 * 2 * 16 * 256 ** 3 * limb_polys
    n = 8192
    a8 = torch.randint(-64, 64, (n, n), dtype=torch.int8, device="cuda")
    b8 = torch.randint(-64, 64, (n, n), dtype=torch.int8, device="cuda")
    a16, b16 = a8.to(torch.bfloat16), b8.to(torch.bfloat16)

    def rate(fn, reps=10):
        fn()
        torch.cuda.synchronize()
        st, en = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        best = float("inf")
        for _ in range(reps):
            st.record()
            fn()
            en.record()
            en.synchronize()
            best = min(best, st.elapsed_time(en))
        return 2 * n ** 3 / (best / 1e3)

    i8 = rate(lambda: torch._int_mm(a8, b8))
    bf = rate(lambda: torch.matmul(a16, b16))
    del a8, b8, a16, b16
    return {"gemm_flop_per_call": ops, "int8_dense_tops_measured": i8 / 1e12, "bf16_dense_tflops_measured": bf / 1e12,
            "int8_floor_ms": ops / i8 * 1e3, "bf16_floor_ms": ops / bf * 1e3, "cuda_core_ntt_ms": cuda_core_ms,
            "method": "GEMM work only (4 x 4 byte planes, 2 passes of 256-point DFTs) at the rates measured in this "
                      "run; a tensor-core NTT is worth building only if its floor is well below the CUDA-core time"}


def ragged_config(args, timed):
    """Ragged batch: 256 ciphertexts of mixed ring degree and limb count, the round-trip
    chain on each; plain loop (default and autotuned NTT plans) against one
    CUDA graph (1 branch, and 8 parallel branches: 8 to 64 measured within 10%, 8 fastest), and
    the transforms of all ciphertexts batched (two heal_ntt_batch calls), plain and as one graph."""
    import hashlib
    from heal_gb300 import capi
    from heal_gb300.configs import RaggedBatch
    hbm, _ = peaks()
    t0 = time.time()
    c3 = RaggedBatch()
    setup_s = time.time() - t0
    c3.run()                                           # caches every table
    steps = max(5, args.steps // 40)
    ms_default, _ = timed(lambda s: c3.run(), steps)
    t0 = time.time()
    plans = c3.autotune()
    tune_s = time.time() - t0
    c3.run()
    ms_tuned, l_plain = timed(lambda s: c3.run(), steps)
    digest = lambda: hashlib.sha256(b"".join(np.ascontiguousarray(a.numpy()).tobytes() for a in c3.AS)).hexdigest()
    want = digest()
    res = {}
    for nb in (1, 8):
        g = c3.graph(nb)
        for a in c3.AS:                                # the replay must rewrite every output
            capi.call("heal_copy_strided", capi.DeviceArray.from_numpy(np.zeros(a.shape, np.int64)), a)
        g.launch()
        same = digest() == want
        ms, launches = timed(lambda s: g.launch(), steps)
        res[nb] = (ms / steps, launches / steps, same)
        del g
    # the transforms of all 256 ciphertexts in two heal_ntt_batch calls
    for a in c3.AS:
        capi.call("heal_copy_strided", capi.DeviceArray.from_numpy(np.zeros(a.shape, np.int64)), a)
    c3.run_batched()
    batched_same = digest() == want
    ms_bplain, l_bplain = timed(lambda s: c3.run_batched(), steps)
    gb = c3.graph_batched(8)
    for a in c3.AS:
        capi.call("heal_copy_strided", capi.DeviceArray.from_numpy(np.zeros(a.shape, np.int64)), a)
    gb.launch()
    batched_same = batched_same and digest() == want
    ms_bgraph, l_bgraph = timed(lambda s: gb.launch(), steps)
    del gb
    round_trip = all(np.array_equal(c3.RA[i].numpy(), c3.A[i].numpy()) for i in range(len(c3.specs)))
    best = min(res[1][0], res[8][0], ms_bgraph / steps)
    # oracle parity and CPU baseline on every 32nd ciphertext (8 of 256, every ring degree present), the
    # CPU time scaled to the whole batch by algorithmic bytes
    from oracle.chain import oracle_roundtrip
    sample = list(range(0, len(c3.specs), 32))
    host = {i: (c3.A[i].numpy(), c3.B[i].numpy(), {k: v.numpy() for k, v in c3.views[i].items()}) for i in sample}
    oracle_equal = True
    for i in sample:
        a_, b_, v = host[i]
        want = oracle_roundtrip(a_, b_, v["p"], v["perm"], v["tw"], v["itw"], v["minv"])
        oracle_equal = oracle_equal and all(np.array_equal(w, g.numpy()) for w, g in
                                            zip(want, (c3.NA[i], c3.NB[i], c3.RA[i], c3.PR[i], c3.AS[i])))
    cpu_s, runs, threads = cpu_run(lambda: [oracle_roundtrip(host[i][0], host[i][1], *(host[i][2][k] for k in
                                                             ("p", "perm", "tw", "itw", "minv"))) for i in sample],
                                   5.0)
    scale = c3.bytes_per_step() / sum(c3.bytes_of(i) for i in sample)
    shapes = sorted(plans)
    return {"workload": "256 ciphertexts [2, N, 1, L] int64, N in 2^12..2^16, L uniform in 2..32, 30-bit primes; "
                        "ntt(A), ntt(B), intt(ntt(A)), modmul, axis_modsum per ciphertext (1280 calls per step)",
            "ring_degrees": {str(n): sum(1 for m, _ in c3.specs if m == n) for n in sorted({n for n, _ in c3.specs})},
            "elements_per_tensor_set": c3.elements(),
            "step_ms_plain_default_plans": ms_default / steps,
            "step_ms_plain_tuned_plans": ms_tuned / steps,
            "step_ms_graph_1_branch": res[1][0], "step_ms_graph_8_branches": res[8][0],
            "step_ms_batched_plain": ms_bplain / steps, "step_ms_batched_graph_8_branches": ms_bgraph / steps,
            "batched_launches_per_step": l_bgraph / steps, "batched_equals_loop": batched_same,
            "graph_speedup_vs_plain": (ms_default / steps) / best,
            "ciphertexts_per_s": len(c3.specs) / (best / 1e3),
            "transform_limbs_per_s": c3.transform_limbs() / (best / 1e3),
            "hbm_frac": c3.bytes_per_step() / (best / 1e3) / 1e9 / hbm,
            "launches_per_step": res[8][1], "plain_launches_per_step": l_plain / steps,
            "graph_equals_loop": res[1][2] and res[8][2], "round_trip_exact": round_trip,
            "oracle_equal": {"ciphertexts_checked": len(sample), "equal": oracle_equal},
            "roofline": hbm_roofline(c3.bytes_per_step(), best, "the fastest form of the step"),
            "cpu_baseline": {"value": len(c3.specs) / (cpu_s * scale), "unit": "ciphertexts/s", "cores": threads,
                             "kind": "port", "sample": f"the oracle chain on {len(sample)} of the 256 ciphertexts "
                                                       f"({runs} runs), scaled to the batch by algorithmic bytes"},
            "autotuned_shapes": len(shapes), "autotune_s": tune_s, "setup_s": setup_s,
            "plans_sample": {f"{n}x{l}": {"fwd": plans[(n, l)][0], "inv": plans[(n, l)][1]}
                             for n, l in shapes[:: max(1, len(shapes) // 6)]}}


def ragged_keyswitch_config(args, timed):
    """Ragged keyswitch: the fused keyswitch step (INTT, g_decomposition + NTT of
    the digits, modmul -> axis_modsum -> permute) of 256 ciphertexts of mixed
    ring degree and limb count, as the plain loop of three calls per
    ciphertext, as that loop captured in one CUDA graph, and as one
    heal_keyswitch_batch launch; the same on 256 small-ring ciphertexts
    (N in 2^12, 2^13), where launch costs dominate."""
    import gc
    from heal_gb300 import capi
    from heal_gb300.configs import RaggedKeyswitch
    from oracle.chain import oracle_chain
    hbm, _ = peaks()
    res = {"workload": "256 ciphertexts [2, N, 1, L] int64, N in 2^12..2^16, L uniform in 2..32, 50-bit primes; "
                       "intt -> g_decomposition (D=3, base 2^17) + ntt of the digits -> modmul(key) -> "
                       "axis_modsum(digits) -> permute(X->X^5) per ciphertext"}
    for name, kw in (("mixed", {}), ("small_rings", {"logns": (12, 13), "lmax": 16})):
        t0 = time.time()
        rk = RaggedKeyswitch(**kw)
        setup_s = time.time() - t0
        rk.run()
        want = [o.numpy() for o in rk.outs]
        steps = max(5, args.steps // 4)
        for _ in range(2):
            rk.run()
        ms_loop, l_loop = timed(lambda s: rk.run(), steps)
        g = capi.Graph(rk.run)
        for _ in range(2):
            g.launch()
        ms_graph, l_graph = timed(lambda s: g.launch(), steps)
        del g
        for _ in range(2):
            rk.run_batched()
        ms_batch, l_batch = timed(lambda s: rk.run_batched(), steps)
        equal = all(np.array_equal(o.numpy(), w) for o, w in zip(rk.outs, want))
        # the oracle on the two smallest ciphertexts
        small = sorted(range(len(rk.specs)), key=lambda i: rk.specs[i][0] * rk.specs[i][1])[:2]
        oracle_equal = all(np.array_equal(want[i], oracle_chain(rk.host_tables(i), rk.host_cts[i], rk.D, rk.BITS))
                           for i in small)
        best = ms_batch / steps
        r = {"ring_degrees": {str(n): sum(1 for m, _ in rk.specs if m == n) for n in sorted({n for n, _ in rk.specs})},
             "step_ms_loop": ms_loop / steps, "step_ms_graph": ms_graph / steps, "step_ms_persistent": best,
             "launches_per_step_loop": l_loop / steps, "launches_per_step_persistent": l_batch / steps,
             "persistent_vs_loop": ms_loop / ms_batch, "persistent_vs_graph": ms_graph / ms_batch,
             "ciphertexts_per_s_persistent": len(rk.specs) / (best / 1e3),
             "persistent_equals_loop": equal, "oracle_equal": {"ciphertexts_checked": len(small), "equal": oracle_equal},
             "roofline": hbm_roofline(rk.bytes_per_step(), best, "heal_keyswitch_batch (one persistent launch)"),
             "setup_s": setup_s}
        if name == "mixed":
            i0 = small[0]
            cpu_s, runs, threads = cpu_run(lambda: oracle_chain(rk.host_tables(i0), rk.host_cts[i0], rk.D, rk.BITS),
                                           3.0)
            n0, l0 = rk.specs[i0]
            scale = rk.bytes_per_step() / (2 * n0 * l0 * 8 * (2 + 4 + 7))
            r["cpu_baseline"] = {"value": len(rk.specs) / (cpu_s * scale), "unit": "ciphertexts/s", "cores": threads,
                                 "kind": "port", "sample": f"the oracle chain on one ciphertext (N={n0}, L={l0}, "
                                                           f"{runs} runs), scaled to the batch by algorithmic bytes"}
        res[name] = r
        del rk
        gc.collect()
    return res


def serving_config(args, count: int = 4000, rate: float = 2000.0):
    """Serving loop: Poisson arrivals of ciphertext x plaintext-matrix products
    admitted by HBM footprint; served with the three HEAL calls (permute
    rotations, modmul, axis_modsum) and with the fused modmul_axis_sum.  The
    fused path is then offered the same schedule at rising rates until it
    saturates (throughput below 90% of the offered rate), which measures its
    capacity and where its p99 latency breaks."""
    from heal_gb300 import serving as S
    out = {"workload": f"{count} Poisson arrivals at {rate:.0f}/s of ct[2][N][L] x (d x d plaintext matrix): "
                       "d in {16, 64, 256}, N in {2^14, 2^15}, L uniform in 8..16, 40-bit primes; sum over d Galois "
                       "rotations of rot_i(ct) * diag_i, H2D of the matrix and D2H of the result per request"}
    for name, fused in (("three_calls", False), ("fused", True)):
        srv, setup_s = serving_server(fused)
        out[name] = serve_once(srv, count, rate, setup_s)
        if fused:
            sweep = []
            for r in (4000.0, 8000.0, 16000.0, 32000.0, 64000.0):
                res = serve_once(srv, count, r, setup_s, detail=False)
                sweep.append(res)
                if res["throughput_req_per_s"] < 0.9 * res["offered_req_per_s"]:
                    break
            out["fused_rate_sweep"] = sweep
            out["fused_capacity_req_per_s"] = max(x["throughput_req_per_s"] for x in sweep + [out[name]])
            out["fused_from_transcripts"] = serve_transcripts(srv)
            out["cpu_baseline"] = serving_cpu(srv)
            out["roofline"] = dict(hbm_roofline(out[name]["algorithmic_GBps"] * 1e9, 1e3,
                                                "the fused serving loop at the offered rate"),
                                   note="achieved = algorithmic bytes of the served requests over the run's span; "
                                        "the loop is bound by the offered load, not by HBM")
        del srv
    return out


def serve_transcripts(srv, count: int = 480, runs=((500.0, 0), (2000.0, 0), (2000.0, 4), (4000.0, 4))):
    """The fused path with every request arriving as a HEAL transcript (the
    UTF-8 JSON bytes a client sends, the diagonals as base64 np.save
    payloads), decoded on arrival: latency and throughput with the intake
    included for each (offered rate, intake threads; 0 = decoded on the
    loop's own thread), and the decode time alone."""
    import torch
    from heal_gb300 import serving as S
    out = {"intake": "HEAL's JSON transcript format: host_to_device of the diagonals (np.save, base64), matvec on "
                     "a resident ciphertext, device_to_host; decoded on arrival inside the timed loop (payloads "
                     "cut out of the JSON and decoded by heal_base64_decode, used in place)", "rates": []}
    for k, (rate, threads) in enumerate(runs):
        reqs = S.poisson_schedule(count, rate, 808, srv.ns, srv.ds, srv.lmin, srv.lmax, srv.cts, srv.mats)
        texts = {r.rid: S.matvec_transcript(S.ct_name(r.n, r.l, r.ct), srv.host_mats[(r.d, r.l, r.mat)][r.n].numpy())
                 .encode() for r in reqs}
        if k == 0:
            dec = {}
            for r in reqs[:48]:
                t1 = time.perf_counter()
                q = srv.from_transcript(texts[r.rid], r.rid, 0.0)
                dec.setdefault(r.d, []).append((time.perf_counter() - t1) * 1e3)
                srv.recycle(q)
            out["decode_ms_p50_by_d"] = {d: statistics.median(v) for d, v in sorted(dec.items())}
            out["mean_transcript_MB"] = sum(len(t) for t in texts.values()) / count / 1e6
        sample = [r.rid for r in reqs[:: count // 8]]
        st = srv.run(reqs, keep=sample, transcripts=texts, intake_threads=threads)
        torch.cuda.synchronize()
        same = all(np.array_equal(srv.out_host[i], srv.alone(reqs[i])) for i in sample)
        ms = lambda xs, q: S.percentile(xs, q) * 1e3
        out["rates"].append({"intake_threads": threads, "requests": count,
                             "offered_req_per_s": count / reqs[-1].arrival,
                             "throughput_req_per_s": count / st.span, "p50_ms": ms(st.latencies, 50),
                             "p99_ms": ms(st.latencies, 99), "max_queue": st.max_queue, "alone_equals_mix": same})
    return out


def serving_server(fused):
    from heal_gb300 import serving as S
    t0 = time.time()
    srv = S.MatVecServer(fused=fused)
    srv.warm()
    return srv, time.time() - t0


def serving_cpu(srv):
    """The oracle's service rate for the request mix: one request of each d at
    N = 2^14, L = 8 timed on the oracle (permute, modmul, axis_modsum on every
    host core), the time per multiply-add fitted over the three and scaled to
    the mix's mean request (E[d] E[N] E[L], the draws being independent)."""
    from oracle.chain import oracle_matvec
    n, l = min(srv.ns), srv.lmin
    ct = srv.ct[(n, l)][0].numpy()
    p = np.array(srv.qs[n][:l], np.int64)
    work, secs, threads = 0, 0.0, 1
    for d in srv.ds:
        t, _, threads = cpu_run(lambda: oracle_matvec(ct, srv.perms[(n, d)].numpy(),
                                                      srv.host_mats[(d, l, 0)][n].numpy(), p), 0.5)
        work += 2 * d * n * l
        secs += t
    mean_work = 2 * np.mean(srv.ds) * np.mean(srv.ns) * (srv.lmin + srv.lmax) / 2
    return {"value": 1.0 / (secs / work * mean_work), "unit": "req/s", "cores": threads, "kind": "port",
            "sample": f"one request per d in {list(srv.ds)} at N={n}, L={l} on the oracle; scaled to the mean "
                      f"request of the mix by multiply-adds, requests served one after another"}


def serve_once(srv, count, rate, setup_s, detail=True):
    import torch
    from heal_gb300 import serving as S
    fused = srv.fused
    reqs = S.poisson_schedule(count, rate, 606, srv.ns, srv.ds, srv.lmin, srv.lmax, srv.cts, srv.mats)
    sample = [r.rid for r in reqs[:: count // 8]]
    st = srv.run(reqs, keep=sample)
    torch.cuda.synchronize()
    same = all(np.array_equal(srv.out_host[i], srv.alone(reqs[i])) for i in sample)
    moved = sum(S.MatVecServer.bytes_moved(r) for r in reqs)
    ms = lambda xs, q: S.percentile(xs, q) * 1e3
    res = {"p50_ms": ms(st.latencies, 50), "p99_ms": ms(st.latencies, 99),
           "mean_ms": float(np.mean(st.latencies)) * 1e3,
           "p50_wait_ms": ms(st.waits, 50), "p99_wait_ms": ms(st.waits, 99),
           "throughput_req_per_s": count / st.span, "offered_req_per_s": count / reqs[-1].arrival,
           "algorithmic_GBps": moved / st.span / 1e9, "max_inflight": st.max_inflight, "max_queue": st.max_queue,
           "alone_equals_mix": same}
    if not detail:
        return res
    alone_ms = {}
    for d in srv.ds:                                   # service time of the largest request of each d
        r = S.Request(-1, 0.0, max(srv.ns), srv.lmax, d, 0, 0)
        ts = []
        for _ in range(5):
            t1 = time.perf_counter()
            srv.alone(r)
            ts.append((time.perf_counter() - t1) * 1e3)
        alone_ms[str(d)] = statistics.median(ts)
    big = S.Request(-1, 0.0, max(srv.ns), srv.lmax, max(srv.ds), 0, 0)
    res.update({"arena_GiB": srv.arena_size / 2**30, "peak_arena_GiB": st.peak_bytes / 2**30,
                "streams": len(srv.streams), "service_ms_alone_largest": alone_ms, "setup_s": setup_s,
                "split_ms_largest": srv.split_ms(big), "largest_request_bytes": S.MatVecServer.bytes_moved(big)})
    return res


def request_probe(args):
    """--mode request: one serving request (d = --d, N = --n, L = 16) on a
    one-shape server, each of its calls timed with CUDA events; for ncu
    captures of the serving kernels.  --fused selects the fused path."""
    import heal_gb300
    from heal_gb300 import capi
    from heal_gb300 import serving as S
    heal_gb300.build()
    capi.check(capi.lib().heal_init(0))
    srv = S.MatVecServer(ns=(args.n,), ds=(args.d,), lmin=16, lmax=16, cts=1, mats=1, budget=4 << 30, streams=1,
                         fused=args.fused)
    srv.warm()
    r = S.Request(-1, 0.0, args.n, 16, args.d, 0, 0)
    print(json.dumps({"mode": "request", "d": args.d, "n": args.n, "fused": args.fused,
                      "split_ms": srv.split_ms(r, reps=3)}), flush=True)
    return 0


def tail_probe(args):
    """--mode tail: heal_modmul_axis_sum_permute alone on the keyswitch tail
    shape (digit transforms and key [2, 65536, 1, 72] int64 -> [2, 65536, 1,
    24]), for ncu captures; prints one JSON line with the CUDA-event time."""
    import torch
    import heal_gb300
    from heal_gb300 import capi
    from heal_gb300 import params as P
    from heal_gb300.chain import KeyswitchChain
    heal_gb300.build()
    capi.check(capi.lib().heal_init(0))
    ch = KeyswitchChain(n=N, limbs=L, digits=D, base_bits=BITS, bound_bits=BOUND)
    ct = capi.DeviceArray.from_numpy(P.residues(5, ch.shape(), ch.qs))
    outs = [capi.DeviceArray.empty(ch.shape(), np.int64) for _ in range(2)]
    ch.run(ct, outs[0])
    tail = lambda s: capi.call("heal_modmul_axis_sum_permute", ch.prod_moved, ch.key_moved, ch.dev["p"], 3,
                               ch.dev["gal"], 2, 1, outs[s % 2])
    for s in range(args.warmup):
        tail(s)
    capi.synchronize()
    stream = torch.cuda.ExternalStream(capi.stream())
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for s in range(args.steps):
        tail(s)
    stop.record(stream)
    stop.synchronize()
    ms = start.elapsed_time(stop) / args.steps
    nbytes = (2 * 2 * N * L * D + 2 * N * L) * 8
    print(json.dumps({"mode": "tail", "ms_per_call": ms, "algorithmic_bytes": nbytes,
                      "achieved_GBps": nbytes / (ms / 1e3) / 1e9}), flush=True)
    return 0


def ntt_probe(args):
    """--mode ntt: one batched NTT alone, for ncu captures of the pass
    kernels.  --probe digits: [batch, 65536, 1, 72] int64 under the chain's
    50-bit primes tiled 3x (the digit tensor of batch/2 chains); --probe int32:
    [batch, 65536, 1, 32] int32 under 31-bit primes (--probe int32-intt: its
    INTT); --probe ct-intt: the INTT
    of [batch, 65536, 1, 24] int64 (the chain's ciphertext); --probe
    gdec-digits: heal_g_decomposition_ntt of [batch, 65536, 1, 24] into the
    [batch, 65536, 1, 72] digit transform (D = 3, base 2^17).  Prints one JSON
    line with the CUDA-event time per call."""
    import torch
    import heal_gb300
    from heal_gb300 import capi
    from heal_gb300 import params as P
    heal_gb300.build()
    capi.check(capi.lib().heal_init(0))
    stream = torch.cuda.ExternalStream(capi.stream())
    inverse = args.probe in ("ct-intt", "int32-intt")
    if args.probe in ("int32", "int32-intt"):
        dt, k, qs = np.int32, 32, P.ntt_primes(1 << 31, N, 32)
        p_t, perm, tw_t, itw, minv = P.ntt_tables(qs, N, dt)
    elif inverse:
        dt, k = np.int64, L
        qs = P.ntt_primes(1 << BOUND, N, L)
        p_t, perm, tw_t, itw, minv = P.ntt_tables(qs, N)
    else:
        dt, k = np.int64, L * D
        qs = P.ntt_primes(1 << BOUND, N, L)
        p, perm, tw, itw, minv = P.ntt_tables(qs, N)
        p_t, tw_t = np.repeat(p, D), np.repeat(tw, D, axis=0)
    shape = (args.batch, N, 1, k)
    gdec = args.probe == "gdec-digits"
    src_shape = (args.batch, N, 1, L) if gdec else shape
    x = capi.DeviceArray.from_numpy(P.residues(3, src_shape, qs if gdec else p_t, dt))
    y = capi.DeviceArray.empty(shape, dt)
    dev = [capi.DeviceArray.from_numpy(v) for v in (p_t, perm, itw if inverse else tw_t, minv)]
    if inverse:
        call = lambda: capi.call("heal_intt", x, dev[0], dev[1], dev[2], dev[3], None, None, y)
    elif gdec:
        call = lambda: capi.call("heal_g_decomposition_ntt", x, D, BITS, dev[0], dev[1], dev[2], y)
    else:
        call = lambda: capi.call("heal_ntt", x, dev[0], dev[1], dev[2], None, None, y)
    for _ in range(args.warmup):
        call()
    capi.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(args.steps):
        call()
    stop.record(stream)
    stop.synchronize()
    ms = start.elapsed_time(stop) / args.steps
    limbs = args.batch * k
    esz = np.dtype(dt).itemsize
    nbytes = (src_shape[0] * src_shape[3] + limbs) * N * esz  # the source read once, the result written once
    print(json.dumps({"mode": "ntt", "probe": args.probe, "shape": list(shape), "ms_per_call": ms,
                      "limbs_per_s": limbs / (ms / 1e3),
                      "algorithmic_GBps": nbytes / (ms / 1e3) / 1e9}), flush=True)
    return 0


def strided_probe(args):
    """--mode strided: the strided and batched kernels, each call timed with
    CUDA events (for ncu captures): heal_copy_strided of a transposed
    [65536, 64] int64 view (make_contiguous's gather), heal_modmul_ttt of a
    [64, 65536] product whose second operand is broadcast over the rows (the
    vector-unit strided kernel), heal_permute of a [8, 4096, 64] source read
    through a transposed view (the general gather), and heal_ntt_batch of 64
    ragged transforms (N 2^12..2^16, 2..8 limbs, 50-bit primes)."""
    import torch
    import heal_gb300
    from heal_gb300 import capi
    from heal_gb300 import params as P
    heal_gb300.build()
    capi.check(capi.lib().heal_init(0))
    stream = torch.cuda.ExternalStream(capi.stream())
    rng = np.random.default_rng(5)
    qs = np.array(P.ntt_primes(1 << 50, 1 << 12, 64), np.int64)
    # copy_strided: the transpose of a [64, 65536] tensor viewed [65536, 64]
    src = capi.DeviceArray.from_numpy(P.residues(1, (64, 1 << 16), np.resize(qs, 1 << 16)))
    srcT = capi.DeviceArray(src.buf, np.int64, (1 << 16, 64), (1, 1 << 16), src.offset)
    dst = capi.DeviceArray.empty((1 << 16, 64), np.int64)
    # modmul with b broadcast over the rows: result [64, 65536] contiguous, b [1, 65536] (stride 0 on rows)
    a = capi.DeviceArray.from_numpy(P.residues(2, (64, 1 << 16), np.resize(qs, 1 << 16)))
    b = capi.DeviceArray.from_numpy(P.residues(3, (1, 1 << 16), np.resize(qs, 1 << 16)))
    pv = capi.DeviceArray.from_numpy(np.resize(qs, 1 << 16))
    prod = capi.DeviceArray.empty((64, 1 << 16), np.int64)
    # permute of a source read through a transposed view: [8, 4096, 64] from a [64, 4096, 8] buffer
    pbuf = capi.DeviceArray.from_numpy(rng.integers(0, 1 << 40, size=(64, 4096, 8), dtype=np.int64))
    psrc = capi.DeviceArray(pbuf.buf, np.int64, (8, 4096, 64), (1, 8, 4096 * 8), pbuf.offset)
    perms = capi.DeviceArray.from_numpy(np.stack([rng.permutation(4096) for _ in range(8)]).astype(np.int64))
    pout = capi.DeviceArray.empty((8, 4096, 64), np.int64)
    # a ragged batch of forward transforms
    jobs, keep = [], []
    for i in range(64):
        n, l = 1 << int(12 + i % 5), 2 + i % 7
        q = P.ntt_primes(1 << 50, n, l)
        pp, perm, tw, _, _ = P.ntt_tables(q, n)
        arrs = [capi.DeviceArray.from_numpy(v) for v in (P.residues(100 + i, (2, n, 1, l), q), pp, perm, tw)]
        out = capi.DeviceArray.empty((2, n, 1, l), np.int64)
        keep += arrs + [out]
        jobs.append((arrs[0], arrs[1], arrs[2], arrs[3], None, out))
    calls = {"copy_strided": lambda: capi.call("heal_copy_strided", srcT, dst),
             "modmul_broadcast": lambda: capi.call("heal_modmul_ttt", a, b, pv, prod),
             "permute_general": lambda: capi.call("heal_permute", psrc, perms, pout, 0, 1),
             "ntt_batch_64": lambda: capi.ntt_batch(False, jobs)}
    res = {}
    for name, fn in calls.items():
        for _ in range(args.warmup):
            fn()
        capi.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        e1.synchronize()
        res[name] = e0.elapsed_time(e1) / args.steps
    print(json.dumps({"mode": "strided", "ms_per_call": res}), flush=True)
    return 0


def keyswitch_batch_probe(args):
    """--mode ksbatch: one heal_keyswitch_batch of --batch ciphertexts (ring
    degrees 2^12..2^16, 2..8 limbs), timed with CUDA events (for ncu)."""
    import torch
    import heal_gb300
    from heal_gb300 import capi
    from heal_gb300.configs import RaggedKeyswitch
    heal_gb300.build()
    capi.check(capi.lib().heal_init(0))
    stream = torch.cuda.ExternalStream(capi.stream())
    rk = RaggedKeyswitch(count=args.batch, lmin=2, lmax=8, seed=31)
    for _ in range(args.warmup):
        rk.run_batched()
    capi.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        rk.run_batched()
    e1.record(stream)
    e1.synchronize()
    capi.synchronize()
    print(json.dumps({"mode": "ksbatch", "ciphertexts": args.batch, "ms_per_call": e0.elapsed_time(e1) / args.steps,
                      "algorithmic_GBps": rk.bytes_per_step() / (e0.elapsed_time(e1) / args.steps / 1e3) / 1e9}),
          flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20, help="timed steps (a chain step is CHAINS_PER_STEP chains)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-configs", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="default NTT plans instead of autotuned ones")
    ap.add_argument("--configs", default=",".join(WORKLOADS),
                    help="comma-separated configurations reported beside the headline")
    ap.add_argument("--mode", default="chain", choices=["chain", "ntt", "request", "tail", "strided", "ksbatch"])
    ap.add_argument("--d", type=int, default=64, help="--mode request: matrix dimension")
    ap.add_argument("--n", type=int, default=1 << 14, help="--mode request: ring degree")
    ap.add_argument("--fused", action="store_true", help="--mode request: the fused path")
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--inflight", type=int, default=2, help="chains in flight on their own streams")
    ap.add_argument("--probe", default="digits", choices=["digits", "int32", "int32-intt", "ct-intt", "gdec-digits"])
    args = ap.parse_args()
    unknown = set(args.configs.split(",")) - set(WORKLOADS) - {""}
    if unknown:
        ap.error(f"--configs: unknown workload(s) {', '.join(sorted(unknown))}; known: {', '.join(WORKLOADS)}")
    if args.warmup < 3:
        args.warmup = 3
    if args.mode == "ntt":
        return ntt_probe(args)
    if args.mode == "tail":
        return tail_probe(args)
    if args.mode == "strided":
        return strided_probe(args)
    if args.mode == "ksbatch":
        return keyswitch_batch_probe(args)
    if args.mode == "request":
        return request_probe(args)
    if args.impl == "reference":
        return reference_arm(args)
    return our_arm(args)


if __name__ == "__main__":
    sys.exit(main())
