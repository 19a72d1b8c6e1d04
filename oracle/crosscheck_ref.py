"""Cross-checks the oracle against HEAL's own sample implementation on seeded
random cases (test infrastructure).

The reference's example_impl is compiled from its sources into oracle/_ref/
by oracle/build_ref.sh (only where those sources are present). This script
loads that module, runs every op of the path on seeded random inputs, and
compares the outputs bit for bit with the oracle in its literal mode. The
literal mode reproduces the reference's element-type arithmetic, including
its overflows. Cases:
  ntt / intt    int32 and int64; 20-, 30- and 50-bit primes; m from 2 to
                1024; random twiddle tables (the same butterfly network,
                whatever the table); random bijective permutations;
                canonical, out-of-range and negative inputs
  modmul / modsum  ttt, ttc, tct and tcc with broadcasting, signed operands
  axis_modsum   every legal axis of 2- to 4-axis tensors, signed operands
  g_decomposition  random power and base, non-negative and negative values
  permute       random axes and in-range permutation tables
  views         random sequences of reshape / expand / squeeze / unsqueeze,
                the reference's DeviceTensor against this backend's
                descriptor edits (heal_tensor_*): dims and strides after
                every step, or the same exception status

    python oracle/crosscheck_ref.py [SEEDS]

Prints one summary line; exits 1 on the first mismatch (after printing it),
and 2 if the compiled reference is missing.
"""
from __future__ import annotations

import glob
import importlib.util
import os
import sys
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

warnings.filterwarnings("ignore", message="The given NumPy array is not writable")


def load_reference():
    hits = glob.glob(os.path.join(HERE, "_ref", "lattica_hw*.so"))
    if not hits:
        return None
    import torch  # noqa: F401  (the module links against torch's Python bindings)
    spec = importlib.util.spec_from_file_location("lattica_hw", hits[0])
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class Ref:
    """The reference's pybind functions on numpy arrays (strides kept)."""

    def __init__(self, mod):
        import torch
        self.m, self.torch = mod, torch

    def f(self, name, dt):
        return getattr(self.m, f"{name}_{'32' if np.dtype(dt) == np.int32 else '64'}")

    def up(self, x):
        return self.f("host_to_device", x.dtype)(self.torch.from_numpy(x))

    def down(self, dt, dev):
        return self.f("device_to_host", dt)(dev).numpy()

    def alloc(self, shape, dt):
        return self.f("allocate_on_hardware", dt)(list(shape))

    def ntt(self, a, p, perm, tw):
        out = self.alloc(a.shape, a.dtype)
        self.f("ntt", a.dtype)(self.up(a), self.up(p), self.up(perm), self.up(tw), None, None, out)
        return self.down(a.dtype, out)

    def intt(self, a, p, perm, itw, minv):
        out = self.alloc(a.shape, a.dtype)
        self.f("intt", a.dtype)(self.up(a), self.up(p), self.up(perm), self.up(itw), self.up(minv), None, None, out)
        return self.down(a.dtype, out)

    def modop(self, op, kind, a, b, p, out_shape):
        out = self.alloc(out_shape, a.dtype)
        bb = self.up(b) if kind[1] == "t" else int(b)
        pp = self.up(p) if kind[2] == "t" else int(p)
        self.f(f"{op}_{kind}", a.dtype)(self.up(a), bb, pp, out)
        return self.down(a.dtype, out)

    def axis_modsum(self, a, p, axis):
        out = self.alloc([d for i, d in enumerate(a.shape) if i != axis], a.dtype)
        self.f("axis_modsum", a.dtype)(self.up(a), self.up(p), out, axis)
        return self.down(a.dtype, out)

    def g_decomposition(self, a, power, bits):
        out = self.alloc(list(a.shape) + [power], a.dtype)
        self.f("g_decomposition", a.dtype)(self.up(a), out, power, bits)
        return self.down(a.dtype, out)

    def permute(self, a, perms, ew, pa):
        out = self.alloc(a.shape, a.dtype)
        self.f("permute", a.dtype)(self.up(a), self.up(perms), out, ew, pa)
        return self.down(a.dtype, out)


def ref_metadata(t):
    """(dims, strides) of a reference DeviceTensor, read from print_metadata
    (it writes "Shape: [d0 d1 ]  Strides: [s0 s1 ]" to the C++ stdout)."""
    import ctypes
    import tempfile
    libc = ctypes.CDLL(None)
    sys.stdout.flush()
    libc.fflush(None)
    with tempfile.TemporaryFile() as f:
        saved = os.dup(1)
        os.dup2(f.fileno(), 1)
        try:
            t.print_metadata()
            libc.fflush(None)
        finally:
            os.dup2(saved, 1)
            os.close(saved)
        f.seek(0)
        text = f.read().decode()
    dims = [int(x) for x in text.split("Shape: [")[1].split("]")[0].split()]
    strides = [int(x) for x in text.split("Strides: [")[1].split("]")[0].split()]
    return dims, strides


def view_sequences(rng, R, same_views, count):
    """Random sequences of reshape / expand / squeeze / unsqueeze on a fresh
    tensor, applied to the reference's DeviceTensor and to this backend's
    descriptor edits (heal_tensor_*: metadata only, no device memory)."""
    import ctypes
    from heal_gb300 import capi
    L = capi.lib()
    status_of = {ValueError: 1, IndexError: 2, RuntimeError: 3}
    for _ in range(count):
        shape = [int(x) for x in rng.choice([1, 1, 2, 3, 4], size=int(rng.integers(1, 5)))]
        ref = R.f("allocate_on_hardware", np.int64)(shape)
        d = capi.desc(None, np.int64, tuple(shape), capi._rowmajor(tuple(shape)))
        steps = []
        for _ in range(4):
            nd = d.ndim
            kind = ("expand", "squeeze", "unsqueeze", "reshape")[int(rng.integers(0, 4))]
            if kind == "expand":
                axis, rep = int(rng.integers(-nd - 1, nd + 1)), int(rng.integers(0, 4))
                call_ref = lambda: R.f("expand", np.int64)(ref, axis, rep)  # noqa: E731
                call_ours = lambda: L.heal_tensor_expand(ctypes.byref(d), axis, rep)  # noqa: E731
                steps.append(f"expand({axis}, {rep})")
            elif kind == "squeeze":
                axis = int(rng.integers(-nd - 1, nd + 1))
                call_ref = lambda: R.f("squeeze", np.int64)(ref, axis)  # noqa: E731
                call_ours = lambda: L.heal_tensor_squeeze(ctypes.byref(d), axis)  # noqa: E731
                steps.append(f"squeeze({axis})")
            elif kind == "unsqueeze":
                axis = int(rng.integers(-nd - 2, nd + 2))
                call_ref = lambda: R.f("unsqueeze", np.int64)(ref, axis)  # noqa: E731
                call_ours = lambda: L.heal_tensor_unsqueeze(ctypes.byref(d), axis)  # noqa: E731
                steps.append(f"unsqueeze({axis})")
            else:
                dims_now = list(d.dims)[:nd]
                strides_now = list(d.strides)[:nd]
                # the reference counts elements over the axes whose stride is not 0
                n = int(np.prod([x for x, st in zip(dims_now, strides_now) if st != 0] or [1]))
                if rng.random() < 0.3:
                    n = int(np.prod(dims_now))
                new = []
                while n > 1 and len(new) < 4:
                    f = int(rng.choice([f for f in (2, 3, 4, n) if n % f == 0]))
                    new.append(f)
                    n //= f
                new = new or [1]
                if rng.random() < 0.3:
                    new.insert(int(rng.integers(0, len(new) + 1)), 1)
                arr = (ctypes.c_int64 * len(new))(*new)
                call_ref = lambda: ref.reshape(new)  # noqa: E731
                call_ours = lambda: L.heal_tensor_reshape(ctypes.byref(d), len(new), arr)  # noqa: E731
                steps.append(f"reshape({new})")
            try:
                call_ref()
                ref_status = 0
            except Exception as e:  # noqa: BLE001  (the pybind-mapped C++ exception)
                ref_status = status_of.get(type(e), -1)
            ours = call_ours()
            ctx = f"start {shape}, ops {steps}"
            if ref_status or ours:
                same_views("view_errors", np.array([ours]), np.array([ref_status]), ctx)
                break
            got = (list(d.dims)[:d.ndim], list(d.strides)[:d.ndim])
            same_views("views", np.array(got[0] + [-1] + got[1]),
                       np.array(ref_metadata(ref)[0] + [-1] + ref_metadata(ref)[1]), ctx)


def primes(bits, m, k):
    from heal_gb300 import params as P
    return P.ntt_primes(1 << bits, m, k)


def values(rng, shape, qs, dt, mode):
    """Residues under the last-axis moduli: canonical, up to 4q, or signed."""
    q = np.asarray(qs, np.int64)
    x = rng.integers(0, 1 << 62, size=shape, dtype=np.int64) % q
    if mode == "wide":
        x = x + q * rng.integers(0, 4, size=shape)
    elif mode == "signed":
        x = x - q * rng.integers(0, 2, size=shape)
    return x.astype(dt)


def run(seeds: int) -> int:
    mod = load_reference()
    if mod is None:
        print("crosscheck: oracle/_ref is not built")
        return 2
    from oracle import oracle as O
    R = Ref(mod)
    counts = {}

    def same(name, got, want, ctx):
        counts[name] = counts.get(name, 0) + 1
        if got.shape != want.shape or not np.array_equal(got, want):
            bad = np.argwhere(got != want)[:3].tolist() if got.shape == want.shape else "shape"
            print(f"crosscheck MISMATCH {name} {ctx}: first differing indices {bad}")
            raise SystemExit(1)

    for seed in range(seeds):
        rng = np.random.default_rng(1000 + seed)
        # ---- ntt / intt
        for dt, bits in ((np.int64, 50), (np.int64, 30), (np.int32, 30), (np.int32, 20)):
            m = 1 << int(rng.integers(1, 11))
            l, r, k = int(rng.integers(1, 3)), int(rng.integers(1, 3)), int(rng.integers(1, 4))
            qs = primes(bits, m, k)
            p = np.asarray(qs, dt)
            tw = (rng.integers(0, 1 << 62, size=(k, m), dtype=np.int64) % np.asarray(qs)[:, None]).astype(dt)
            itw = (rng.integers(0, 1 << 62, size=(k, m), dtype=np.int64) % np.asarray(qs)[:, None]).astype(dt)
            minv = (rng.integers(1, 1 << 62, size=k, dtype=np.int64) % np.asarray(qs)).astype(dt)
            perm = rng.permutation(m).astype(dt)
            mode = ("canonical", "wide", "signed")[seed % 3]
            if dt == np.int32 and mode == "wide":
                mode = "canonical"    # 4q does not fit 32 bits
            a = values(rng, (l, m, r, k), qs, dt, mode)
            ctx = f"seed={seed} {np.dtype(dt).name} q<2^{bits} m={m} {mode}"
            same("ntt", O.ntt(a, p, perm, tw, exact=False), R.ntt(a, p, perm, tw), ctx)
            same("intt", O.intt(a, p, perm, itw, minv, exact=False), R.intt(a, p, perm, itw, minv), ctx)
        # ---- modmul / modsum with broadcasting
        for dt, bits in ((np.int64, 50), (np.int32, 30)):
            k = int(rng.integers(1, 5))
            shape = tuple(int(d) for d in rng.integers(1, 5, size=int(rng.integers(1, 4)))) + (k,)
            bshape = tuple(1 if rng.random() < 0.4 else d for d in shape)
            qs = primes(bits, 8, k)
            a = values(rng, shape, qs, dt, "signed")
            b = values(rng, bshape, qs, dt, "signed")
            p = np.asarray(qs, dt)
            for op, f in (("modmul", O.modmul), ("modsum", O.modsum)):
                ctx = f"seed={seed} {np.dtype(dt).name} {shape} x {bshape}"
                same(op + "_ttt", f(a, b, p, out_shape=shape), R.modop(op, "ttt", a, b, p, shape), ctx)
                bs = int(rng.integers(-(1 << 20), 1 << 20))
                ps = int(qs[0])
                same(op + "_ttc", f(a, b, ps, out_shape=shape), R.modop(op, "ttc", a, b, ps, shape), ctx)
                same(op + "_tct", f(a, bs, p, out_shape=shape), R.modop(op, "tct", a, bs, p, shape), ctx)
                same(op + "_tcc", f(a, bs, ps, out_shape=shape), R.modop(op, "tcc", a, bs, ps, shape), ctx)
        # ---- axis_modsum
        for dt, bits in ((np.int64, 50), (np.int32, 30)):
            nd = int(rng.integers(2, 5))
            k = int(rng.integers(1, 4))
            shape = tuple(int(d) for d in rng.integers(1, 6, size=nd - 1)) + (k,)
            qs = primes(bits, 8, k)
            a = values(rng, shape, qs, dt, "signed")
            p = np.asarray(qs, dt)
            for axis in range(nd - 1):
                same("axis_modsum", O.axis_modsum(a, p, axis, exact=False), R.axis_modsum(a, p, axis),
                     f"seed={seed} {np.dtype(dt).name} {shape} axis={axis}")
        # ---- g_decomposition
        for dt, top in ((np.int64, 62), (np.int32, 30)):
            shape = tuple(int(d) for d in rng.integers(1, 5, size=int(rng.integers(1, 4))))
            a = rng.integers(-(1 << top), 1 << top, size=shape, dtype=np.int64).astype(dt)
            bits = int(rng.integers(1, 20))
            power = int(rng.integers(1, 6))
            d, _ = O.g_decomposition(a, power, bits)
            same("g_decomposition", d, R.g_decomposition(a, power, bits),
                 f"seed={seed} {np.dtype(dt).name} {shape} power={power} bits={bits}")
        # ---- permute
        for dt in (np.int64, np.int32):
            nd = int(rng.integers(2, 5))
            shape = tuple(int(d) for d in rng.integers(1, 6, size=nd))
            ew, pa = (int(x) for x in rng.choice(nd, size=2, replace=False))
            perms = rng.integers(0, shape[pa], size=(shape[ew], shape[pa])).astype(dt)
            a = rng.integers(-(1 << 30), 1 << 30, size=shape, dtype=np.int64).astype(dt)
            same("permute", O.permute(a, perms, ew, pa), R.permute(a, perms, ew, pa),
                 f"seed={seed} {np.dtype(dt).name} {shape} ew={ew} pa={pa}")
    view_sequences(np.random.default_rng(7), R, same, 40 * seeds)
    total = sum(counts.values())
    print(f"crosscheck: {total} cases bit-exact against the reference ({seeds} seeds; " +
          ", ".join(f"{k} {v}" for k, v in sorted(counts.items())) + ")")
    return 0


if __name__ == "__main__":
    sys.exit(run(int(sys.argv[1]) if len(sys.argv) > 1 else 24))
