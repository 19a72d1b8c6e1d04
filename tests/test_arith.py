"""The modular-arithmetic routines of heal_gb300/csrc/heal_arith.h (shared by
the CUDA kernels) compiled for the host and checked against Python integers
on random and boundary operands.  No GPU needed."""
import os
import random
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("arith") / "arith_check")
    subprocess.run(["g++", "-std=c++17", "-O2", os.path.join(HERE, "native", "arith_check.cpp"), "-o", exe],
                   check=True)
    return exe


def run(exe, rows):
    inp = "".join(f"{op} {a} {b} {q}\n" for op, a, b, q in rows)
    out = subprocess.run([exe], input=inp, capture_output=True, text=True, check=True).stdout.split()
    return [int(x) for x in out]


def moduli(bits_lo, bits_hi, rng, n):
    qs = [2 ** bits_lo + 1, 2 ** bits_hi - 1, 3, 2 ** (bits_hi - 1), 2 ** (bits_hi - 1) + 1]
    qs += [rng.randrange(2, 2 ** rng.randint(bits_lo, bits_hi)) for _ in range(n)]
    return [q for q in qs if q >= 2]


def test_mg64(harness):
    rng = random.Random(1)
    rows, want = [], []
    for q in moduli(2, 63, rng, 400):
        for _ in range(8):
            a = rng.choice([0, 1, q - 1, rng.randrange(q), rng.randrange(2 ** 63)])
            b = rng.choice([0, q - 1, rng.randrange(q), rng.randrange(2 ** 63)])
            rows.append(("mul64", a, b, q))
            want.append(a * b % q)
            x1, x0 = rng.randrange(2 ** 64), rng.randrange(2 ** 64)
            x1 = rng.choice([x1, x1 % q, 0, 2 ** 64 - 1])
            rows.append(("mod128", x1, x0, q))
            want.append(((x1 << 64) | x0) % q)
    assert run(harness, rows) == want


def test_mg32(harness):
    rng = random.Random(2)
    rows, want = [], []
    for q in moduli(2, 31, rng, 400):
        for _ in range(8):
            x1, x0 = rng.randrange(2 ** 32), rng.randrange(2 ** 32)
            x1 = rng.choice([x1, x1 % q, 0, 2 ** 32 - 1])
            rows.append(("mod32", x1, x0, q))
            want.append(((x1 << 32) | x0) % q)
    assert run(harness, rows) == want


def test_shoup(harness):
    rng = random.Random(3)
    rows, want = [], []
    for q in moduli(2, 62, rng, 300):
        for _ in range(6):
            w = rng.randrange(q)
            y = rng.choice([rng.randrange(2 ** 64), rng.randrange(q), 2 ** 64 - 1, 0])
            rows.append(("shoup64", y, w, q))
            want.append(y * w % q)
    for q in moduli(2, 31, rng, 300):
        for _ in range(6):
            w = rng.randrange(q)
            y = rng.choice([rng.randrange(2 ** 32), rng.randrange(q), 2 ** 32 - 1])
            rows.append(("shoup32", y, w, q))
            want.append(y * w % q)
    assert run(harness, rows) == want


def test_fastdiv(harness):
    rng = random.Random(4)
    rows, want = [], []
    ds = [1, 2, 3, 5, 7, 24, 72, 2 ** 31, 2 ** 31 + 1, 2 ** 32 - 1] + [rng.randrange(1, 2 ** 32) for _ in range(300)]
    for d in ds:
        for n in [0, 1, d - 1, d, d + 1, 2 ** 32 - 1, 2 ** 31] + [rng.randrange(2 ** 32) for _ in range(10)]:
            n &= 0xFFFFFFFF
            rows.append(("fastdiv", n, 0, d))
            want.append(n // d)
    assert run(harness, rows) == want


def test_view_coalescing(tmp_path):
    """heal_view.h: merged views address every element exactly as the
    original views do (64-bit and FastDiv decomposition), kept axes keep
    their coordinates."""
    exe = str(tmp_path / "view_check")
    subprocess.run(["g++", "-std=c++17", "-O2", os.path.join(HERE, "native", "view_check.cpp"), "-o", exe],
                   check=True)
    out = subprocess.run([exe], capture_output=True, text=True).stdout.strip()
    assert out == "ok 20000", out
