"""Builds HEAL's own C++ test suite (tests/test_*.cpp of a HEAL checkout,
unmodified) against this backend, and runs it where a GPU is present.

Each file is compiled against HEAL's include/ headers and libtorch, with
tests/native/gtest/gtest.h standing in for GoogleTest (HEAL's CMake fetches
GoogleTest from the network). It is then linked to libheal_hw.so (HEAL's C++
API) and libheal_gb300.so. A link that succeeds shows that every
lattica_hw_api template and DeviceTensor method the suite calls is exported
under HEAL's mangled name.

    python tests/native/heal_suite.py HEAL_DIR [OUT_DIR]   # build, then run each binary
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def sources(heal_dir: str) -> list[str]:
    """HEAL's test files (tests/CMakeLists.txt builds one executable from each)."""
    return sorted(glob.glob(os.path.join(heal_dir, "tests", "test_*.cpp")))


def build(heal_dir: str, out_dir: str) -> dict[str, str]:
    """Compiles and links every test file; returns {source: executable}.
    Raises CalledProcessError (with the compiler's output) on the first failure."""
    import heal_gb300
    from heal_gb300 import native
    heal_gb300.build()
    inc, tlib, abi = native._torch_paths()
    os.makedirs(out_dir, exist_ok=True)
    cxx = ["g++", "-std=c++17", "-O1", f"-D_GLIBCXX_USE_CXX11_ABI={abi}", "-I", HERE,
           "-I", os.path.join(heal_dir, "include")] + sum((["-I", p] for p in inc), [])
    main_obj = os.path.join(out_dir, "gtest_main.o")
    jobs = [(os.path.join(HERE, "gtest_main.cpp"), main_obj)]
    srcs = sources(heal_dir)
    jobs += [(s, os.path.join(out_dir, os.path.basename(s)[:-4] + ".o")) for s in srcs]

    def run(cmd):
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode:
            raise subprocess.CalledProcessError(p.returncode, cmd, p.stdout, p.stderr)

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(run, cxx + ["-c", s, "-o", o]) for s, o in jobs]:
            f.result()
    lib_dir = os.path.join(ROOT, "heal_gb300")
    exes = {}
    for s, o in jobs[1:]:
        exe = o[:-2]
        run(["g++", "-o", exe, o, main_obj, "-L", lib_dir, "-lheal_hw", "-lheal_gb300", "-L", tlib, "-lc10",
             "-ltorch_cpu", "-ltorch", f"-Wl,-rpath,{lib_dir}", f"-Wl,-rpath,{tlib}"])
        exes[s] = exe
    return exes


def main(argv: list[str]) -> int:
    if len(argv) < 2:
        print(__doc__)
        return 2
    heal_dir = argv[1]
    out_dir = argv[2] if len(argv) > 2 else os.path.join(ROOT, "heal_gb300", "_build", "heal_suite")
    failed = 0
    for src, exe in build(heal_dir, out_dir).items():
        rc = subprocess.run([exe]).returncode
        print(f"{os.path.basename(src)}: {'passed' if rc == 0 else 'FAILED'}")
        failed += rc != 0
    return 1 if failed else 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
