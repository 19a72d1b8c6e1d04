"""HEAL's own C++ test suite, unmodified, builds against this backend.

HEAL's ten GoogleTest files are compiled against HEAL's include/ headers,
with tests/native/gtest/gtest.h in place of GoogleTest, and linked to
libheal_hw.so and libheal_gb300.so. The check is that every HEAL symbol the
suite imports (lattica_hw_api templates, DeviceTensor methods) is defined by
libheal_hw.so under HEAL's mangled name. The binaries need a GPU to run
(tests/native/heal_suite.py runs them); the same cases run on the GPU through
the Python mirror in test_gpu_reference_suite.py. Skipped where HEAL's
sources are not present."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests", "native"))
import heal_suite  # noqa: E402

from oracle import reference  # noqa: E402

HEAL_DIR = reference.path() or ""


def _symbols(path, undefined):
    flag = "--undefined-only" if undefined else "--defined-only"
    out = subprocess.run(["nm", "-D", flag, path], capture_output=True, text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def _heal(sym):
    return sym.startswith("_ZN14lattica_hw_api") or sym.startswith("_ZN12DeviceTensor") or \
        sym.startswith("_ZNK12DeviceTensor")


@pytest.mark.skipif(not HEAL_DIR or not os.path.isdir(os.path.join(HEAL_DIR, "tests")), reason="HEAL's sources are not present")
def test_heal_test_suite_links_against_this_backend(tmp_path):
    exes = heal_suite.build(HEAL_DIR, str(tmp_path))
    assert len(exes) == 10, sorted(exes)
    provided = _symbols(os.path.join(ROOT, "heal_gb300", "libheal_hw.so"), undefined=False)
    imported = set()
    for exe in exes.values():
        imported |= {s for s in _symbols(exe, undefined=True) if _heal(s)}
    # the suite calls into every layer: memory, views, contiguous, modops, reductions, NTT, permute
    for name in ("allocate_on_hardware", "host_to_device", "device_to_host", "make_contiguous", "modmul_ttt",
                 "axis_modsum", "g_decomposition", "nttI", "inttI", "permute", "squeeze", "reshape", "print"):
        assert any(name in s for s in imported), name
    missing = sorted(imported - provided)
    assert not missing, missing


SHIM_CHECK = r'''
#include <stdexcept>
#include "gtest/gtest.h"
TEST(Shim, Passes) {
  ASSERT_TRUE(1 + 1 == 2) << "never printed";
  ASSERT_FALSE(1 == 2);
  ASSERT_EQ(std::string("a"), std::string("a"));
  EXPECT_THROW(throw std::invalid_argument("x"), std::invalid_argument);
  testing::internal::CaptureStderr();
  std::fprintf(stderr, "captured text");
  ASSERT_EQ(testing::internal::GetCapturedStderr(), std::string("captured text"));
}
TEST(Shim, AssertStops) {
  ASSERT_EQ(1, 2) << "streamed " << 42;
  std::printf("after a failed assert\n");
}
TEST(Shim, ExpectGoesOn) {
  EXPECT_THROW((void)0, std::invalid_argument);
  EXPECT_THROW(throw std::out_of_range("y"), std::invalid_argument);
  std::printf("after two failed expects\n");
}
TEST(Shim, UnbracedIf) {
  if (true) ASSERT_TRUE(true); else std::printf("wrong branch\n");
}
'''


def test_gtest_shim_reports_failures(tmp_path):
    src = tmp_path / "shim_check.cpp"
    src.write_text(SHIM_CHECK)
    exe = str(tmp_path / "shim_check")
    native = os.path.join(ROOT, "tests", "native")
    subprocess.run(["g++", "-std=c++17", "-I", native, str(src), os.path.join(native, "gtest_main.cpp"), "-o", exe],
                   check=True)
    p = subprocess.run([exe], capture_output=True, text=True)
    assert p.returncode == 1
    out, err = p.stdout, p.stderr
    assert "[       OK ] Shim.Passes" in out and "[       OK ] Shim.UnbracedIf" in out
    assert "[  FAILED  ] Shim.AssertStops" in out and "[  FAILED  ] Shim.ExpectGoesOn" in out
    assert "after a failed assert" not in out and "after two failed expects" in out
    assert "wrong branch" not in out
    assert "streamed 42" in err and "did not throw" in err and "threw another type" in err
    assert "4 tests, 2 failed" in out
