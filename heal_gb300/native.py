"""In-tree build of the GB300 backend (no CMake).

Produces, next to this file:
  libheal_gb300.so   CUDA kernels + the C ABI (include/heal_gb300.h); nvcc,
                     sm_103a only, static CUDA runtime, no torch dependency
  libheal_hw.so      HEAL's lattica_hw_api C++ templates over the C ABI
  lattica_hw<ext>    the `lattica_hw` Python module (pybind11 from torch)
Objects go to heal_gb300/_build/.  Every step is skipped when its outputs are
newer than its inputs, and independent compilations run in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

LIB_CUDA = os.path.join(HERE, "libheal_gb300.so")
LIB_API = os.path.join(HERE, "libheal_hw.so")
EXT = os.path.join(HERE, "lattica_hw" + sysconfig.get_config_var("EXT_SUFFIX"))


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the backend")


def _mtime(paths) -> float:
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def _stale(out: str, deps) -> bool:
    return not os.path.exists(out) or os.path.getmtime(out) < _mtime(deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def _torch_paths():
    import torch
    tdir = os.path.dirname(torch.__file__)
    inc = [os.path.join(tdir, "include"), os.path.join(tdir, "include", "torch", "csrc", "api", "include")]
    abi = int(torch._C._GLIBCXX_USE_CXX11_ABI)
    return inc, os.path.join(tdir, "lib"), abi


def build(verbose: bool = False, force: bool = False) -> dict:
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    headers = (glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
               + glob.glob(os.path.join(ROOT, "include", "*.h")))
    api_headers = headers + glob.glob(os.path.join(CSRC, "lattica", "*.h"))
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    tinc, tlib, abi = _torch_paths()
    pyinc = sysconfig.get_paths()["include"]
    cxx = ["g++", "-std=c++17", "-O2", "-fPIC", f"-D_GLIBCXX_USE_CXX11_ABI={abi}"]
    cxx += sum((["-I", p] for p in tinc), [])

    jobs = []
    cu_objs = []
    for src in cu:
        obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
        cu_objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         *os.environ.get("HEAL_NVCC_EXTRA", "").split(), "-c", src, "-o", obj])
    api_src = os.path.join(CSRC, "lattica", "lattica_api.cpp")
    api_obj = os.path.join(OBJ, "lattica_api.o")
    if force or _stale(api_obj, [api_src] + api_headers):
        jobs.append(cxx + ["-c", api_src, "-o", api_obj])
    py_src = os.path.join(CSRC, "lattica", "py_bindings.cpp")
    py_obj = os.path.join(OBJ, "py_bindings.o")
    if force or _stale(py_obj, [py_src] + api_headers):
        jobs.append(cxx + ["-I", pyinc, "-c", py_src, "-o", py_obj])

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, j, verbose) for j in jobs]:
            f.result()

    if force or _stale(LIB_CUDA, cu_objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB_CUDA + ".tmp", *cu_objs], verbose)
        os.replace(LIB_CUDA + ".tmp", LIB_CUDA)
    if force or _stale(LIB_API, [api_obj, LIB_CUDA]):
        _run(["g++", "-shared", "-o", LIB_API + ".tmp", api_obj, "-L", HERE, "-lheal_gb300", "-L", tlib,
              "-lc10", "-ltorch_cpu", "-Wl,-rpath,$ORIGIN", f"-Wl,-rpath,{tlib}"], verbose)
        os.replace(LIB_API + ".tmp", LIB_API)
    if force or _stale(EXT, [py_obj, LIB_API]):
        _run(["g++", "-shared", "-o", EXT + ".tmp", py_obj, "-L", HERE, "-lheal_hw", "-lheal_gb300", "-L", tlib,
              "-lc10", "-ltorch_cpu", "-ltorch", "-ltorch_python", "-Wl,-rpath,$ORIGIN", f"-Wl,-rpath,{tlib}"],
             verbose)
        os.replace(EXT + ".tmp", EXT)
    return {"libheal_gb300": LIB_CUDA, "libheal_hw": LIB_API, "lattica_hw": EXT}


if __name__ == "__main__":
    import sys
    print(build(verbose=True, force="--force" in sys.argv))
