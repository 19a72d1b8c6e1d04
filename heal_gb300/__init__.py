"""GB300-native vendor backend for HEAL (Lattica's Homomorphic Encryption
Abstraction Layer).

Layers, bottom up:
  include/heal_gb300.h + libheal_gb300.so   C ABI over the sm_103a kernels
  libheal_hw.so                             HEAL's lattica_hw_api C++ templates
  lattica_hw (Python module)                HEAL's pybind module names
  heal_gb300.capi                           ctypes binding of the C ABI
  heal_gb300.runtime                        GPU dispatcher for HEAL transcripts

There is no CPU fallback: importing `lattica_hw` or `capi.lib()` without the
built extension raises ImportError.
"""
import importlib.util
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def build(verbose: bool = False, force: bool = False) -> dict:
    """Compiles the CUDA backend and its C++ / Python bindings in place."""
    from . import native as _b
    return _b.build(verbose=verbose, force=force)


def lattica_hw():
    """The `lattica_hw` module (HEAL's pybind surface) backed by this GPU
    backend, registered in sys.modules under that name."""
    mod = sys.modules.get("lattica_hw")
    if mod is not None and getattr(mod, "__file__", "").startswith(HERE):
        return mod
    import torch  # noqa: F401  (the module links against torch's Python bindings)
    from . import native as _b
    if not os.path.exists(_b.EXT):
        raise ImportError(f"{_b.EXT} is missing: build the backend first (heal_gb300.build())")
    spec = importlib.util.spec_from_file_location("lattica_hw", _b.EXT)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    sys.modules["lattica_hw"] = mod
    return mod
