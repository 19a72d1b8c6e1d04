"""Helpers of the GPU tests: upload / call / download through the C ABI."""
import numpy as np
import pytest

import heal_gb300
from heal_gb300 import capi


def ready():
    heal_gb300.build()
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a CUDA GPU is required for tests marked gpu")
    capi.check(capi.lib().heal_init(0))
    return capi


def up(x):
    return capi.DeviceArray.from_numpy(np.asarray(x))


# position of `result` in the C-ABI signatures that do not take it last
OUT_POS = {"heal_g_decomposition": 1, "heal_axis_modsum": 2, "heal_permute": 2}


def run(name, *args, out_shape=None, dtype=None, out=None):
    """Calls C-ABI `name`; numpy arguments are uploaded first.  The output
    (a fresh zeroed device array unless `out` is given) is returned as numpy."""
    dev = [up(a) if isinstance(a, np.ndarray) else a for a in args]
    if out is None:
        out = capi.DeviceArray.empty(out_shape, dtype)
    dev.insert(OUT_POS.get(name, len(dev)), out)
    capi.call(name, *dev)
    return out.numpy()


def ntt(a, p, perm, tw):
    return run("heal_ntt", a, p, perm, tw, None, None, out_shape=a.shape, dtype=a.dtype)


def intt(a, p, perm, itw, minv, prior=None):
    out = up(prior) if prior is not None else capi.DeviceArray.empty(a.shape, a.dtype)
    return run("heal_intt", a, p, perm, itw, minv, None, None, out=out)
