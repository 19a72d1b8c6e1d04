"""GB300Dispatcher: the backend behind HEAL's DeviceDispatcher
(python_execution/lattica_heal_runtime/device_interface.py:3-114), on this
repository's lattica_hw module.

HEAL's own PythonToCppDispatcher (py_wrapper.py:112-180) wires memory, views,
modmul/modsum, axis_modsum and ntt only.  This one answers every op the
DeviceDispatcher routes.  Argument order follows PythonToCppDispatcher where
it defines the op (host_to_device(tensor, dtype), axis_modsum(a, axis,
q_list, out), _modmul_ttt(a, b, p, out), expand(a, repeat, axis), ntt(a,
perm, perm_pairs, q_list, log2p, mu_list, psi_arr, out, tile, skip_perm));
the others are:

  zeros(shape, dtype)
  intt(a, perm, perm_pairs, q_list, log2p, mu_list, psi_inv_arr, m_inv, out, tile, skip_perm)
  _mod_tt(a, b, out) / _mod_tc(a, b, out) / _mod_ct(a, b, out)
  _modneg_tt(a, p, out) / _modneg_tc(a, p, out)
  apply_g_decomp(a, power, base_bits, out)            HEAL g_decomposition
  take_along_axis(a, perms, elementwise_axis, perm_axis, out)   HEAL permute
  modmul_axis_sum(a, b, p, axis, out, perms=None, perm_axis=0)
  modmul_axis_sum_permute(a, b, p, axis, perms, elementwise_axis, perm_axis, out)   (extension)
  g_decomposition_ntt(a, power, base_bits, p, perm, twiddles, out)                 (extension)
  moveaxis(a, source, destination)                    a new view
  get_slice(a, *index)                                ints, slices (step > 0), Ellipsis; a new view
  new_reference(a)                                    a new view of the same tensor
  flatten(a, start_dim=0, end_dim=-1)

Ops that compute return their `out`.  As in HEAL, reshape / expand /
squeeze / unsqueeze change the tensor they are given.  abs, set_const_val
and pad_single_axis have no definition in HEAL and raise NotImplementedError.
"""
from __future__ import annotations

import numpy as np


class GB300Dispatcher:
    def __init__(self, lattica_hw=None):
        if lattica_hw is None:
            import heal_gb300
            heal_gb300.build()
            lattica_hw = heal_gb300.lattica_hw()
        self.m = lattica_hw
        import torch
        self.torch = torch
        self._sfx_of_dtype = {torch.int32: "32", torch.int64: "64", torch.float64: "float64"}
        self._sfx_of_type = {lattica_hw.DeviceTensor32: "32", lattica_hw.DeviceTensor64: "64",
                             lattica_hw.DeviceTensorfloat64: "float64"}

    # ---- helpers
    def _f(self, name, t):
        sfx = self._sfx_of_type.get(type(t))
        if sfx is None:
            raise TypeError(f"Unsupported tensor type: {type(t)}")
        return getattr(self.m, f"{name}_{sfx}")

    def _fd(self, name, dtype):
        sfx = self._sfx_of_dtype.get(dtype)
        if sfx is None:
            raise TypeError(f"Unsupported dtype: {dtype}")
        return getattr(self.m, f"{name}_{sfx}")

    # ---- memory and I/O
    def empty(self, shape, dtype):
        return self._fd("allocate_on_hardware", dtype)(list(shape))

    def zeros(self, shape, dtype):
        return self._fd("allocate_on_hardware", dtype)(list(shape))   # HEAL's allocation is zeroed

    def host_to_device(self, tensor, dtype):
        t = tensor if isinstance(tensor, self.torch.Tensor) else self.torch.as_tensor(np.asarray(tensor))
        return self._fd("host_to_device", dtype)(t.to(dtype))

    def device_to_host(self, a):
        return self._f("device_to_host", a)(a)

    # ---- modular arithmetic
    def _modop(self, name, a, b, p, out):
        self._f(name, a)(a, b, p, out)
        return out

    def _modmul_ttt(self, a, b, p, out): return self._modop("modmul_ttt", a, b, p, out)
    def _modmul_ttc(self, a, b, p, out): return self._modop("modmul_ttc", a, b, p, out)
    def _modmul_tct(self, a, b, p, out): return self._modop("modmul_tct", a, b, p, out)
    def _modmul_tcc(self, a, b, p, out): return self._modop("modmul_tcc", a, b, p, out)
    def _modsum_ttt(self, a, b, p, out): return self._modop("modsum_ttt", a, b, p, out)
    def _modsum_ttc(self, a, b, p, out): return self._modop("modsum_ttc", a, b, p, out)
    def _modsum_tct(self, a, b, p, out): return self._modop("modsum_tct", a, b, p, out)
    def _modsum_tcc(self, a, b, p, out): return self._modop("modsum_tcc", a, b, p, out)

    def _mod_tt(self, a, b, out):
        self._f("mod_tt", a)(a, b, out)
        return out

    def _mod_tc(self, a, b, out):
        self._f("mod_tc", a)(a, b, out)
        return out

    def _mod_ct(self, a, b, out):
        self._f("mod_ct", b)(a, b, out)
        return out

    def _modneg_tt(self, a, p, out):
        self._f("modneg_tt", a)(a, p, out)
        return out

    def _modneg_tc(self, a, p, out):
        self._f("modneg_tc", a)(a, p, out)
        return out

    def axis_modsum(self, a, axis, q_list, out):
        self._f("axis_modsum", a)(a, q_list, out, axis)
        return out

    def modmul_axis_sum(self, a, b, p, axis, out, perms=None, perm_axis=0):
        self._f("modmul_axis_sum", a)(a, b, p, perms, perm_axis, out, axis)
        return out

    def g_decomposition_ntt(self, a, power, base_bits, p, perm, twiddles, out):
        """ntt(reshape(g_decomposition(a, power, base_bits), [l, m, r, k * power]),
        p, perm, twiddles) in one call (an extension op of this backend)."""
        self._f("g_decomposition_ntt", a)(a, power, base_bits, p, perm, twiddles, out)
        return out

    def modmul_axis_sum_permute(self, a, b, p, axis, perms, elementwise_axis, perm_axis, out):
        """permute(axis_modsum(modmul(a, b, p), axis), perms, elementwise_axis,
        perm_axis) in one call (an extension op of this backend)."""
        self._f("modmul_axis_sum_permute", a)(a, b, p, axis, perms, elementwise_axis, perm_axis, out)
        return out

    def apply_g_decomp(self, a, power, base_bits, out):
        self._f("g_decomposition", a)(a, out, power, base_bits)
        return out

    def take_along_axis(self, a, perms, elementwise_axis, perm_axis, out):
        self._f("permute", a)(a, perms, out, elementwise_axis, perm_axis)
        return out

    def ntt(self, a, perm, perm_pairs, q_list, log2p, mu_list, psi_arr, out, tile, skip_perm):
        if skip_perm:
            raise NotImplementedError(f"skip_perm is not supported. {skip_perm=}")
        if tile:
            a = self.expand(a, 2, -1)
        self._f("ntt", a)(a, q_list, perm, psi_arr, log2p, mu_list, out)
        return out

    def intt(self, a, perm, perm_pairs, q_list, log2p, mu_list, psi_inv_arr, m_inv, out, tile, skip_perm):
        if skip_perm:
            raise NotImplementedError(f"skip_perm is not supported. {skip_perm=}")
        if tile:
            a = self.expand(a, 2, -1)
        self._f("intt", a)(a, q_list, perm, psi_inv_arr, m_inv, log2p, mu_list, out)
        return out

    # ---- views
    def reshape(self, a, new_shape):
        a.reshape(list(new_shape))
        return a

    def expand(self, a, repeat, axis):
        return self._f("expand", a)(a, axis, repeat)

    def squeeze(self, a, axis):
        return self._f("squeeze", a)(a, axis)

    def unsqueeze(self, a, axis):
        return self._f("unsqueeze", a)(a, axis)

    def contiguous(self, a):
        return self._f("make_contiguous", a)(a)

    def new_reference(self, a):
        return self._f("view", a)(a)

    def moveaxis(self, a, source, destination):
        v = self.new_reference(a)
        return self._f("moveaxis", v)(v, source, destination)

    def get_slice(self, a, *index):
        if len(index) == 1 and isinstance(index[0], (tuple, list)):
            index = tuple(index[0])
        nd = len(a.dims)
        n_ell = sum(1 for i in index if i is Ellipsis)
        if n_ell > 1:
            raise IndexError("an index can only have a single ellipsis")
        if n_ell:
            k = index.index(Ellipsis)
            index = index[:k] + (slice(None),) * (nd - len(index) + 1) + index[k + 1:]
        if len(index) > nd:
            raise IndexError("too many indices")
        v = self.new_reference(a)
        drop = []
        for axis, ix in enumerate(index):
            n = v.dims[axis]
            if isinstance(ix, slice):
                start, stop, step = ix.indices(n)
                if step <= 0:
                    raise ValueError("slice step must be positive")
                v = self._f("get_slice", v)(v, axis, start, max(stop, start), step)
            else:
                i = int(ix)
                i = i + n if i < 0 else i
                if not 0 <= i < n:
                    raise IndexError(f"index {ix} out of range for axis {axis} of size {n}")
                v = self._f("get_slice", v)(v, axis, i, i + 1, 1)
                drop.append(axis)
        for axis in reversed(drop):
            v = self.squeeze(v, axis)
        return v

    def flatten(self, a, start_dim=0, end_dim=-1):
        dims = list(a.dims)
        nd = len(dims)
        s, e = start_dim % nd if nd else 0, end_dim % nd if nd else 0
        new = dims[:s] + [int(np.prod(dims[s:e + 1]))] + dims[e + 1:]
        a = self.contiguous(a)
        a.reshape(new)
        return a

    # ---- named by DeviceDispatcher, defined nowhere in HEAL
    def abs(self, *args, **kwargs):
        raise NotImplementedError("abs: HEAL defines no semantics for this op")

    def set_const_val(self, *args, **kwargs):
        raise NotImplementedError("set_const_val: HEAL defines no semantics for this op")

    def pad_single_axis(self, *args, **kwargs):
        raise NotImplementedError("pad_single_axis: HEAL defines no semantics for this op")

    def synchronize(self):
        self.m.synchronize()
