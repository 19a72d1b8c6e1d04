"""The reference's GoogleTest suite (tests/test_*.cpp of HEAL), case for case,
run against this backend through the `lattica_hw` module with torch tensors,
as HEAL's Python runtime drives it."""
import numpy as np
import pytest
import torch

import heal_gb300
from _gpu import ready

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def hw():
    ready()
    return heal_gb300.lattica_hw()


def i32(x):
    return torch.tensor(x, dtype=torch.int32)


def i64(x):
    return torch.tensor(x, dtype=torch.int64)


# ---- tests/test_ntt.cpp
def test_ntt_round_trip(hw):
    a = i32([[[[1, 2]], [[3, 4]], [[5, 6]], [[7, 8]]]])
    H = hw.host_to_device_32
    p, minv, perm = H(i32([17, 257])), H(i32([13, 193])), H(i32([0, 2, 1, 3]))
    tw = H(i32([[1, 4, 2, 8], [1, 16, 4, 64]]))
    itw = H(i32([[1, 13, 9, 15], [1, 241, 193, 253]]))
    res, back = hw.allocate_on_hardware_32([1, 4, 1, 2]), hw.allocate_on_hardware_32([1, 4, 1, 2])
    hw.ntt_32(H(a), p, perm, tw, None, None, res)
    hw.intt_32(res, p, perm, itw, minv, None, None, back)
    assert torch.equal(hw.device_to_host_32(back), a)
    assert hw.device_to_host_32(res).flatten().tolist() == [15, 112, 2, 194, 10, 84, 11, 132]


# ---- tests/test_modop.cpp
def _ttt(hw, fn, a, b, p, shape):
    r = hw.allocate_on_hardware_32(shape)
    fn(hw.host_to_device_32(a), hw.host_to_device_32(b), hw.host_to_device_32(p), r)
    return hw.device_to_host_32(r)


def test_modop_scalar_variants(hw):
    a = i32([[1, 2], [3, 4]])
    H = hw.host_to_device_32
    for fn, op in [(hw.modsum_tcc_32, lambda x, y, p: (x + y) % p), (hw.modmul_tcc_32, lambda x, y, p: (x * y) % p)]:
        r = hw.allocate_on_hardware_32([2, 2])
        fn(H(a), 5, 6, r)
        assert torch.equal(hw.device_to_host_32(r), op(a, 5, 6))
    p = i32([6, 7])
    for fn, op in [(hw.modsum_tct_32, lambda x, y, p: (x + y) % p), (hw.modmul_tct_32, lambda x, y, p: (x * y) % p)]:
        r = hw.allocate_on_hardware_32([2, 2])
        fn(H(a), 5, H(p), r)
        assert torch.equal(hw.device_to_host_32(r), op(a, 5, p))
    b = i32([[5, 6], [7, 8]])
    for fn, op in [(hw.modsum_ttc_32, lambda x, y, p: (x + y) % p), (hw.modmul_ttc_32, lambda x, y, p: (x * y) % p)]:
        r = hw.allocate_on_hardware_32([2, 2])
        fn(H(a), H(b), 9, r)
        assert torch.equal(hw.device_to_host_32(r), op(a, b, 9))
    r = hw.allocate_on_hardware_32([1, 2])
    hw.modsum_tct_32(H(i32([[10, 20]])), 3, H(i32([4, 5])), r)
    assert hw.device_to_host_32(r).tolist() == [[1, 3]]


def test_modop_broadcast(hw):
    g = torch.Generator().manual_seed(0)
    a = torch.randint(1, 100, (2, 3, 4), generator=g, dtype=torch.int32)
    b = torch.randint(1, 100, (1, 3, 4), generator=g, dtype=torch.int32)
    p = torch.randint(100, 200, (4,), generator=g, dtype=torch.int32)
    assert torch.equal(_ttt(hw, hw.modsum_ttt_32, a, b, p, [2, 3, 4]), (a + b) % p)
    r = _ttt(hw, hw.modmul_ttt_32, i32([[1], [2]]), i32([10, 20, 30]), i32([11, 17, 23]), [2, 3])
    assert torch.equal(r, (i32([[1], [2]]) * i32([10, 20, 30])) % i32([11, 17, 23]))
    with pytest.raises(ValueError):
        _ttt(hw, hw.modsum_ttt_32, torch.zeros(2, 3, dtype=torch.int32), torch.zeros(2, 4, dtype=torch.int32),
             i32([101, 102, 103]), [2, 3])
    with pytest.raises(ValueError):
        _ttt(hw, hw.modsum_ttt_32, torch.zeros(2, 3, dtype=torch.int32), torch.zeros(2, 3, dtype=torch.int32),
             torch.full((4, 1), 150, dtype=torch.int32), [2, 3])


def test_mod_variants(hw):
    a, b = i64([[5, 7, 9], [10, 12, 14]]), i64([[3, 5, 7], [4, 6, 8]])
    H = hw.host_to_device_64
    r = hw.allocate_on_hardware_64([2, 3])
    hw.mod_tt_64(H(a), H(b), r)
    assert torch.equal(hw.device_to_host_64(r), torch.remainder(a, b))
    hw.mod_tc_64(H(a), 6, r)
    assert torch.equal(hw.device_to_host_64(r), torch.remainder(a, 6))
    hw.mod_ct_64(6, H(b), r)
    assert torch.equal(hw.device_to_host_64(r), torch.remainder(torch.full((2, 3), 6), b))
    base = torch.arange(1, 25, dtype=torch.int64).reshape(2, 3, 4)
    at, bt = base.transpose(0, 2), (base + 24).permute(2, 1, 0)
    r = hw.allocate_on_hardware_64([4, 3, 2])
    hw.mod_tt_64(H(at), H(bt), r)
    assert torch.equal(hw.device_to_host_64(r), torch.remainder(at, bt))
    x = torch.randint(1, 100, (2, 2, 2, 2), dtype=torch.int32)
    y = torch.randint(1, 100, (2, 2, 2, 2), dtype=torch.int32)
    r32 = hw.allocate_on_hardware_32([2, 2, 2, 2])
    hw.mod_tt_32(hw.host_to_device_32(x), hw.host_to_device_32(y), r32)
    assert torch.equal(hw.device_to_host_32(r32), torch.remainder(x, y))
    with pytest.raises(ValueError):
        hw.mod_tt_64(None, H(b), r)
    with pytest.raises(ValueError):
        hw.mod_tt_64(H(a), H(i64([[1, 2], [3, 4]])), r)
    with pytest.raises(ValueError):
        hw.mod_tc_64(H(a), 5, hw.allocate_on_hardware_64([3, 2]))


# ---- tests/test_axis_modsum.cpp
def test_axis_modsum(hw):
    H = hw.host_to_device_32
    a = torch.arange(1, 25, dtype=torch.int32).reshape(2, 3, 4)
    p = i32([11, 13, 17, 19])
    r = hw.allocate_on_hardware_32([2, 4])
    hw.axis_modsum_32(H(a), H(p), r, 1)
    assert torch.equal(hw.device_to_host_32(r), a.sum(1) % p)
    a = i32([[1, 2, 3, 4], [4, 5, 6, 7], [7, 8, 9, 10]])
    p = i32([5, 7, 11, 13])
    r = hw.allocate_on_hardware_32([4])
    hw.axis_modsum_32(H(a), H(p), r, 0)
    assert torch.equal(hw.device_to_host_32(r), a.sum(0) % p)
    a = torch.arange(24, dtype=torch.int32).reshape(2, 2, 2, 3)
    p = i32([7, 11, 13])
    r = hw.allocate_on_hardware_32([2, 2, 3])
    hw.axis_modsum_32(H(a), H(p), r, 2)
    assert torch.equal(hw.device_to_host_32(r), a.sum(2) % p)
    z = H(torch.zeros(2, 2, 2, dtype=torch.int32))
    r = hw.allocate_on_hardware_32([2, 2])
    for ax in (-1, 3):
        with pytest.raises(ValueError):
            hw.axis_modsum_32(z, H(i32([7, 11])), r, ax)
    with pytest.raises(ValueError):
        hw.axis_modsum_32(z, H(i32([7, 11, 13])), r, 2)


# ---- tests/test_g_decomposition.cpp and test_decomp_reconstruct.cpp
def test_g_decomposition(hw, capfd):
    H = hw.host_to_device_32
    r = hw.allocate_on_hardware_32([4, 2])
    hw.g_decomposition_32(H(i32([0, 1, 2, 3])), r, 2, 1)
    assert hw.device_to_host_32(r).tolist() == [[0, 0], [1, 0], [0, 1], [1, 1]]
    r = hw.allocate_on_hardware_32([5, 4])
    hw.g_decomposition_32(H(torch.zeros(5, dtype=torch.int32)), r, 4, 2)
    assert (hw.device_to_host_32(r) == 0).all()
    a = i32([[[5, 12], [3, 1]], [[8, 7], [9, 2]]])
    r = hw.allocate_on_hardware_32([2, 2, 2, 3])
    hw.g_decomposition_32(H(a), r, 3, 2)
    assert hw.device_to_host_32(r).tolist() == [[[[1, 1, 0], [0, 3, 0]], [[3, 0, 0], [1, 0, 0]]],
                                                [[[0, 2, 0], [3, 1, 0]], [[1, 2, 0], [2, 0, 0]]]]
    r = hw.allocate_on_hardware_32([1, 3])
    hw.g_decomposition_32(H(i32([255])), r, 3, 3)
    hw.synchronize()
    assert "exceeds" not in capfd.readouterr().err
    with pytest.raises(ValueError):
        hw.g_decomposition_32(H(i32([10, 20])), hw.allocate_on_hardware_32([3, 2]), 2, 2)
    # a residual beyond the capacity is reported (g_decomposition_impl.cpp:58-65)
    r = hw.allocate_on_hardware_32([1, 2])
    hw.g_decomposition_32(H(i32([255])), r, 2, 3)
    hw.synchronize()
    assert "exceeds capacity with base_bits=3 and power=2" in capfd.readouterr().err


def test_decomp_reconstruct(hw):
    H = hw.host_to_device_32
    a = i32([51, 29, 63])
    d = hw.allocate_on_hardware_32([3, 6])
    hw.g_decomposition_32(H(a), d, 6, 1)
    hw.modmul_ttt_32(d, H(i32([1, 2, 4, 8, 16, 32])), H(i32([1024] * 6)), d)   # in place
    d.reshape([3, 6, 1])
    r = hw.allocate_on_hardware_32([3, 1])
    hw.axis_modsum_32(d, H(i32([1024])), r, 1)
    r.reshape([3])
    assert torch.equal(hw.device_to_host_32(r), a)


# ---- tests/test_permute.cpp
def _perm_expected(a, perms, ew, pa):
    am = torch.movedim(a.clone(), (ew, pa), (-2, -1))
    shape = [1] * am.dim()
    shape[-2], shape[-1] = perms.size(0), perms.size(1)
    pe = perms.view(shape).expand_as(am).to(torch.long)
    return torch.movedim(torch.take_along_dim(am, pe, -1), (-2, -1), (ew, pa))


@pytest.mark.parametrize("shape,perms,ew,pa", [
    ((2, 3, 4, 5), [[2, 1, 0], [0, 2, 1]], 0, 1),
    ((2, 2, 2, 3, 5), [[1, 0, 2], [2, 1, 0]], 0, 3),
    ((3, 4, 5), [[3, 2, 1, 0], [0, 2, 3, 1], [1, 0, 3, 2]], 0, 1),
    ((5, 3, 7), [[2, 1, 0], [0, 2, 1], [1, 0, 2], [2, 0, 1], [0, 1, 2]], 0, 1),
    ((3, 4, 2), [[1, 2, 0, 3], [3, 0, 1, 2]], 2, 1),
])
def test_permute(hw, shape, perms, ew, pa):
    a = torch.randint(0, 100, shape, dtype=torch.int32)
    perms = i32(perms)
    r = hw.allocate_on_hardware_32(list(shape))
    hw.permute_32(hw.host_to_device_32(a), hw.host_to_device_32(perms), r, ew, pa)
    assert torch.equal(hw.device_to_host_32(r), _perm_expected(a, perms, ew, pa))


def test_permute_errors(hw):
    H = hw.host_to_device_32
    a = H(torch.zeros(2, 3, 4, dtype=torch.int32))
    r = hw.allocate_on_hardware_32([2, 3, 4])
    perms = H(torch.zeros(2, 3, dtype=torch.int32))
    for ew, pa in [(3, 1), (1, 1), (0, 3)]:
        with pytest.raises(ValueError):
            hw.permute_32(a, perms, r, ew, pa)
    with pytest.raises(IndexError):
        hw.permute_32(a, H(i32([[0, 1, 3], [1, 2, 0]])), r, 0, 1)


# ---- tests/test_noncontiguous.cpp, test_contiguous.cpp, test_reshape.cpp, test_memory_ops.cpp
def test_noncontiguous_modmul(hw, capfd):
    a = torch.arange(18, dtype=torch.int32).reshape(2, 3, 3, 1)
    at = a.transpose(1, 2)
    r = hw.allocate_on_hardware_32([2, 3, 3, 1])
    hw.modmul_ttt_32(hw.host_to_device_32(a), hw.host_to_device_32(at), hw.host_to_device_32(i32([100])), r)
    r.print()
    assert "Data: {{{{0}" in capfd.readouterr().out
    assert torch.equal(hw.device_to_host_32(r), (a * at).remainder(100))


def test_contiguous(hw):
    t = torch.arange(12, dtype=torch.int32).reshape(3, 4).transpose(0, 1)
    d = hw.host_to_device_32(t)
    assert d.strides == [1, 4]
    c = hw.make_contiguous_32(d)
    assert c.strides == [3, 1]
    assert torch.equal(hw.device_to_host_32(c), t)
    x = hw.host_to_device_64(torch.randint(0, 60000, (5, 6), dtype=torch.int64))
    assert hw.make_contiguous_64(x) is x


def test_reshape(hw):
    c = hw.host_to_device_32(i32([[[1, 2, 3], [4, 5, 6]], [[7, 8, 9], [10, 11, 12]]]))
    c.reshape([6, 2])
    assert hw.device_to_host_32(c).tolist() == [[1, 2], [3, 4], [5, 6], [7, 8], [9, 10], [11, 12]]
    c.reshape([3, 4])
    assert hw.device_to_host_32(c).tolist() == [[1, 2, 3, 4], [5, 6, 7, 8], [9, 10, 11, 12]]


def test_memory_ops(hw):
    x = i64([[[1, 2, 3]]])
    assert torch.equal(hw.device_to_host_64(hw.squeeze_64(hw.host_to_device_64(x), 1)), x.squeeze(1))
    with pytest.raises(ValueError):
        hw.squeeze_64(hw.host_to_device_64(i64([[1, 2, 3]])), 1)
    y = i32([[1, 2], [3, 4]])
    assert torch.equal(hw.device_to_host_32(hw.unsqueeze_32(hw.host_to_device_32(y), 1)), y.unsqueeze(1))
    assert torch.equal(hw.device_to_host_32(hw.unsqueeze_32(hw.host_to_device_32(y), -1)), y.unsqueeze(-1))
    z = hw.host_to_device_64(torch.randint(0, 10, (2, 3)))
    for ax in (4, -4):
        with pytest.raises(ValueError):
            hw.unsqueeze_64(z, ax)
    e = hw.expand_64(hw.host_to_device_64(i64([[1], [2]])), 1, 3)
    assert hw.device_to_host_64(e).tolist() == [[1, 1, 1], [2, 2, 2]]
    f = hw.host_to_device_float64(torch.tensor([[1.5, 2.5]], dtype=torch.float64))
    assert torch.equal(hw.device_to_host_float64(hw.make_contiguous_float64(hw.expand_float64(
        hw.unsqueeze_float64(hw.squeeze_float64(f, 0), 0), 0, 2))), torch.tensor([[1.5, 2.5]] * 2,
                                                                                  dtype=torch.float64))
    with pytest.raises(RuntimeError):
        hw.host_to_device_64(torch.zeros(3, dtype=torch.int32))
