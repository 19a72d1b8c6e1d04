"""Transcript payload decoding on the host: the C library's base64 decoder
against base64.b64decode, and runtime.loads (long payloads cut out of the
JSON text and decoded natively, numpy payloads used in place) against the
plain json.loads + base64.b64decode + np.load / torch.load that HEAL's
serializer runs (python_execution/lattica_heal_runtime/serialization.py:
30-37, 143-148).  No GPU is touched."""
import base64
import binascii
import ctypes
import json

import numpy as np
import pytest
import torch

from heal_gb300 import capi
from heal_gb300 import runtime as R
from heal_gb300.runtime import serialization as Z
from heal_gb300.runtime import DeviceOpArgType as A
from heal_gb300.runtime import TranscriptBuilder


def native(text: bytes, threads=0, cap=None):
    out = np.empty(max(1, len(text) // 4 * 3 if cap is None else cap), np.uint8)
    w = ctypes.c_size_t(12345)
    rc = capi.lib().heal_base64_decode(text, len(text), out.ctypes.data, len(text) // 4 * 3 if cap is None else cap,
                                       ctypes.byref(w), threads)
    return rc, bytes(out[:w.value]) if rc == 0 else w.value


@pytest.mark.parametrize("threads", [0, 1, 3, 16])
def test_decoder_equals_b64decode(threads):
    rng = np.random.default_rng(threads)
    sizes = list(range(0, 40)) + [3 * (1 << 16) - 1, 3 * (1 << 16), 1_000_001, 3 * (1 << 20) + 2]
    for n in sizes:
        raw = rng.integers(0, 256, n, dtype=np.uint8).tobytes()
        text = base64.b64encode(raw)
        rc, got = native(text, threads)
        assert rc == 0 and got == raw == base64.b64decode(text), n


def test_decoder_rejects_what_is_not_canonical():
    good = base64.b64encode(bytes(range(200)))
    bad = [b"abc", b"ab=c", b"a===", b"====", b"ab\ncd==", b"ab*d", b"ab-_", good[:-4] + b"A=B=",
           good[:100] + b"!" + good[101:], b"QUJD" * 70000 + b"QU$D" + b"QUJD" * 70000]
    for text in bad:
        rc, written = native(text)
        assert rc == 1, text[:16]  # HEAL_ERR_INVALID_ARGUMENT
        assert written == 0
    # an output buffer one byte too small
    rc, _ = native(good, cap=len(good) // 4 * 3 - 2)
    assert rc == 1 and "too small" in capi.lib().heal_last_error().decode()


def plain(text):
    return json.loads(text, object_hook=Z._decode)


def same(a, b):
    """Two decoded transcripts hold the same records and host tensors."""
    assert len(a.transcript) == len(b.transcript)
    for (ka, pa), (kb, pb) in zip(a.transcript, b.transcript):
        assert ka == kb and type(pa) is type(pb)
        if hasattr(pa, "args"):
            assert pa.name == pb.name
            for x, y in zip(pa.args + [pa.out], pb.args + [pb.out]):
                assert x.arg_type == y.arg_type
                if x.arg_type == A.HOST_TENSOR:
                    tx, ty = x.value.tensor, y.value.tensor
                    assert type(tx) is type(ty) and tx.dtype == ty.dtype and tuple(tx.shape) == tuple(ty.shape)
                    if isinstance(tx, np.ndarray):
                        assert np.array_equal(tx, ty)
                        assert tx.flags.c_contiguous == ty.flags.c_contiguous and tx.flags.writeable
                    else:
                        assert torch.equal(tx, ty)
                elif x.arg_type == A.DEVICE_TENSOR:
                    assert x.value.inf_name == y.value.inf_name and x.value.dtype == y.value.dtype
                else:
                    assert repr(x.value) == repr(y.value)


def transcript(tensors, indent=None):
    tb = TranscriptBuilder(prefix="t")
    tb.segment("s")
    ptrs = [tb.host_to_device(t) for t in tensors]
    for p, t in zip(ptrs, tensors):
        tb.device_to_host(p, t)
    tb.end_segment()
    return R.dumps(tb.transcript(), indent=indent)


def payloads(seed):
    rng = np.random.default_rng(seed)
    return [rng.integers(0, 1 << 40, (64, 1, 1, 64, 12), dtype=np.int64),            # 3 MB, threaded
            np.asfortranarray(rng.integers(-9, 9, (300, 70), dtype=np.int32)),        # Fortran order
            torch.from_numpy(rng.integers(0, 1 << 30, (2, 4096, 3), dtype=np.int64)),  # torch.save payload
            rng.integers(0, 5, (3, 4), dtype=np.int64),                               # below the cut size
            rng.standard_normal((5000,))]                                             # float64


@pytest.mark.parametrize("indent", [None, 1])
def test_loads_equals_the_plain_parse(indent):
    text = transcript(payloads(indent or 0), indent)
    skeleton, spans = Z._lift(text.encode(), b"__tag_")
    # every payload above the cut size (4 tensors, each uploaded and expected back) was cut
    assert len(spans) == 8 and len(skeleton) < 20000
    want = plain(text)
    for t in (text, text.encode()):
        same(R.loads(t), want)


def test_strings_cut_outside_a_tensor_are_put_back():
    big = "x" * 50000 + "é" + "y" * 10
    text = transcript([np.arange(40000, dtype=np.int64)])
    obj = json.loads(text)
    # a long "data" string as a DeviceOpArg value, next to the real payload
    int_arg = lambda v: {"__type__": "DeviceOpArg", "arg_type": {"__type__": "DeviceOpArgType", "value": "INT"},
                         "value": v}
    obj["transcript"].insert(0, ["DEVICE_OP", {"__type__": "DeviceOp", "name": "note", "out": int_arg(0),
                                               "args": [int_arg({"data": big, "k": 1})]}])
    obj["transcript"][0][0] = {"__type__": "ExecutionTranscriptOpType", "value": "DEVICE_OP"}
    text2 = json.dumps(obj, ensure_ascii=False)
    got, want = R.loads(text2), plain(text2)
    assert got.transcript[0][1].args[0].value == want.transcript[0][1].args[0].value == {"data": big, "k": 1}
    same(got, want)
    # a tensor encoding outside any HostTensor: the whole text is parsed the plain way
    obj["transcript"][0][1]["args"][0]["value"] = {"type": "numpy", "data": base64.b64encode(bytes(60000)).decode()}
    text3 = json.dumps(obj)
    got = R.loads(text3)
    assert got.transcript[0][1].args[0].value == plain(text3).transcript[0][1].args[0].value
    assert isinstance(got.transcript[0][1].args[0].value["data"], str)


def test_payloads_the_native_decoder_refuses_decode_as_heal_does():
    arr = np.arange(30000, dtype=np.int64)
    enc = Z.encode_tensor(arr)["data"]
    decoded = 0
    for data in (enc[:-1],                       # padding cut short
                 enc.replace("A", "-A", 1),      # a character outside the alphabet, which b64decode drops
                 enc + "===="):                  # padding after the end
        text = transcript([arr]).replace(enc, data)
        assert text.count(data) == 2
        try:
            want = plain(text)
        except (binascii.Error, ValueError) as e:
            with pytest.raises(type(e)):
                R.loads(text)
            continue
        same(R.loads(text), want)
        decoded += 1
    assert decoded >= 1
