"""Transcript JSON: every record is an object tagged "__type__", host tensors
are base64 of torch.save (or np.save) bytes.  The tags and field names are
those HEAL's runtime reads and writes (python_execution/lattica_heal_runtime/
serialization.py:15-148), so transcripts move between the two unchanged.

Reading large transcripts.  HEAL's loader hands the whole text to json.loads
and each payload to base64.b64decode (serialization.py:31,143-148); for a
request carrying megabytes of tensor data both run character by character on
one thread.  `loads` here first cuts every long string under a "data" key out
of the text (a string with no escape in it, so its JSON value is its bytes),
parses the rest, and decodes each cut payload with the C library's
multi-threaded heal_base64_decode.  The result is the same object:
  * a payload the native decoder does not take (not canonical base64) is
    read by json and base64.b64decode as HEAL reads it;
  * a cut string anywhere but in a HostTensor's encoding is put back as the
    string json would have made;
  * when anything does not match (a payload dict outside a HostTensor, text
    that is not UTF-8), the whole text is parsed again the plain way.
Without the C library (a host with no built backend) the payloads go to
base64.b64decode, which gives the same bytes."""
from __future__ import annotations

import base64
import ctypes
import io
import json
import uuid

import numpy as np

from .datatypes import (DeviceOp, DeviceOpArg, DeviceOpArgType, DeviceTensorPointer, ExecutionTranscript,
                        ExecutionTranscriptOpType, FreeDeviceTensor, HostTensor)


def _torch():
    import torch
    return torch


def encode_tensor(tensor) -> dict:
    buf = io.BytesIO()
    if isinstance(tensor, np.ndarray):
        np.save(buf, tensor)
        tag = "numpy"
    else:
        torch = _torch()
        if not isinstance(tensor, torch.Tensor):
            raise TypeError(f"unsupported host tensor type {type(tensor)}")
        torch.save(tensor, buf)
        tag = "torch"
    return {"type": tag, "data": base64.b64encode(buf.getvalue()).decode("ascii")}


# strings under a "data" key at least this long are cut out before parsing
_LIFT_MIN = 1 << 15


class _Payload:
    """A base64 string cut out of transcript text: bytes [a, b) of `raw`."""
    __slots__ = ("raw", "a", "b")

    def __init__(self, raw: bytes, a: int, b: int):
        self.raw, self.a, self.b = raw, a, b

    def text(self) -> str:
        """The string json.loads makes of it (it raises as json would)."""
        return json.loads(b'"' + self.raw[self.a:self.b] + b'"')


def _native_b64decode(p: _Payload, sink=None):
    """heal_base64_decode of the payload in place in its text, into a new
    array or into sink(nbytes) (a writable uint8 array of at least nbytes);
    None when the library is not built or the text is not canonical
    base64."""
    try:
        from .. import capi
        lib = capi.lib()
    except (ImportError, OSError):
        return None
    n = p.b - p.a
    out = np.empty(n // 4 * 3, np.uint8) if sink is None else sink(n // 4 * 3)
    if out.dtype != np.uint8 or out.ndim != 1 or out.size < n // 4 * 3 or not out.flags.writeable:
        raise ValueError("a payload sink must return a writable 1-D uint8 array of the size asked for")
    written = ctypes.c_size_t(0)
    src = ctypes.cast(ctypes.c_char_p(p.raw), ctypes.c_void_p).value + p.a
    if lib.heal_base64_decode(src, n, out.ctypes.data, out.size, ctypes.byref(written), 0) != 0:
        return None
    return memoryview(out)[:written.value]


def _b64decode(data, sink=None):
    if isinstance(data, _Payload):
        got = _native_b64decode(data, sink)
        if got is not None:
            return got
        data = data.text()
    return base64.b64decode(data)


def _npy_view(buf: memoryview):
    """np.load of .npy bytes as an array over `buf` itself (no copy), for a
    version 1.0 or 2.0 header and a plain dtype; None for anything else."""
    fmt = np.lib.format
    f = io.BytesIO(bytes(buf[:1 << 16]))
    try:
        version = fmt.read_magic(f)
        if version == (1, 0):
            shape, fortran, dtype = fmt.read_array_header_1_0(f)
        elif version == (2, 0):
            shape, fortran, dtype = fmt.read_array_header_2_0(f)
        else:
            return None
    except ValueError:
        return None
    count = 1
    for e in shape:
        count *= int(e)
    off = f.tell()
    if dtype.hasobject or off + count * dtype.itemsize > len(buf):
        return None
    return np.frombuffer(buf, dtype=dtype, count=count, offset=off).reshape(shape, order="F" if fortran else "C")


def decode_tensor(obj: dict, sink=None):
    """The host tensor of an encoded payload, as HEAL's decode_tensor makes
    it (serialization.py:30-37).  A numpy payload decoded by the C library
    comes back as an array over the decoded bytes, without np.load's copy
    (in memory from `sink`, when given: see loads)."""
    data = _b64decode(obj["data"], sink)
    if obj["type"] == "numpy":
        if isinstance(data, memoryview) and not data.readonly:
            arr = _npy_view(data)
            if arr is not None:
                return arr
        return np.load(io.BytesIO(data))
    if obj["type"] == "torch":
        return _torch().load(io.BytesIO(data), weights_only=True)
    raise ValueError(f"unknown tensor encoding {obj['type']!r}")


def _dtype_name(d) -> str:
    return str(d).split(".")[-1]


def _encode(obj):
    torch = _torch()
    if isinstance(obj, (DeviceOpArgType, ExecutionTranscriptOpType)):
        return {"__type__": type(obj).__name__, "value": obj.name}
    if isinstance(obj, DeviceTensorPointer):
        return {"__type__": "DeviceTensorPointer", "dtype": str(obj.dtype), "inf_name": obj.inf_name}
    if isinstance(obj, HostTensor):
        return {"__type__": "HostTensor", "tensor_base64": encode_tensor(obj.tensor)}
    if isinstance(obj, DeviceOpArg):
        return {"__type__": "DeviceOpArg", "arg_type": obj.arg_type, "value": obj.value}
    if isinstance(obj, DeviceOp):
        return {"__type__": "DeviceOp", "name": obj.name, "args": obj.args, "out": obj.out}
    if isinstance(obj, FreeDeviceTensor):
        return {"__type__": "FreeDeviceTensor", "tensor_name": obj.tensor_name}
    if isinstance(obj, ExecutionTranscript):
        return {"__type__": "ExecutionTranscript", "transcript": obj.transcript}
    if isinstance(obj, slice):
        return {"__type__": "slice", "start": obj.start, "stop": obj.stop, "step": obj.step}
    if obj is Ellipsis:
        return {"__type__": "ellipsis"}
    if isinstance(obj, torch.dtype):
        return {"__type__": "dtype", "value": _dtype_name(obj)}
    if isinstance(obj, (complex, np.complexfloating)):
        return {"__type__": "complex", "real": obj.real, "imag": obj.imag}
    if isinstance(obj, np.integer):
        return int(obj)
    raise TypeError(f"cannot serialise {type(obj)}")


class _Encoder(json.JSONEncoder):
    def default(self, obj):
        return _encode(obj)


def _decode(d: dict, sink=None):
    t = d.get("__type__")
    if t is None:
        return d
    if t == "DeviceOpArgType":
        return DeviceOpArgType[d["value"]]
    if t == "ExecutionTranscriptOpType":
        return ExecutionTranscriptOpType[d["value"]]
    if t == "DeviceTensorPointer":
        return DeviceTensorPointer(d["inf_name"], getattr(_torch(), _dtype_name(d["dtype"])))
    if t == "HostTensor":
        return HostTensor(decode_tensor(d["tensor_base64"], sink))
    if t == "DeviceOpArg":
        return DeviceOpArg(d["arg_type"], d["value"])
    if t == "DeviceOp":
        return DeviceOp(d["name"], d["args"], d["out"])
    if t == "FreeDeviceTensor":
        return FreeDeviceTensor(d["tensor_name"])
    if t == "ExecutionTranscript":
        return ExecutionTranscript([tuple(item) for item in d["transcript"]])
    if t == "slice":
        return slice(d["start"], d["stop"], d["step"])
    if t == "ellipsis":
        return Ellipsis
    if t == "dtype":
        return getattr(_torch(), d["value"])
    if t == "complex":
        return complex(d["real"], d["imag"])
    raise ValueError(f"unknown record type {t!r}")


def dumps(transcript: ExecutionTranscript, indent=None) -> str:
    return json.dumps(transcript, cls=_Encoder, indent=indent)


def _lift(raw: bytes, tag: bytes):
    """(text with long "data" strings replaced by tag + index, their spans)."""
    pieces, spans, pos, i, n = [], [], 0, 0, len(raw)
    while True:
        i = raw.find(b'"data"', i)
        if i < 0:
            break
        j = i + 6
        if i and raw[i - 1] == 0x5C:  # an escaped quote inside some string
            i = j
            continue
        while j < n and raw[j] in b" \t\r\n":
            j += 1
        if j >= n or raw[j] != 0x3A:  # not a key
            i = j
            continue
        j += 1
        while j < n and raw[j] in b" \t\r\n":
            j += 1
        if j >= n or raw[j] != 0x22:  # the value is not a string
            i = j
            continue
        a = j + 1
        b = raw.find(b'"', a)
        if b < 0:
            break
        if b - a >= _LIFT_MIN and raw.find(b"\\", a, b) < 0:
            pieces += [raw[pos:a], tag + str(len(spans)).encode()]
            spans.append((a, b))
            pos = b
        i = b + 1
    pieces.append(raw[pos:])
    return b"".join(pieces), spans


def loads(text, sink=None) -> ExecutionTranscript:
    """A transcript from its JSON text (str or UTF-8 bytes); the same object
    HEAL's load_transcript_from_json makes of it (serialization.py:143-148).
    With `sink`, every payload the C library decodes is written into
    sink(nbytes), a writable 1-D uint8 array the caller provides (a server
    passes pinned host memory, so that a numpy payload is ready for an
    asynchronous upload where it lands)."""
    try:
        raw = text.encode("utf-8") if isinstance(text, str) else bytes(text)
    except UnicodeEncodeError:
        return json.loads(text, object_hook=_decode)
    tag = f"__heal_payload_{uuid.uuid4().hex}_".encode()
    skeleton, spans = _lift(raw, tag)
    if not spans:
        return json.loads(text, object_hook=_decode)
    stag, count = tag.decode(), {"cut": 0, "used": 0}

    def hook(d: dict):
        v = d.get("data")
        if isinstance(v, str) and v.startswith(stag):
            a, b = spans[int(v[len(stag):])]
            if set(d) == {"type", "data"}:
                d["data"] = _Payload(raw, a, b)
                count["cut"] += 1
            else:
                d["data"] = _Payload(raw, a, b).text()
        if d.get("__type__") == "HostTensor" and isinstance(d.get("tensor_base64"), dict) and \
                isinstance(d["tensor_base64"].get("data"), _Payload):
            count["used"] += 1
        return _decode(d, sink)

    out = json.loads(skeleton, object_hook=hook)
    if count["cut"] != count["used"]:
        return json.loads(text, object_hook=_decode)
    return out


def save_transcript_to_json(transcript: ExecutionTranscript, filename: str):
    with open(filename, "w") as f:
        f.write(dumps(transcript, indent=1))


def load_transcript_from_json(filename: str) -> ExecutionTranscript:
    with open(filename) as f:
        return loads(f.read())
