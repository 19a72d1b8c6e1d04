"""Transcript JSON: every record is an object tagged "__type__", host tensors
are base64 of torch.save (or np.save) bytes.  The tags and field names are
those HEAL's runtime reads and writes (python_execution/lattica_heal_runtime/
serialization.py:15-148), so transcripts move between the two unchanged."""
from __future__ import annotations

import base64
import io
import json

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


def decode_tensor(obj: dict):
    raw = io.BytesIO(base64.b64decode(obj["data"]))
    if obj["type"] == "numpy":
        return np.load(raw)
    if obj["type"] == "torch":
        return _torch().load(raw, weights_only=True)
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


def _decode(d: dict):
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
        return HostTensor(decode_tensor(d["tensor_base64"]))
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


def loads(text: str) -> ExecutionTranscript:
    return json.loads(text, object_hook=_decode)


def save_transcript_to_json(transcript: ExecutionTranscript, filename: str):
    with open(filename, "w") as f:
        f.write(dumps(transcript, indent=1))


def load_transcript_from_json(filename: str) -> ExecutionTranscript:
    with open(filename) as f:
        return loads(f.read())
