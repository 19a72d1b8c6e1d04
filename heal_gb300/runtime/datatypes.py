"""Records of an execution transcript.  The class names, fields and enum
values are those of HEAL's python_execution/lattica_heal_runtime/
datatypes.py:1-41, because the JSON that compilers emit names them."""
from __future__ import annotations

from enum import Enum
from typing import Any


class DeviceTensorPointer:
    """A device tensor by name: the transcript refers to tensors by inf_name."""

    def __init__(self, inf_name: str | None = None, dtype: Any = None):
        self.inf_name = inf_name
        self.dtype = dtype

    def __repr__(self):
        return f"DeviceTensorPointer({self.inf_name}, {self.dtype})"


class HostTensor:
    """A host tensor carried in the transcript (torch.Tensor or numpy)."""

    def __init__(self, tensor=None):
        self.tensor = tensor


class DeviceOpArgType(Enum):
    HOST_TENSOR = "HostTensor"
    DEVICE_TENSOR = "DeviceTensor"
    SHAPE = "Shape"
    INT = "int"
    NONE = "None"
    TENSOR_TYPE = "tensor_type"
    SLICE = "slice"
    ELLIPSIS = "Ellipsis"


class DeviceOpArg:
    def __init__(self, arg_type: DeviceOpArgType | None = None, value: Any = None):
        self.arg_type = arg_type
        self.value = value


class DeviceOp:
    def __init__(self, name: str | None = None, args: list | None = None, out: DeviceOpArg | None = None):
        self.name = name
        self.args = args if args is not None else []
        self.out = out


class FreeDeviceTensor:
    def __init__(self, tensor_name: str):
        self.tensor_name = tensor_name


class ExecutionTranscriptOpType(Enum):
    SEGMENT_START = "SegmentStart"
    SEGMENT_END = "SegmentEnd"
    DEVICE_OP = "DeviceOp"
    FREE_DEVICE_TENSOR = "FreeDeviceTensor"


class ExecutionTranscript:
    def __init__(self, transcript: list | None = None):
        self.transcript = transcript if transcript is not None else []
