"""TranscriptBuilder: records an ExecutionTranscript from Python calls, the
way a compiler front end emits one.  Device tensors are handles
(DeviceTensorPointer) with generated names; arguments are typed like the
transcript's DeviceOpArg records."""
from __future__ import annotations

from .datatypes import (DeviceOp, DeviceOpArg, DeviceOpArgType, DeviceTensorPointer, ExecutionTranscript,
                        ExecutionTranscriptOpType, FreeDeviceTensor, HostTensor)


class TranscriptBuilder:
    def __init__(self, prefix: str = "t"):
        self.entries = []
        self.prefix = prefix
        self.count = 0

    def _ptr(self, dtype) -> DeviceTensorPointer:
        self.count += 1
        return DeviceTensorPointer(f"{self.prefix}{self.count}", dtype)

    def _arg(self, v) -> DeviceOpArg:
        import torch
        if isinstance(v, DeviceTensorPointer):
            return DeviceOpArg(DeviceOpArgType.DEVICE_TENSOR, v)
        if v is None:
            return DeviceOpArg(DeviceOpArgType.NONE, None)
        if isinstance(v, bool):
            return DeviceOpArg(DeviceOpArgType.INT, bool(v))
        if isinstance(v, int):
            return DeviceOpArg(DeviceOpArgType.INT, int(v))
        if isinstance(v, (tuple, list)):
            return DeviceOpArg(DeviceOpArgType.SHAPE, [self._arg(x) for x in v])
        if isinstance(v, torch.dtype):
            return DeviceOpArg(DeviceOpArgType.TENSOR_TYPE, v)
        if isinstance(v, slice):
            return DeviceOpArg(DeviceOpArgType.SLICE, v)
        if v is Ellipsis:
            return DeviceOpArg(DeviceOpArgType.ELLIPSIS, None)
        if hasattr(v, "item"):                       # numpy / torch scalars
            return DeviceOpArg(DeviceOpArgType.INT, int(v))
        raise TypeError(f"cannot record argument of type {type(v)}")

    # ---- records
    def segment(self, name: str):
        self.entries.append((ExecutionTranscriptOpType.SEGMENT_START, name))

    def end_segment(self):
        self.entries.append((ExecutionTranscriptOpType.SEGMENT_END, None))

    def host_to_device(self, tensor) -> DeviceTensorPointer:
        out = self._ptr(tensor.dtype)
        self.entries.append((ExecutionTranscriptOpType.DEVICE_OP,
                             DeviceOp("host_to_device", [DeviceOpArg(DeviceOpArgType.HOST_TENSOR, HostTensor(tensor))],
                                      DeviceOpArg(DeviceOpArgType.DEVICE_TENSOR, out))))
        return out

    def device_to_host(self, ptr: DeviceTensorPointer, expected):
        self.entries.append((ExecutionTranscriptOpType.DEVICE_OP,
                             DeviceOp("device_to_host", [self._arg(ptr)],
                                      DeviceOpArg(DeviceOpArgType.HOST_TENSOR, HostTensor(expected)))))

    def op(self, name: str, *args, dtype) -> DeviceTensorPointer:
        """A DeviceOp returning a device tensor of `dtype`."""
        out = self._ptr(dtype)
        self.entries.append((ExecutionTranscriptOpType.DEVICE_OP,
                             DeviceOp(name, [self._arg(a) for a in args], DeviceOpArg(DeviceOpArgType.DEVICE_TENSOR, out))))
        return out

    def free(self, *ptrs: DeviceTensorPointer):
        for p in ptrs:
            self.entries.append((ExecutionTranscriptOpType.FREE_DEVICE_TENSOR, FreeDeviceTensor(p.inf_name)))

    def transcript(self) -> ExecutionTranscript:
        return ExecutionTranscript(list(self.entries))
