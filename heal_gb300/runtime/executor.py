"""run_transcript: executes an ExecutionTranscript op by op, with the
semantics of HEAL's python_execution/lattica_heal_runtime/runtime.py:69-92:
tensors are held by inf_name, host_to_device / device_to_host are handled
here (the latter compared with the transcript's expected tensor when
verify=True), FREE_DEVICE_TENSOR drops a name, segments are markers, and
every other DeviceOp calls the dispatcher method of the same name with its
decoded arguments.  Returns counts and the wall time (the GPU is
synchronised before the clock stops)."""
from __future__ import annotations

import time

import numpy as np

from .datatypes import DeviceOp, DeviceOpArgType, ExecutionTranscriptOpType


class VerificationError(AssertionError):
    pass


def _arg(refs, arg):
    t = arg.arg_type
    if t == DeviceOpArgType.DEVICE_TENSOR:
        return refs[arg.value.inf_name]
    if t == DeviceOpArgType.SHAPE:
        return tuple(_arg(refs, a) for a in arg.value)
    if t in (DeviceOpArgType.INT, DeviceOpArgType.TENSOR_TYPE):
        return arg.value
    if t == DeviceOpArgType.NONE:
        return None
    if t == DeviceOpArgType.SLICE:
        v = arg.value
        return v if isinstance(v, slice) else slice(v.start, v.stop, v.step)
    if t == DeviceOpArgType.ELLIPSIS:
        return Ellipsis
    if t == DeviceOpArgType.HOST_TENSOR:
        raise ValueError("a host tensor is only an argument of host_to_device")
    raise ValueError(f"unknown argument type {t}")


def _equal(got, want) -> bool:
    g = got.numpy() if hasattr(got, "numpy") else np.asarray(got)
    w = want.numpy() if hasattr(want, "numpy") else np.asarray(want)
    return g.shape == w.shape and np.array_equal(g, w)


def run_device_op(device, refs, op: DeviceOp, verify: bool, stats: dict):
    if op.name == "host_to_device":
        refs[op.out.value.inf_name] = device.host_to_device(op.args[0].value.tensor, op.out.value.dtype)
        return
    if op.name == "device_to_host":
        got = device.device_to_host(refs[op.args[0].value.inf_name])
        stats["device_to_host"] += 1
        if verify:
            if not _equal(got, op.out.value.tensor):
                raise VerificationError(f"device_to_host of {op.args[0].value.inf_name} differs from the "
                                        "transcript's expected tensor")
            stats["verified"] += 1
        return got
    fn = getattr(device, op.name, None)
    if fn is None:
        raise NotImplementedError(f"device op {op.name!r} is not provided by {type(device).__name__}")
    out = fn(*[_arg(refs, a) for a in op.args])
    if op.out is not None and op.out.arg_type == DeviceOpArgType.DEVICE_TENSOR:
        refs[op.out.value.inf_name] = out


def run_transcript(device, transcript, verify: bool = False, log=None) -> dict:
    ops = transcript.transcript if hasattr(transcript, "transcript") else transcript
    refs: dict = {}
    stats = {"device_ops": 0, "device_to_host": 0, "verified": 0, "segments": 0, "freed": 0}
    t0 = time.perf_counter()
    for kind, payload in ops:
        if kind == ExecutionTranscriptOpType.DEVICE_OP:
            if log:
                log(f"device op {payload.name}")
            run_device_op(device, refs, payload, verify, stats)
            stats["device_ops"] += 1
        elif kind == ExecutionTranscriptOpType.FREE_DEVICE_TENSOR:
            del refs[payload.tensor_name]
            stats["freed"] += 1
        elif kind == ExecutionTranscriptOpType.SEGMENT_START:
            stats["segments"] += 1
            if log:
                log(f"segment {payload}")
        elif kind in (ExecutionTranscriptOpType.SEGMENT_END, None):
            pass
        else:
            raise ValueError(f"unknown transcript entry {kind}")
    if hasattr(device, "synchronize"):
        device.synchronize()
    stats["seconds"] = time.perf_counter() - t0
    stats["live_tensors"] = len(refs)
    return stats
