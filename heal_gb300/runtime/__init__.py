"""HEAL's transcript runtime on the GB300 backend.

  datatypes      the transcript's records (the field layout of HEAL's
                 python_execution/lattica_heal_runtime/datatypes.py:1-41)
  serialization  JSON with base64 tensors, the format HEAL's runtime reads
                 and writes (serialization.py:15-148)
  dispatcher     GB300Dispatcher: every op DeviceDispatcher routes
                 (device_interface.py:3-114) on the lattica_hw module
  executor       run_transcript (runtime.py:69-92 semantics)
  builder        TranscriptBuilder: records a transcript from Python calls
"""
from .datatypes import (DeviceOp, DeviceOpArg, DeviceOpArgType, DeviceTensorPointer, ExecutionTranscript,
                        ExecutionTranscriptOpType, FreeDeviceTensor, HostTensor)
from .serialization import load_transcript_from_json, save_transcript_to_json, dumps, loads
from .builder import TranscriptBuilder

__all__ = ["DeviceOp", "DeviceOpArg", "DeviceOpArgType", "DeviceTensorPointer", "ExecutionTranscript",
           "ExecutionTranscriptOpType", "FreeDeviceTensor", "HostTensor", "load_transcript_from_json",
           "save_transcript_to_json", "dumps", "loads", "TranscriptBuilder"]
