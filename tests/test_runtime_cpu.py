"""Transcript runtime on CPU: the JSON format round-trips and is the one
HEAL's runtime reads and writes (checked against HEAL's own serializer when
its sources are present), the executor's semantics on a host-only fake
device, and that the committed transcripts are what their generator makes."""
import glob
import importlib
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

from heal_gb300 import runtime as R
from heal_gb300.runtime.executor import VerificationError, run_transcript

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = sorted(glob.glob(os.path.join(HERE, "golden", "transcripts", "*.json")))
from oracle import reference  # noqa: E402

REF_RUNTIME = os.path.join(reference.path(), "python_execution") if reference.path() else ""


def flat(t):
    """Comparable form of a transcript: op kinds, names, argument types and
    decoded values."""
    out = []

    def val(a):
        v = a.value
        if isinstance(v, R.DeviceTensorPointer) or hasattr(v, "inf_name"):
            return ("ptr", v.inf_name, str(v.dtype))
        if isinstance(v, R.HostTensor) or hasattr(v, "tensor"):
            return ("host", np.asarray(v.tensor).tobytes(), tuple(v.tensor.shape))
        if isinstance(v, list):
            return ("shape", tuple(val(x) for x in v))
        return ("v", repr(v))

    for kind, payload in t.transcript:
        if hasattr(payload, "name") and hasattr(payload, "args"):
            out.append((kind.name, payload.name, tuple((a.arg_type.name, val(a)) for a in payload.args),
                        (payload.out.arg_type.name, val(payload.out))))
        elif hasattr(payload, "tensor_name"):
            out.append((kind.name, payload.tensor_name))
        else:
            out.append((kind.name, payload))
    return out


def test_golden_transcripts_exist():
    assert [os.path.basename(p) for p in GOLD] == ["keyswitch_n256.json", "matvec_n256.json", "roundtrip_ops_n256.json"]


@pytest.mark.parametrize("path", GOLD, ids=os.path.basename)
def test_round_trip(path):
    t = R.load_transcript_from_json(path)
    assert flat(R.loads(R.dumps(t))) == flat(t)
    n_d2h = sum(1 for k, p in t.transcript if k == R.ExecutionTranscriptOpType.DEVICE_OP and p.name == "device_to_host")
    assert n_d2h >= 2


def _reference_serialization():
    if not os.path.isdir(REF_RUNTIME):
        pytest.skip("HEAL's runtime sources are not on this machine")
    sys.path.insert(0, REF_RUNTIME)
    try:
        return importlib.import_module("lattica_heal_runtime.serialization")
    finally:
        sys.path.remove(REF_RUNTIME)


@pytest.mark.parametrize("path", GOLD, ids=os.path.basename)
def test_heal_serializer_reads_ours_and_we_read_its(path, tmp_path):
    ref = _reference_serialization()
    ours = R.load_transcript_from_json(path)
    theirs = ref.load_transcript_from_json(path)
    assert flat(theirs) == flat(ours)
    again = tmp_path / "again.json"
    ref.save_transcript_to_json(theirs, str(again))
    assert flat(R.load_transcript_from_json(str(again))) == flat(ours)


class HostDevice:
    """A host-only device: just enough ops to drive the executor."""

    def host_to_device(self, tensor, dtype):
        return np.array(tensor.to(dtype).numpy())

    def device_to_host(self, a):
        return torch.from_numpy(np.ascontiguousarray(a))

    def empty(self, shape, dtype):
        return np.zeros(shape, np.int64)

    def reshape(self, a, shape):
        return a.reshape(shape)

    def _modsum_tcc(self, a, b, p, out):
        out[...] = (a + b) % p
        return out


def test_executor_semantics():
    b = R.TranscriptBuilder()
    b.segment("s")
    x = b.host_to_device(torch.arange(6, dtype=torch.int64))
    y = b.op("reshape", x, (2, 3), dtype=torch.int64)
    z = b.op("_modsum_tcc", y, 5, 7, b.op("empty", (2, 3), torch.int64, dtype=torch.int64), dtype=torch.int64)
    b.device_to_host(z, torch.tensor([[5, 6, 0], [1, 2, 3]]))
    b.free(x, y)
    b.end_segment()
    st = run_transcript(HostDevice(), b.transcript(), verify=True)
    assert st["device_ops"] == 5 and st["verified"] == 1 and st["freed"] == 2 and st["segments"] == 1
    assert st["live_tensors"] == 2
    bad = R.TranscriptBuilder()
    x = bad.host_to_device(torch.arange(3, dtype=torch.int64))
    bad.device_to_host(x, torch.tensor([0, 1, 3]))
    with pytest.raises(VerificationError):
        run_transcript(HostDevice(), bad.transcript(), verify=True)
    assert run_transcript(HostDevice(), bad.transcript(), verify=False)["verified"] == 0
    unknown = R.TranscriptBuilder()
    unknown.op("no_such_op", dtype=torch.int64)
    with pytest.raises(NotImplementedError):
        run_transcript(HostDevice(), unknown.transcript())


def test_generator_reproduces_the_committed_transcripts(tmp_path):
    gen = os.path.join(HERE, "golden", "make_transcripts.py")
    env = dict(os.environ, PYTHONPATH=os.path.dirname(HERE))
    code = (f"import runpy, sys; sys.argv=['x']; m = runpy.run_path({gen!r}); "
            f"import heal_gb300.runtime as R; import os; "
            f"[R.save_transcript_to_json(fn(), os.path.join({str(tmp_path)!r}, n)) for n, fn in "
            f"(('keyswitch_n256.json', m['keyswitch']), ('roundtrip_ops_n256.json', m['roundtrip_ops']), "
            f"('matvec_n256.json', m['matvec']))]")
    subprocess.run([sys.executable, "-c", code], check=True, env=env, cwd=os.path.dirname(HERE))
    for path in GOLD:
        new = R.load_transcript_from_json(str(tmp_path / os.path.basename(path)))
        assert flat(new) == flat(R.load_transcript_from_json(path)), path


def _reference_runtime():
    if not os.path.isdir(REF_RUNTIME):
        pytest.skip("HEAL's runtime sources are not on this machine")
    sys.path.insert(0, REF_RUNTIME)
    try:
        return tuple(importlib.import_module(f"lattica_heal_runtime.{m}")
                     for m in ("runtime", "device_interface", "serialization"))
    finally:
        sys.path.remove(REF_RUNTIME)


class _Token:
    def __init__(self, n):
        self.n = n


class Recorder:
    """Stands in for a device: records every call with its arguments resolved
    (a device tensor as the index of the call that produced it) and returns a
    new token per call."""

    def __init__(self):
        self.calls = []

    def _norm(self, v):
        if isinstance(v, _Token):
            return ("dev", v.n)
        if isinstance(v, torch.Tensor):
            return ("host", str(v.dtype), tuple(v.shape), v.contiguous().numpy().tobytes())
        if isinstance(v, (tuple, list)):
            return tuple(self._norm(x) for x in v)
        if isinstance(v, slice):
            return ("slice", v.start, v.stop, v.step)
        return ("v", repr(v))

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)

        def call(*args, **kwargs):
            self.calls.append((name, self._norm(args), self._norm(tuple(sorted(kwargs.items())))))
            return _Token(len(self.calls) - 1)
        return call


@pytest.mark.parametrize("path", GOLD, ids=os.path.basename)
def test_heal_runtime_makes_the_calls_our_executor_makes(path):
    """HEAL's own run_transcript, through HEAL's DeviceDispatcher, issues the
    same device calls with the same arguments as this repository's executor,
    which the GPU tests run on GB300Dispatcher."""
    runtime, device_interface, serialization = _reference_runtime()
    theirs = Recorder()
    runtime.run_transcript(device_interface.DeviceDispatcher(theirs),
                           serialization.load_transcript_from_json(path).transcript, verify=False)
    ours = Recorder()
    run_transcript(ours, R.load_transcript_from_json(path), verify=False)
    ours_calls = [c for c in ours.calls if c[0] != "synchronize"]
    assert len(theirs.calls) > 10
    assert theirs.calls == ours_calls
