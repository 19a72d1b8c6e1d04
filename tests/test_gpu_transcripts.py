"""The committed verify-transcripts (HEAL's transcript format, expected
tensors from the oracle) run on GB300Dispatcher through the transcript
executor, every device_to_host bit-exact."""
import glob
import os

import pytest
import torch

from heal_gb300 import runtime as R
from heal_gb300.runtime.dispatcher import GB300Dispatcher
from heal_gb300.runtime.executor import VerificationError, run_transcript
from _gpu import ready

pytestmark = pytest.mark.gpu
GOLD = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "transcripts", "*.json")))


@pytest.fixture(scope="module")
def device():
    ready()
    return GB300Dispatcher()


@pytest.mark.parametrize("path", GOLD, ids=os.path.basename)
def test_transcript_verifies(device, path):
    t = R.load_transcript_from_json(path)
    n_d2h = sum(1 for k, p in t.transcript if k == R.ExecutionTranscriptOpType.DEVICE_OP and p.name == "device_to_host")
    st = run_transcript(device, t, verify=True)
    assert st["verified"] == n_d2h >= 2


def test_a_wrong_expected_tensor_is_caught(device):
    t = R.load_transcript_from_json([p for p in GOLD if "matvec" in p][0])
    for kind, op in reversed(t.transcript):
        if kind == R.ExecutionTranscriptOpType.DEVICE_OP and op.name == "device_to_host":
            exp = op.out.value.tensor.clone()
            exp.view(-1)[17] += 1
            op.out.value.tensor = exp
            break
    with pytest.raises(VerificationError):
        run_transcript(device, t, verify=True)
