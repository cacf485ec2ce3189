"""Failure detection on the GPU without a fault: a bounded device wait that
runs out reports LSG_TIMEOUT and leaves the context usable.

The FP32 Gram streams the history through shared memory with bulk copies
whose completion each stage's mbarrier waits for, with a time limit.  Setting
LSG_FAULT_GRAM_TX arms every stage with more bytes than its copies deliver:
all copies land, the barrier phase never completes, the waits give up after
their limit (LSG_GRAM_WAIT_CYCLES, here ~10 ms; solves use ~2 s), and the
kernel sets LSG_TIMEOUT and stops the solve.
The child process then runs an FP64 solve (no bulk-copy Gram) on the same
context, which must converge as usual.
"""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import sys
sys.path.insert(0, "linear-solver_gb300")
import torch, lsg, workloads
op = lsg.Operator(32)
b = torch.from_numpy(workloads.uniform_rhs(32, 2)).cuda()
try:
    lsg.aar(op, b.float(), tol=1e-5)
    print("FP32 status ok")
except lsg.CudaLibraryError as e:
    print("FP32 error:", e)
x, r = lsg.aar(op, b, tol=1e-8)
print("FP64 status", r["status"], r["iters"])
"""


def test_gram_wait_timeout_reported_context_usable():
    # each wait gives up after 2e7 SM clocks (~10 ms) instead of the solves' ~2 s
    env = dict(os.environ, LSG_FAULT_GRAM_TX="16", LSG_GRAM_WAIT_CYCLES="20000000")
    out = subprocess.run([sys.executable, "-c", CHILD], cwd=ROOT, env=env, capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = out.stdout.splitlines()
    assert any(l.startswith("FP32 error:") and "timeout" in l for l in lines), out.stdout
    fp64 = [l for l in lines if l.startswith("FP64 status")]
    assert fp64 and fp64[0].split()[2] == "0", out.stdout
