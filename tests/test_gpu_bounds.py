"""Bounds-checked build (LSG_BOUNDS=1 python linear-solver_gb300/build.py):
the stencil marches check every global and shared index, record the first
one out of range and skip the access.  The solves below cover both marches
(one-column and paired) on odd, ragged and even grids, every vector type,
batches and the generic radius; none may record an index.  In the normal
build the test is skipped (lsg.bounds_errors() is None).

Also: tracing (LSG_NVTX=1) in a child process leaves a solve unchanged."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_no_out_of_range_index(lsg):
    import torch
    if lsg.bounds_errors() is None:
        pytest.skip("normal build (no index checks)")
    rng = np.random.default_rng(1)
    grids = [(13, 17, 11), (12, 10, 8), (5, 7, 9), (64, 48, 40), (66, 34, 20)]
    for n in grids:
        b = rng.uniform(-0.5, 0.5, n[::-1])
        b -= b.mean()
        op = lsg.Operator(n, a=-float(n[0] * n[1]) ** 0.5, sigma=1.0)
        bt = torch.from_numpy(b).cuda()
        lsg.aar(op, bt, max_iter=40)
        lsg.aar(op, bt.float(), max_iter=40)
        lsg.aar_mixed(op, bt, tol=1e-6, max_iter=200)
        lsg.cg(op, bt, max_iter=20)
        lsg.pgr(op, bt, max_iter=20)
        lsg.aar(lsg.Operator(n, radius=4, sigma=1.0), bt, max_iter=20)
        lsg.apply(op, bt)
        bc = (bt + 1j * bt).to(torch.complex128)
        lsg.aar(lsg.Operator(n, sigma=2.0 + 1.0j), bc, max_iter=24)
        lsg.aar(lsg.Operator(n, sigma=2.0 + 1.0j), bc.to(torch.complex64), max_iter=24)
    ops = [lsg.Operator(g, sigma=3.0) for g in grids[:3]]
    bs = [torch.from_numpy(rng.uniform(-0.5, 0.5, g[::-1])).cuda() for g in grids[:3]]
    lsg.aar_batched(ops, bs, max_iter=30)
    lsg.aar_batched(ops, bs, mixed=True, tol=1e-6, max_iter=120)
    lsg.autotune(lsg.Operator(64), torch.float32)
    lsg.aar(lsg.Operator(64), torch.from_numpy(rng.uniform(-0.5, 0.5, (64, 64, 64))).cuda().float(), max_iter=30)
    torch.cuda.synchronize()
    assert lsg.bounds_errors() == -1


CHILD = r"""
import sys
sys.path.insert(0, "linear-solver_gb300")
import torch, lsg, workloads
op = lsg.Operator(32)
b = torch.from_numpy(workloads.uniform_rhs(32, 2)).cuda()
x, r = lsg.aar_mixed(op, b - b.mean(), tol=1e-8)
print("status", r["status"], r["iters"])
"""


def test_tracing_leaves_solve_unchanged():
    outs = []
    for flag in ("0", "1"):
        env = dict(os.environ, LSG_NVTX=flag)
        out = subprocess.run([sys.executable, "-c", CHILD], cwd=ROOT, env=env, capture_output=True, text=True,
                             timeout=300)
        assert out.returncode == 0, out.stderr[-2000:]
        outs.append([l for l in out.stdout.splitlines() if l.startswith("status")])
    assert outs[0] == outs[1] and outs[0][0].split()[1] == "0", outs
