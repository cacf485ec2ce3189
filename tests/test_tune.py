"""Autotuner of the stencil launch shape (lsg_tune.cu).

Host side (no GPU): the tuned-shape cache file round trip and argument
checks.  GPU: every candidate shape is timed and the fastest cached; the
Richardson pass writes no partial sums and each point's stencil sum is
evaluated in the same order whatever the tile, so a solve on a tuned shape
reproduces the default-shape solve bit for bit; batched solves tune their
tile variant and z depth and keep each instance's iteration count.
"""
import os

import numpy as np
import pytest


def test_cache_file_round_trip(lsg, tmp_path):
    src = tmp_path / "in.txt"
    src.write_text("# comment\n0 1 63 61 59 2 16 12.5 14.0\n0 0 47 45 43 1 43 30.0 31.0\n"
                   "0 1 31 29 27 7 8 1.0 1.0\nnot a line\n")
    assert lsg.autotune_load(str(src)) == 2  # tile 7 is not a variant: skipped
    out = tmp_path / "out.txt"
    lsg.autotune_save(str(out))
    rows = [l.split() for l in out.read_text().splitlines() if not l.startswith("#")]
    keyed = {tuple(r[:5]): r[5:7] for r in rows}
    assert keyed[("0", "1", "63", "61", "59")] == ["2", "16"]
    assert keyed[("0", "0", "47", "45", "43")] == ["1", "43"]


def test_bad_arguments(lsg):
    with pytest.raises(lsg.CudaLibraryError):
        lsg.set_autotune(3)
    with pytest.raises(lsg.CudaLibraryError):
        lsg.autotune_load("/nonexistent/lsg_tune_cache.txt")
    lsg.set_autotune(1)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype_name,n", [("float32", 64), ("float64", 48), ("complex64", 40), ("complex128", 32)])
def test_tuned_shape_reproduces_default_solve(lsg, dtype_name, n):
    import torch
    dt = getattr(torch, dtype_name)
    rng = np.random.default_rng(n)
    b = rng.uniform(-0.5, 0.5, (n, n, n))
    if dt.is_complex:
        b = b + 1j * rng.uniform(-0.5, 0.5, (n, n, n))
    b = torch.from_numpy(b - b.mean()).to(device="cuda", dtype=dt)
    op = lsg.Operator(n, a=-float(n * n), sigma=(2.0 + 3.0j) if dt.is_complex else 2.0)
    tol = 1e-5 if dt in (torch.float32, torch.complex64) else 1e-9
    lsg.set_autotune(0)
    x0, r0 = lsg.aar(op, b, tol=tol)
    info = lsg.autotune(op, dt)
    assert info["candidates"] >= 4
    assert 0 <= info["tile"] <= 4 and 1 <= info["lz"] <= n  # 3, 4: the paired FP32 march (two shapes)
    assert info["us_best"] <= info["us_default"]
    lsg.set_autotune(1)
    x1, r1 = lsg.aar(op, b, tol=tol)
    assert r1["iters"] == r0["iters"]
    assert torch.equal(x0, x1)


@pytest.mark.gpu
def test_batched_tuning_keeps_iterations(lsg):
    import torch
    ns = [32, 48, 24, 40]
    ops = [lsg.Operator(n, a=-float(n * n), sigma=1.0 + k) for k, n in enumerate(ns)]
    rng = np.random.default_rng(7)
    bs = [torch.from_numpy(rng.uniform(-0.5, 0.5, (n, n, n))).cuda() for n in ns]
    lsg.set_autotune(0)
    xs0, rs0 = lsg.aar_batched(ops, bs, mixed=True, tol=1e-9)
    lsg.set_autotune(2)
    try:
        xs1, rs1 = lsg.aar_batched(ops, bs, mixed=True, tol=1e-9)
    finally:
        lsg.set_autotune(1)
    for x0, x1, r0, r1 in zip(xs0, xs1, rs0, rs1):
        assert r1["status"] == 0
        assert abs(r1["iters"] - r0["iters"]) <= 12
        assert ((x0 - x1).norm() / x0.norm()).item() <= 1e-7
