"""The reference's own driver (MPI_REAL main.c, system.c, tools.c, unmodified)
links against liblsg.so in place of its four solver files and runs: its
callbacks are recognised by address (exported with -rdynamic), and without a
GPU every solver reports its failure on stderr and leaves the driver running
(no CPU fallback).  Needs the reference checkout; skipped elsewhere."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
try:
    from oracle.oracle import reference_dir
    REF = reference_dir()
except Exception:  # the checker's loader itself unavailable
    REF = ""


@pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "main.c")), reason="reference checkout absent")
def test_reference_driver_links_and_runs(lsg, tmp_path):
    lsg.lib()  # liblsg.so built
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "dropin", f"REF={REF}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    exe = os.path.join(ROOT, "oracle", "_ref", "mpi_real_lsg")
    nm = subprocess.run(["nm", "-D", exe], capture_output=True, text=True).stdout
    for sym in ("AAR", "PGR", "PL2R", "CG"):
        assert f" U {sym}\n" in nm + "\n"  # resolved from liblsg.so
    run = subprocess.run([exe, "1e-8", "7", "6", "0.6", "0.6"], cwd=tmp_path, capture_output=True,
                         text=True, timeout=600)
    assert run.returncode == 0
    for who in ("AAR", "PGR", "PL2R", "CG"):
        ran = f"{who} converged!" in run.stdout
        refused_no_gpu = f"{who} (liblsg): device allocation" in run.stderr or \
            f"{who} (liblsg): " in run.stderr and "CUDA" in run.stderr
        assert ran or refused_no_gpu, (who, run.stdout[-500:], run.stderr[-500:])
        assert "not the reference periodic FD operator" not in run.stderr
