"""The C-ABI library loads and exports every function include/*.h declares
(no device calls), plus host-side argument checks that return before any
CUDA call."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in ("lsg.h", "lsg_compat.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?!typedef)(?:const\s+)?[a-z_]+\s*\**\s*([A-Za-z_0-9]+)\s*\(", src, flags=re.M):
            if m.group(1) not in ("if", "return", "sizeof", "typedef"):
                names.add(m.group(1))
    return names


def test_headers_declare_expected_entry_points():
    names = _declared()
    for n in ("AAR", "PGR", "PL2R", "CG", "lsg_aar", "lsg_pgr", "lsg_pl2r", "lsg_cg",
              "lsg_aar_mixed", "lsg_apply", "lsg_pinv_solve"):
        assert n in names


def test_library_exports_every_declared_symbol(lsg):
    out = subprocess.run(["nm", "-D", "--defined-only", lsg.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = sorted(_declared() - exported)
    assert not missing, missing
    for name in _declared():
        assert hasattr(lsg.lib(), name)


def test_host_only_entry_points(lsg):
    L = lsg.lib()
    assert L.lsg_version().decode().startswith("lsg")
    assert lsg.lap_coefficient(6)[1] == pytest.approx(12.0 / 7.0, rel=1e-15)
    assert L.lsg_status_string(1).decode() == "not converged"
    op = lsg.Operator((9, 10, 11), radius=3, sigma=0.5)
    assert op.shape == (11, 10, 9)
    assert op.diag == pytest.approx(op.a * 3 * op.coeff[0] + 0.5)
    assert L.lsg_status_string(5).decode() == "device wait timed out"
    # the index checks exist only in the LSG_BOUNDS=1 build
    variant = os.path.join(os.path.dirname(lsg.__file__), "_build", "liblsg.variant")
    if not os.path.exists(variant) or open(variant).read().strip() == "normal":
        assert lsg.bounds_errors() is None


def test_bad_arguments_rejected_before_any_device_call(lsg):
    L = lsg.lib()
    prm = lsg._params()
    res = lsg._Result()
    # NULL operator
    assert L.lsg_aar(None, C.byref(prm), 0, None, None, C.byref(res), None) == 3
    op = lsg._Operator()
    L.lsg_operator_init(C.byref(op), 8, 8, 8, 6, -1.0, 0.0, 1)
    op.radius = 9
    assert L.lsg_aar(C.byref(op), C.byref(prm), 0, C.c_void_p(1), C.c_void_p(1), C.byref(res), None) == 3
    assert b"radius" in L.lsg_last_error()
    op.radius = 6
    prm.m = 33
    assert L.lsg_aar(C.byref(op), C.byref(prm), 0, C.c_void_p(1), C.c_void_p(1), C.byref(res), None) == 3
    prm.m = 7
    prm.p = 0
    assert L.lsg_pgr(C.byref(op), C.byref(prm), 0, C.c_void_p(1), C.c_void_p(1), C.byref(res), None) == 3
    prm.p = 6
    assert L.lsg_cg(C.byref(op), C.byref(prm), 7, C.c_void_p(1), C.c_void_p(1), C.byref(res), None) == 3
    assert L.lsg_pinv_solve(None, None, None, 40, None) == 3


def test_compat_refuses_unknown_callbacks_and_distributed_domains(lsg):
    import numpy as np
    x = np.zeros((8, 8, 8))
    b = np.ones((8, 8, 8))
    foreign = lsg.LAP_FN(lambda *a: None)
    r = lsg.compat_solve("aar", x, b, lap=foreign)
    assert r["last_status"] == 6  # unsupported: no CPU fallback
    foreign_pc = lsg.PRECOND_FN(lambda *a: None)
    r = lsg.compat_solve("cg", x, b, pc=foreign_pc)
    assert r["last_status"] == 6
    s = lsg.make_poisson((8, 8, 8))
    s.psize[0] = 4  # a 2-rank split along x
    r = lsg.compat_solve("pgr", x, b, system=s)
    assert r["last_status"] == 6
    assert np.all(x == 0)  # x untouched on refusal
