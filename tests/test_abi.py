"""CPU tests of the C ABI: the library loads, exports every symbol the header
declares, validates its inputs like the reference's asserts, and refuses to
compute without a CUDA device (there is no CPU fallback)."""

import ctypes as C
import os
import re

import numpy as np
import pytest

import montecarlocpp_gb300 as M
from montecarlocpp_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "mc_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mc_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    syms = header_symbols()
    assert len(syms) >= 18
    for s in syms:
        assert hasattr(L, s), s
    assert set(syms) == set(_lib.SYMBOLS)


def test_version():
    assert b"sm_103a" in _lib.lib().mc_version()


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_material_validation():
    L = _lib.lib()
    h = C.c_void_p()
    disp, relax = M.silicon_tables()
    bad = np.ascontiguousarray(relax.copy())
    bad[0, 0] = -1.0
    d = np.ascontiguousarray(disp)
    rc = L.mc_material_create(d.ctypes.data_as(C.POINTER(C.c_double)), d.shape[0], 3,
                              bad.ctypes.data_as(C.POINTER(C.c_double)), 300.0, C.byref(h))
    assert rc == -1 and b"negative" in L.mc_last_error()
    rc = L.mc_material_load(b"/nonexistent/disp", b"/nonexistent/relax", 300.0, C.byref(h))
    assert rc == -5
    # omega = 0 makes tau infinite (montecarlo/material.cpp:205-206)
    z = d.copy()
    z[0, 0] = 0.0
    rc = L.mc_material_create(z.ctypes.data_as(C.POINTER(C.c_double)), z.shape[0], 3,
                              np.ascontiguousarray(relax).ctypes.data_as(C.POINTER(C.c_double)), 300.0,
                              C.byref(h))
    assert rc == -1 and b"infinite" in L.mc_last_error()


def test_domain_validation():
    # Spec face with a temperature
    with pytest.raises(ValueError):
        M.Domain([M.Parallelepiped(np.zeros(3), np.eye(3), np.zeros(3, int), np.zeros(3),
                                   (M.SPEC,) * 6, (1.0, 0, 0, 0, 0, 0))], [])
    # unpaired Peri face rejected by the library as well
    p = M.Parallelepiped(np.zeros(3), np.eye(3), np.zeros(3, int), np.zeros(3),
                         (M.PERI, M.SPEC, M.SPEC, M.PERI, M.SPEC, M.SPEC))
    ps, n, qs, m = M.problem.domain_descs(type("D", (), {"ppeds": [p], "pairs": []})())
    h = C.c_void_p()
    assert _lib.lib().mc_domain_create_shapes(ps, n, qs, 0, C.byref(h)) == -1
    # the same through the Parallelepiped entry point
    pp = (_lib.PpedDesc * 1)()
    pp[0].M[:] = [1.0, 0, 0, 0, 1.0, 0, 0, 0, 1.0]
    pp[0].kind[:] = [M.PERI, M.SPEC, M.SPEC, M.PERI, M.SPEC, M.SPEC]
    assert _lib.lib().mc_domain_create(pp, 1, qs, 0, C.byref(h)) == -1
    pp[0].kind[:] = [M.SPEC] * 6
    assert _lib.lib().mc_domain_create(pp, 1, qs, 0, C.byref(h)) == 0
    assert _lib.lib().mc_domain_cols(h) == 1
    _lib.lib().mc_domain_destroy(h)
    # more cells than the packed cell index holds
    big = M.FilmDomain.from_cli(1e-7, 1e-7, 600)
    with pytest.raises(_lib.McError) as e:
        M.problem.DomainHandle(big)
    assert e.value.code == -4


def test_domain_columns_and_volumes():
    dom = M.PoreCellDomain(5e-7, 2.5e-7, (2, 4, 2))
    h = M.problem.DomainHandle(dom)
    assert h.cols == dom.cols() == 8 ** 3 - 4 ** 3
    assert np.allclose(h.cell_volumes(), dom.cell_volumes())
    assert np.isclose(h.cell_volumes().sum(), 5e-7 ** 3 - 2.5e-7 ** 3, rtol=1e-12)


def test_problem_validation(gmat):
    dom = M.FilmDomain.from_cli(1e-7, 1e-7, 10)
    with pytest.raises(ValueError):
        M.TempProblem(gmat, dom, 0, 10)
    p = M.TempProblem(gmat, dom, 10, 10)
    with pytest.raises(_lib.McError):
        p.solve(dt=-1.0, nsteps=10)


@pytest.mark.skipif(_has_gpu(), reason="a CUDA device is present")
def test_no_cpu_fallback(gmat):
    p = M.MultiProblem(gmat, M.FilmDomain.from_cli(1e-7, 1e-7, 10), 100, 10)
    with pytest.raises(_lib.McError) as e:
        p.solve(dt=1e-12, nsteps=10)
    assert e.value.code == -3


@pytest.mark.skipif(_has_gpu(), reason="a CUDA device is present")
def test_bounded_wait_check_needs_a_device():
    import ctypes as C
    st, w = C.c_uint(0), C.c_double(0.0)
    assert _lib.lib().mc_check_bounded_wait(10.0, C.byref(st), C.byref(w)) == -3
    assert _lib.lib().mc_check_bounded_wait(0.0, C.byref(st), C.byref(w)) == -1
