"""mc_solve_noalloc against mc_solve, both called through the C ABI.

mc_solve_noalloc is for callers that cannot call cudaMalloc / cudaFree: a
process whose GPU memory is already owned by another allocator (a caching
pool, a runtime that reserves the device at start-up), where a new
cudaMalloc can fail although that pool has room, or a loop that cannot take
the device-wide synchronisation of cudaFree. It places every device buffer
of the solve in one fixed array of MC_NOALLOC_SCRATCH_BYTES (32 MiB) that
all calls share, so these tests run two different solves back to back (the
second must not see the first's counters, tally or phonons) and repeat the
first, each checked against mc_solve with the tolerances of the other GPU
tests: FP64 flight fields within 1e-12 and FP32 within 1e-10 of each row's
largest magnitude, event counts identical. Once a first call has loaded the
kernels, further calls leave the device's free memory unchanged.

The file is named to be collected last.
"""

import ctypes as C

import numpy as np
import pytest

import montecarlocpp_gb300 as M
from montecarlocpp_gb300 import _lib

pytestmark = pytest.mark.gpu

SCRATCH_BYTES = 32 << 20  # MC_NOALLOC_SCRATCH_BYTES in include/mc_gb300.h


def _field_err(a, b):
    scale = np.abs(a).max(axis=1, keepdims=True)
    scale[scale == 0] = 1
    return float((np.abs(a - b) / scale).max())


def _call(fn, P, **kw):
    d, keep, _ = P.desc(**kw)
    out = np.zeros(P.rows() * P.handle.cols)
    st = _lib.Stats()
    rc = fn(P.mat.h, P.handle.h, C.byref(d), out.ctypes.data_as(C.POINTER(C.c_double)), C.byref(st))
    del keep
    return rc, out.reshape(P.rows(), P.handle.cols, order="F"), st.as_dict()


def _both(P, **kw):
    L = _lib.lib()
    rc, ref, sref = _call(L.mc_solve, P, **kw)
    _lib.check(rc)
    rc, got, sgot = _call(L.mc_solve_noalloc, P, **kw)
    _lib.check(rc)
    return ref, sref, got, sgot


def _check(P, tol, **kw):
    ref, sref, got, sgot = _both(P, **kw)
    for k in ("nemit", "events", "scatters", "absorbed", "horizon_stops", "phonon_steps"):
        assert sgot[k] == sref[k], k
    assert _field_err(ref, got) < tol
    assert np.allclose(sgot["checksum"], sref["checksum"], rtol=1e-12, atol=0)
    return got


def test_noalloc_matches_mc_solve_on_consecutive_calls():
    mat = M.Material.silicon(300.0)
    film = M.MultiProblem(mat, M.FilmDomain.from_cli(1e-7, 1e-7, 100), 20000, 10**6)
    pore = M.MultiProblem(mat, M.PoreCellDomain(5e-7, 2.5e-7), 6000, 10**6)
    kw_film = dict(dt=0.5e-12, nsteps=400, precision=64, steps_per_launch=50, seed=5)
    first = _check(film, 1e-12, **kw_film)
    _check(pore, 1e-10, dt=0.5e-12, nsteps=300, precision=32, steps_per_launch=30, seed=9)
    again = _check(film, 1e-12, **kw_film)
    assert _field_err(first, again) < 1e-12


def test_noalloc_rejects_problems_above_the_scratch_size():
    mat = M.Material.silicon(300.0)
    nemit = SCRATCH_BYTES // 48 + 1000  # 48 B of state per phonon in FP32 flight
    P = M.MultiProblem(mat, M.FilmDomain.from_cli(1e-7, 1e-7, 100), nemit, 10**6)
    rc, _, _ = _call(_lib.lib().mc_solve_noalloc, P, dt=0.5e-12, nsteps=10, precision=32)
    assert rc == -1  # MC_ERR_ARG
    assert b"MC_NOALLOC_SCRATCH_BYTES" in _lib.lib().mc_last_error()
    # the array is still usable after a refusal
    small = M.MultiProblem(mat, M.FilmDomain.from_cli(1e-7, 1e-7, 100), 5000, 10**6)
    _check(small, 1e-10, dt=0.5e-12, nsteps=200, precision=32, steps_per_launch=200, seed=3)


def _free_bytes():
    import torch
    return torch.cuda.mem_get_info(0)[0]  # cudaMemGetInfo on the primary context the library uses


def test_noalloc_calls_leave_free_device_memory_unchanged():
    """No device allocation: after a warm-up call of each problem (module
    loading, the scratch array's first touch), repeated calls leave the
    free device memory exactly as it was."""
    mat = M.Material.silicon(300.0)
    film = M.MultiProblem(mat, M.FilmDomain.from_cli(1e-7, 1e-7, 100), 20000, 10**6)
    pore = M.MultiProblem(mat, M.PoreCellDomain(5e-7, 2.5e-7), 6000, 10**6)
    calls = [(film, dict(dt=0.5e-12, nsteps=200, precision=64, steps_per_launch=50, seed=5)),
             (pore, dict(dt=0.5e-12, nsteps=150, precision=32, steps_per_launch=30, seed=9))]
    L = _lib.lib()
    for P, kw in calls:
        _lib.check(_call(L.mc_solve_noalloc, P, **kw)[0])
    before = _free_bytes()
    for _ in range(3):
        for P, kw in calls:
            _lib.check(_call(L.mc_solve_noalloc, P, **kw)[0])
    assert _free_bytes() == before


def test_noalloc_validates_the_schedule_as_mc_solve_does():
    mat = M.Material.silicon(300.0)
    P = M.MultiProblem(mat, M.FilmDomain.from_cli(1e-7, 1e-7, 20), 2000, 10**6)
    L = _lib.lib()
    for fn in (L.mc_solve, L.mc_solve_noalloc):
        rc, _, _ = _call(fn, P, dt=0.5e-12, nsteps=20, precision=32, schedule=7)
        assert rc == -1  # MC_ERR_ARG
