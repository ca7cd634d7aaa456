"""Materials of many temperatures built on the GPU in one launch
(mc_material_create_many) against the host build (mc_material_create), one
temperature at a time: every table -- velocities, relaxation times, the
inverse-CDF thresholds of the scattering and flux distributions -- and
every sum (energy, flux, scattering, bulk conductivity) identical bit for
bit; and a solve with a device-built material equal to one with the host's."""

import time

import numpy as np
import pytest

import montecarlocpp_gb300 as M

pytestmark = pytest.mark.gpu


def test_device_build_equals_host_build_bit_for_bit():
    Ts = np.concatenate([np.linspace(100.0, 400.0, 61), [1.0, 4.2, 77.0, 1000.0, 2000.0]])
    t0 = time.perf_counter()
    many = M.Material.many(Ts)
    t_dev = time.perf_counter() - t0
    t0 = time.perf_counter()
    host = [M.Material.silicon(T) for T in Ts]
    t_host = time.perf_counter() - t0
    print(f"materials: {len(Ts)} temperatures, device build {t_dev * 1e3:.2f} ms, host build {t_host * 1e3:.2f} ms")
    for a, b in zip(many, host):
        va, ta = a.tables()
        vb, tb = b.tables()
        assert np.array_equal(va, vb) and np.array_equal(ta, tb), a.T
        assert np.array_equal(a._sums, b._sums), a.T
        for x, y in zip(a.thresholds(), b.thresholds()):
            assert np.array_equal(x, y), a.T


def test_solve_with_device_built_material():
    dom = M.FilmDomain.from_cli(1e-7, 1e-7, 50)
    (dev,) = M.Material.many([237.5])
    host = M.Material.silicon(237.5)
    kw = dict(dt=0.5e-12, nsteps=300, precision=64, steps_per_launch=100, seed=2)
    a = M.MultiProblem(dev, dom, 20000, 10**6).solve(**kw)
    b = M.MultiProblem(host, dom, 20000, 10**6).solve(**kw)
    assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()


def test_device_build_refuses_invalid_temperatures():
    with pytest.raises(M._lib.McError):
        M.Material.many([300.0, -1.0])
