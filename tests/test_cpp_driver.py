"""The C++ driver (reference CLI grammar, C++ mirror of the reference API
over the C ABI): builds, fails loudly without a device, and on a GPU gives
the same field as the Python binding for the same seed."""

import os
import subprocess

import numpy as np
import pytest

import montecarlocpp_gb300 as M
from montecarlocpp_gb300 import build as B


def _run(tmp_path, *extra):
    M.write_material_files(str(tmp_path))
    B.build()
    cmd = [B.MAIN, str(tmp_path), "silicon", "300", "film", "1e-7", "1e-7", "10", "multi", "500", "1000000", "0",
           "1", "5e-13", "100", "64", "3", *extra]
    return subprocess.run(cmd, capture_output=True, text=True, timeout=300)


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="a CUDA device is present")
def test_driver_fails_loudly_without_device(tmp_path):
    r = _run(tmp_path)
    assert r.returncode == 1 and "no CUDA device" in r.stderr


def test_driver_rejects_bad_arguments(tmp_path):
    M.write_material_files(str(tmp_path))
    B.build()
    r = subprocess.run([B.MAIN, str(tmp_path), "silicon", "300", "torus", "1", "2"], capture_output=True, text=True)
    assert r.returncode == 1 and "Invalid domain" in r.stderr
    r = subprocess.run([B.MAIN, "/nonexistent/dir", "silicon", "300"], capture_output=True, text=True)
    assert r.returncode == 1 and "Invalid directory" in r.stderr


@pytest.mark.gpu
def test_driver_matches_python_binding(tmp_path, gmat):
    r = _run(tmp_path)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip() and not ln.startswith("Solution")]
    field = np.array([[float(x) for x in ln.split()] for ln in lines])
    dom = M.FilmDomain.from_cli(1e-7, 1e-7, 10)
    P = M.MultiProblem(gmat, dom, 500, 1000000)
    ref = P.solve(dt=5e-13, nsteps=100, precision=64, seed=3)
    assert field.shape == ref.shape
    assert np.allclose(field, ref, rtol=1e-8, atol=1e-8 * np.abs(ref).max())


@pytest.mark.gpu
def test_driver_cumflux_with_replicas(tmp_path, gmat):
    """`cumflux nemit size maxscat maxloop nsim` (montecarlo/main.cpp:
    446-456): the printed mean and standard deviation of the replicas match
    mc_solve_replicas for the same seeds."""
    M.write_material_files(str(tmp_path))
    B.build()
    cmd = [B.MAIN, str(tmp_path), "silicon", "300", "film", "1e-7", "1e-7", "10", "cumflux", "400", "2", "11", "0",
           "3", "5e-13", "80", "64", "5"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    text = r.stdout.split("Mean\n")[1]
    mean_txt, sd_txt = text.split("Standard Deviation\n")
    parse = lambda t: np.array([[float(x) for x in ln.split()] for ln in t.splitlines() if ln.strip()])
    mean, sd = parse(mean_txt), parse(sd_txt)
    P = M.CumFluxProblem(gmat, M.FilmDomain.from_cli(1e-7, 1e-7, 10), 400, 2, 11)
    rm, rs = P.solve_replicas(3, dt=5e-13, nsteps=80, precision=64, seed=5)
    assert mean.shape == rm.shape == (9, 10)
    assert np.allclose(mean, rm, rtol=1e-8, atol=1e-8 * np.abs(rm).max())
    assert np.allclose(sd, rs, rtol=1e-6, atol=1e-8 * np.abs(rs).max())


@pytest.mark.gpu
@pytest.mark.parametrize("args,dom", [
    (["pyr", "1e-7", "8e-8"], lambda: M.PyrDomain.from_cli(1e-7, 8e-8)),
    (["hex", "1e-7", "4e-8"], lambda: M.HexDomain.from_cli(1e-7, 4e-8)),
    (["jct", "5e-8", "4e-8"], lambda: M.JctDomain.from_cli(5e-8, 4e-8)),
    (["tee", "5e-8", "3e-8", "4"], lambda: M.TeeDomain.from_cli(5e-8, 3e-8, 4)),
    (["tube", "1e-7", "5e-8", "2e-8", "5", "3"], lambda: M.TubeDomain.from_cli(1e-7, 5e-8, 2e-8, 5, 3)),
    (["octet", "3e-7", "5e-8", "5e-8", "5e-9", "4", "3", "2", "2", "0.1"],
     lambda: M.OctetDomain((3e-7, 5e-8, 5e-8, 5e-9), (4, 3, 2, 2), 0.1)),
])
def test_driver_domains_match_python_binding(tmp_path, gmat, args, dom):
    """The reference's other CLI domains (montecarlo/main.cpp:320-374)
    through the C++ mirror give the Python binding's field."""
    M.write_material_files(str(tmp_path))
    B.build()
    cmd = [B.MAIN, str(tmp_path), "silicon", "300", *args, "multi", "400", "1000000", "0", "1", "5e-13", "100",
           "64", "4"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip() and not ln.startswith("Solution")]
    field = np.array([[float(x) for x in ln.split()] for ln in lines])
    P = M.MultiProblem(gmat, dom(), 400, 1000000)
    ref = P.solve(dt=5e-13, nsteps=100, precision=64, seed=4)
    assert field.shape == ref.shape
    assert np.allclose(field, ref, rtol=1e-8, atol=1e-8 * np.abs(ref).max())
