"""Material input files for the phonon Monte Carlo solver.

montecarlocpp reads a dispersion file and a relaxation-time file
(montecarlo/material.cpp:158-186; the names Si_disp.txt / Si_relax2.txt are
opened at montecarlo/main.cpp:269-273) but does not ship them. This module
writes files of exactly that format from an analytic silicon-like model:

* dispersion file: first line ``nw np``; then nw rows of
  ``omega domega (v_p dos_p) x np`` (montecarlo/material.cpp:162-179);
* relaxation file: np rows of 8 coefficients, two Matthiessen terms
  ``c0 c1 c2 c3`` each giving ``c0 * omega^c1 * T^c2 * exp(-c3 / T)``
  (montecarlo/material.cpp:185-204).

The model: isotropic branches omega(k) = v_s k + c k^2 for k <= k_max, LA
(v_s = 9010 m/s, c = -2.0e-7 m^2/s) and two TA (v_s = 5230 m/s,
c = -2.26e-7 m^2/s), k_max = 1.157e10 1/m; nw frequency bins centred on
(i + 1/2) * omega_max / nw (never omega = 0, which would make tau infinite);
group velocity v = v_s + 2 c k and density of states k^2 / (2 pi^2 v);
bins above a branch's maximum frequency get zero density of states.
Scattering: tau^-1 = A omega^4 + B omega^2 T exp(-C / T) with
A = 1.32e-45 s^3, B = 1.73e-19 s/K, C = 137.3 K.
"""

from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

__all__ = ["Branch", "SiliconModel", "silicon_tables", "write_material_files"]


@dataclass(frozen=True)
class Branch:
    vs: float  # sound velocity, m/s
    c: float  # quadratic coefficient, m^2/s

    def omega_max(self, kmax: float) -> float:
        return self.vs * kmax + self.c * kmax * kmax


@dataclass(frozen=True)
class SiliconModel:
    branches: tuple = field(default_factory=lambda: (
        Branch(9010.0, -2.0e-7), Branch(5230.0, -2.26e-7), Branch(5230.0, -2.26e-7)))
    kmax: float = 1.157e10
    nw: int = 1000
    A: float = 1.32e-45
    B: float = 1.73e-19
    C: float = 137.3


_DEFAULT_TABLES = None


def silicon_tables(model: SiliconModel | None = None):
    """Return (disp, relax): disp is nw x (2 + 2 np), relax is np x 8 (fresh
    arrays; the default model's are built once)."""
    global _DEFAULT_TABLES
    if model is None:
        if _DEFAULT_TABLES is None:
            _DEFAULT_TABLES = _silicon_tables(SiliconModel())
        return tuple(x.copy() for x in _DEFAULT_TABLES)
    return _silicon_tables(model)


def _silicon_tables(m: SiliconModel):
    np_ = len(m.branches)
    wmax = max(b.omega_max(m.kmax) for b in m.branches)
    dw = wmax / m.nw
    disp = np.zeros((m.nw, 2 + 2 * np_), dtype=np.float64)
    for i in range(m.nw):
        w = (i + 0.5) * dw
        disp[i, 0] = w
        disp[i, 1] = dw
        for p, b in enumerate(m.branches):
            wb = b.omega_max(m.kmax)
            disc = b.vs * b.vs + 4.0 * b.c * w
            if w < wb and disc > 0.0:
                v = math.sqrt(disc)
                k = 2.0 * w / (b.vs + v)  # smaller root of c k^2 + vs k - w
                v = b.vs + 2.0 * b.c * k
                dos = k * k / (2.0 * math.pi * math.pi * v)
            else:
                v = b.vs + 2.0 * b.c * m.kmax
                dos = 0.0
            disp[i, 2 + 2 * p] = v
            disp[i, 3 + 2 * p] = dos
    relax = np.tile(np.array([m.A, 4.0, 0.0, 0.0, m.B, 2.0, 1.0, m.C]), (np_, 1))
    return disp, relax


def write_material_files(directory: str, model: SiliconModel | None = None,
                         disp_name: str = "Si_disp.txt",
                         relax_name: str = "Si_relax2.txt"):
    """Write the two files in the reference's format; return their paths."""
    disp, relax = silicon_tables(model)
    os.makedirs(directory, exist_ok=True)
    dpath = os.path.join(directory, disp_name)
    rpath = os.path.join(directory, relax_name)
    with open(dpath, "w") as f:
        f.write(f"{disp.shape[0]} {(disp.shape[1] - 2) // 2}\n")
        for row in disp:
            f.write(" ".join(repr(float(x)) for x in row) + "\n")
    with open(rpath, "w") as f:
        for row in relax:
            f.write(" ".join(repr(float(x)) for x in row) + "\n")
    return dpath, rpath


def read_material_files(disp_path: str, relax_path: str):
    """Parse the two files (montecarlo/material.cpp:158-186 formats)."""
    with open(disp_path) as f:
        vals = f.read().split()
    nw, np_ = int(vals[0]), int(vals[1])
    if nw <= 0 or np_ <= 0:
        raise ValueError("Invalid dispersion file")
    ncol = 2 + 2 * np_
    data = np.array([float(x) for x in vals[2:2 + nw * ncol]], dtype=np.float64)
    if data.size != nw * ncol:
        raise ValueError("Array extraction failed")
    with open(relax_path) as f:
        rv = np.array([float(x) for x in f.read().split()], dtype=np.float64)
    if rv.size < 8 * np_:
        raise ValueError("Array extraction failed")
    return data.reshape(nw, ncol), rv[:8 * np_].reshape(np_, 8)
