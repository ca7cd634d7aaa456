"""Seeded synthetic workloads of the benchmark configurations.

* batched films: 64 in-plane films (FilmDomain, montecarlo/domain.cpp:188-199)
  with thickness log-uniform in [10 nm, 10 um], equilibrium temperature
  uniform in [100, 400] K, phonon count proportional to thickness from 1e4
  to 1e6, 100 cells across the thickness;
* served requests: a Poisson stream of solves, each the in-plane film or the
  periodic pore cell, size log-uniform in [20 nm, 2 um], temperature uniform
  in [100, 400] K, phonon count log-uniform in [1e4, 1e7].
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass
class FilmSpec:
    thickness: float
    T: float
    nemit: int
    cells: int = 100


def batched_films(seed: int = 0, n: int = 64, tmin=1e-8, tmax=1e-5, nmin=10_000, nmax=1_000_000):
    rng = np.random.default_rng(seed)
    th = np.exp(rng.uniform(math.log(tmin), math.log(tmax), n))
    T = rng.uniform(100.0, 400.0, n)
    # phonon count proportional to thickness, mapped onto [nmin, nmax]
    N = nmin + (th - tmin) / (tmax - tmin) * (nmax - nmin)
    return [FilmSpec(float(t), float(tt), int(round(k))) for t, tt, k in zip(th, T, N)]


@dataclass
class Request:
    t_arrival: float
    geometry: str        # "film" or "pore"
    size: float          # film thickness or pore cell side, m
    T: float
    nemit: int           # phonons per round


def served_requests(seed: int = 0, rate: float = 200.0, duration: float = 60.0, nmin=10_000,
                    nmax=10_000_000, smin=2e-8, smax=2e-6):
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        geo = "film" if rng.random() < 0.5 else "pore"
        size = float(np.exp(rng.uniform(math.log(smin), math.log(smax))))
        T = float(rng.uniform(100.0, 400.0))
        N = int(np.exp(rng.uniform(math.log(nmin), math.log(nmax))))
        out.append(Request(t, geo, size, T, N))
    return out
