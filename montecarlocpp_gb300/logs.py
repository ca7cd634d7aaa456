"""Comparison of per-phonon event logs (the replay/trajectory logs of
mc_problem_desc.log): where two runs of the same phonons first part ways.

A log holds, per phonon, records of 12 values: loop index, subdomain before,
face hit (-1 scatter, -2 horizon, -3 escape), subdomain after, cell, x, y, z,
time, nscat, w, p. Two trajectories agree while every discrete field (loop
index, subdomains, face, cell, nscat, w, p) agrees record by record; the
divergence time is the time of the first record where they do not (or of the
first record one run has and the other lacks).
"""

from __future__ import annotations

import numpy as np

DISCRETE = [0, 1, 2, 3, 4, 9, 10, 11]
TIME = 8


def divergence_times(a, b):
    """Per phonon, the time at which the trajectories of logs `a` and `b`
    (each (records, counts)) first differ in a discrete field, or inf if they
    never do within the records both kept. Returns a float array."""
    (ra, ca), (rb, cb) = a, b
    n = min(len(ca), len(cb))
    cap = min(ra.shape[1], rb.shape[1])
    out = np.full(n, np.inf)
    for i in range(n):
        ka, kb = int(min(ca[i], cap)), int(min(cb[i], cap))
        k = min(ka, kb)
        x, y = ra[i, :k][:, DISCRETE], rb[i, :k][:, DISCRETE]
        diff = np.flatnonzero((x != y).any(axis=1))
        if diff.size:
            j = int(diff[0])
            out[i] = min(ra[i, j, TIME], rb[i, j, TIME])
        elif ka != kb:
            j = k  # the first record only one of them has
            out[i] = ra[i, j, TIME] if ka > kb else rb[i, j, TIME]
    return out


def mismatch_rate(tdiv, horizons):
    """Fraction of trajectories that diverged at or before each horizon
    time."""
    tdiv = np.asarray(tdiv)
    return [float(np.mean(tdiv <= h)) for h in horizons]
