"""Batched solves: many (Material, Domain, problem) instances with uneven
phonon counts advanced to one time horizon in one persistent kernel launch
per window (mc_batch_* in include/mc_gb300.h), optionally replayed from a
captured CUDA graph.

Each instance keeps the reference's meaning (its own FieldProblem,
montecarlo/problem.h:121-203) and its own Philox key, so instance i of a
batch gives the same trajectories as the same problem solved alone.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .problem import FieldProblem, _dp


class Batch:
    """Batch(problems, dt, nsteps, seeds=None, precision=32, steps_per_launch=0,
    use_graph=True): `problems` are Temp/Flux/MultiProblem objects."""

    def __init__(self, problems, *, dt, nsteps, seeds=None, precision=32, steps_per_launch=0,
                 block_size=0, grid_blocks=0, use_graph=True, stream=None):
        self.problems = list(problems)
        n = len(self.problems)
        seeds = list(seeds) if seeds is not None else list(range(n))
        mats = (C.c_void_p * n)(*[p.mat.h.value for p in self.problems])
        doms = (C.c_void_p * n)(*[p.handle.h.value for p in self.problems])
        descs = (_lib.ProblemDesc * n)()
        for i, (p, s) in enumerate(zip(self.problems, seeds)):
            d, _, _ = p.desc(dt=dt, nsteps=nsteps, seed=s)
            descs[i] = d
        bd = _lib.BatchDesc(dt, nsteps, precision, steps_per_launch, block_size, grid_blocks, int(use_graph),
                            stream)
        h = C.c_void_p()
        _lib.check(_lib.lib().mc_batch_create(n, mats, doms, descs, C.byref(bd), C.byref(h)))
        self.h = h
        self.n = n

    def run(self):
        _lib.check(_lib.lib().mc_batch_run(self.h))

    def result(self, i):
        p: FieldProblem = self.problems[i]
        out = np.zeros(p.rows() * p.handle.cols)
        st = _lib.Stats()
        _lib.check(_lib.lib().mc_batch_result(self.h, i, _dp(out), C.byref(st)))
        return out.reshape(p.rows(), p.handle.cols, order="F"), st.as_dict()

    def stats(self):
        st = _lib.Stats()
        _lib.check(_lib.lib().mc_batch_stats(self.h, C.byref(st)))
        return st.as_dict()

    def state_bytes(self):
        return _lib.lib().mc_batch_state_bytes(self.h)

    def close(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.mc_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
