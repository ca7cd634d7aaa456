"""Serving: a request loop that runs many kappa solves at once on one GPU.

`Server` wraps mc_server_* (include/mc_gb300.h): the loop runs on a library
thread, admits submitted solves against an HBM budget (a free range of its
resident state buffer), and advances one window of every admitted solve per
tick in one persistent batched launch, so a request that arrives while
others run joins them at the next window.
Each round splits its phonons into batch-mean groups; a solve completes when
the standard error of kappa = -<q_axis>/gradT_axis is within the target.
The error estimate is the reference's replica statistics
(montecarlo/main.cpp:181-210, montecarlo/field.cpp:323-330) over groups
instead of whole repeated runs, pooled over rounds of unequal size: the
first round has the requested phonons, later ones the estimated remainder.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .problem import FLUX, MULTI, _dp, _handle


class Server:
    def __init__(self, *, dt, nsteps, precision=32, hbm_budget=8 << 30, max_active=256, groups=8,
                 target_rel_se=0.01, min_rounds=1, max_rounds=1000, block_size=0, steps_per_window=0):
        d = _lib.ServerDesc(dt, nsteps, precision, hbm_budget, max_active, groups, target_rel_se, min_rounds,
                            max_rounds, block_size, steps_per_window)
        h = C.c_void_p()
        _lib.check(_lib.lib().mc_server_create(C.byref(d), C.byref(h)))
        self.h = h
        self._keep = {}

    def submit(self, mat, dom, nemit, *, problem=FLUX, maxscat=10**6, maxloop=0, seed=0, axis=0, volume=0.0,
               gradient=0.0, field=True, max_rounds=0):
        """Queue a kappa solve with `nemit` phonons in its first round;
        field=False skips the per-cell field (kappa only); max_rounds > 0
        overrides the server's round limit for this request."""
        handle = _handle(dom)
        r = _lib.Request(mat.h.value, handle.h.value, problem, int(nemit), int(maxscat), int(maxloop), int(seed),
                         int(axis), float(volume), float(gradient), int(bool(field)), int(max_rounds))
        t = C.c_long()
        _lib.check(_lib.lib().mc_server_submit(self.h, C.byref(r), C.byref(t)))
        self._keep[t.value] = (mat, handle, problem, bool(field))
        return t.value

    def _result(self, ticket, rc, res, field):
        if rc < 0:
            _lib.check(rc)
        if rc == 0:
            return None
        out = res.as_dict()
        mat, handle, problem, keep_field = self._keep.pop(ticket)
        rows = 3 if problem == FLUX else 4
        out["field"] = field[: rows * handle.cols].reshape(rows, handle.cols, order="F").copy() if keep_field else None
        return out

    def cancel(self, ticket):
        """Cancel a request (queued: at once; running: at the next window
        boundary). True if it was cancelled, False if it had completed."""
        rc = _lib.lib().mc_server_cancel(self.h, int(ticket))
        if rc < 0:
            _lib.check(rc)
        return rc == 1

    def poll(self, ticket):
        res = _lib.Result()
        field = np.zeros(4 * self._keep[ticket][1].cols)
        rc = _lib.lib().mc_server_poll(self.h, ticket, C.byref(res), _dp(field))
        return self._result(ticket, rc, res, field)

    def wait(self, ticket, timeout=600.0):
        res = _lib.Result()
        field = np.zeros(4 * self._keep[ticket][1].cols)
        rc = _lib.lib().mc_server_wait(self.h, ticket, float(timeout), C.byref(res), _dp(field))
        return self._result(ticket, rc, res, field)

    def stats(self):
        st = _lib.ServerCounters()
        _lib.check(_lib.lib().mc_server_stats(self.h, C.byref(st)))
        return st.as_dict()

    def clock(self):
        return _lib.lib().mc_server_clock(self.h)

    def close(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.mc_server_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
