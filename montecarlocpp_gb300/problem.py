"""Host-side mirror of montecarlocpp's Material / Problem API over the C ABI.

``Material(disp, relax, T)`` mirrors montecarlo/material.h:51-67;
``TempProblem`` / ``FluxProblem`` / ``MultiProblem(mat, dom, nemit, maxscat,
maxloop=0)`` mirror montecarlo/problem.h:157-203, and their ``solve()``
replaces ``FieldProblem::solve`` (montecarlo/problem.cpp:370-445) for all
phonons at once on the GPU. Results are rows x cols numpy arrays with the
reference's row meaning: Temp (1 row), Flux (3 rows x, y, z), Multi (4 rows:
temperature then flux).
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from .domains import Domain
from .materials import silicon_tables

TEMP, FLUX, MULTI, CUMTEMP, CUMFLUX = 0, 1, 2, 3, 4
TALLY_AUTO, TALLY_SHARED, TALLY_GLOBAL = -1, 0, 1


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Material:
    """Material(disp, relax, T): dispersion + relaxation files, temperature."""

    def __init__(self, disp=None, relax=None, T=300.0, *, tables=None):
        L = _lib.lib()
        h = C.c_void_p()
        if tables is not None:
            d, r = (np.ascontiguousarray(x, dtype=np.float64) for x in tables)
            _lib.check(L.mc_material_create(_dp(d), d.shape[0], (d.shape[1] - 2) // 2, _dp(r), float(T),
                                            C.byref(h)))
            self.nw, self.np = d.shape[0], (d.shape[1] - 2) // 2
        else:
            if not (os.path.exists(disp) and os.path.exists(relax)):
                raise FileNotFoundError("Error opening dispersion or relaxation time file")
            _lib.check(L.mc_material_load(disp.encode(), relax.encode(), float(T), C.byref(h)))
            with open(disp) as f:
                nw, np_ = f.readline().split()[:2]
            self.nw, self.np = int(nw), int(np_)
        self.h = h
        self.T = float(T)
        self._sums = np.zeros(4)
        _lib.check(L.mc_material_sums(self.h, _dp(self._sums)))

    @classmethod
    def silicon(cls, T=300.0, model=None):
        return cls(T=T, tables=silicon_tables(model))

    @classmethod
    def many(cls, temperatures, tables=None):
        """Material(disp, relax, T) for every T of `temperatures`, the
        temperature-dependent tables built on the GPU in one launch
        (mc_material_create_many); each equals Material(T=T, tables=...)
        bit for bit. tables: (disp, relax), default the silicon model."""
        d, r = (np.ascontiguousarray(x, dtype=np.float64) for x in (tables or silicon_tables()))
        Ts = np.ascontiguousarray(temperatures, dtype=np.float64)
        hs = (C.c_void_p * len(Ts))()
        _lib.check(_lib.lib().mc_material_create_many(_dp(d), d.shape[0], (d.shape[1] - 2) // 2, _dp(r), _dp(Ts),
                                                      len(Ts), hs))
        out = []
        for h, T in zip(hs, Ts):
            m = cls.__new__(cls)
            m.h = C.c_void_p(h)
            m.nw, m.np = d.shape[0], (d.shape[1] - 2) // 2
            m.T = float(T)
            m._sums = np.zeros(4)
            _lib.check(_lib.lib().mc_material_sums(m.h, _dp(m._sums)))
            out.append(m)
        return out

    def thresholds(self):
        """Inverse-CDF thresholds (scattering bins, scattering branches, flux
        bins, flux branches) as uint64 arrays."""
        sw = np.zeros(self.nw, dtype=np.uint64)
        sp = np.zeros((self.nw, self.np), dtype=np.uint64)
        fw = np.zeros(self.nw, dtype=np.uint64)
        fp = np.zeros((self.nw, self.np), dtype=np.uint64)
        u = lambda a: a.ctypes.data_as(C.POINTER(C.c_uint64))
        _lib.check(_lib.lib().mc_material_thresholds(self.h, u(sw), u(sp), u(fw), u(fp)))
        return sw, sp, fw, fp

    def temp(self):
        return self.T

    def cond(self):
        return float(self._sums[3])

    def energySum(self):
        return float(self._sums[0])

    def fluxSum(self):
        return float(self._sums[1])

    def scatSum(self):
        return float(self._sums[2])

    def tables(self):
        vel = np.zeros((self.nw, self.np))
        tau = np.zeros((self.nw, self.np))
        _lib.check(_lib.lib().mc_material_tables(self.h, _dp(vel), _dp(tau)))
        return vel, tau

    def __del__(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.mc_material_destroy(self.h)
            self.h = None


def domain_descs(dom: Domain):
    """The C-ABI descriptions of a domain: one mc_sdom_desc per subdomain
    (any shape) and the pair list."""
    n = len(dom.ppeds)
    ps = (_lib.SdomDesc * n)()
    for i, p in enumerate(dom.ppeds):
        cols = p.columns()
        ps[i].shape = int(p.shape_kind)
        ps[i].ncols = int(cols.shape[1])
        ps[i].o[:] = [float(x) for x in p.o]
        ps[i].mat[:cols.size] = [float(x) for x in cols.reshape(-1, order="F")]
        ps[i].div[:] = [int(x) for x in p.divisions()]
        ps[i].gradT[:] = [float(x) for x in p.gradT]
        ps[i].kind[:len(p.kinds)] = [int(k) for k in p.kinds]
        ps[i].T[:len(p.T)] = [float(t) for t in p.T]
    m = len(dom.pairs)
    qs = (_lib.PairDesc * max(m, 1))()
    for i, q in enumerate(dom.pairs):
        qs[i].kind, qs[i].sdom1, qs[i].face1, qs[i].sdom2, qs[i].face2 = q.kind, q.s1, q.f1, q.s2, q.f2
        qs[i].transl[:] = [float(x) for x in q.transl]
        qs[i].rot[:] = [float(x) for x in np.asarray(q.rot, dtype=np.float64).reshape(-1)]
    return ps, n, qs, m


class DomainHandle:
    """The library's image of a Domain description."""

    def __init__(self, dom: Domain):
        L = _lib.lib()
        ps, n, qs, m = domain_descs(dom)
        h = C.c_void_p()
        _lib.check(L.mc_domain_create_shapes(ps, n, qs, m, C.byref(h)))
        self.h = h
        self.dom = dom
        self.cols = L.mc_domain_cols(h)

    def cell_volumes(self):
        out = np.zeros(self.cols)
        _lib.check(_lib.lib().mc_domain_cell_volumes(self.h, _dp(out)))
        return out

    def __del__(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.mc_domain_destroy(self.h)
            self.h = None


def _handle(dom):
    if isinstance(dom, DomainHandle):
        return dom
    h = getattr(dom, "_mc_handle", None)
    if h is None:
        h = DomainHandle(dom)
        dom._mc_handle = h
    return h


class FieldProblem:
    """Common part of the field problems (montecarlo/problem.h:121-147)."""

    kind = MULTI
    loopFactor = 100  # montecarlo/problem.h:124
    size = 0          # CumTemp / CumFlux bins after the first

    def __init__(self, mat: Material, dom, nemit: int, maxscat: int, maxloop: int = 0):
        if nemit <= 0 or maxscat <= 0 or maxloop < 0:
            raise ValueError("Invalid problem arguments")
        self.mat, self.dom = mat, dom
        self.handle = _handle(dom)
        self.nemit_requested, self.maxscat = int(nemit), int(maxscat)
        self.maxloop = int(maxloop) if maxloop else self.loopFactor * int(maxscat)
        self.stats = None

    def rows(self):
        return {TEMP: 1, FLUX: 3, MULTI: 4, CUMTEMP: self.size + 1, CUMFLUX: 3 * (self.size + 1)}[self.kind]

    def desc(self, *, dt, nsteps, seed=0, precision=32, steps_per_launch=0, block_size=0,
             grid_blocks=0, tally_mode=TALLY_AUTO, replay=None, log_cap=0, log_phonons=0, stream=None,
             schedule=0, compact_interval=0):
        d = _lib.ProblemDesc()
        d.problem, d.nemit, d.maxscat, d.maxloop = self.kind, self.nemit_requested, self.maxscat, self.maxloop
        d.dt, d.nsteps, d.precision, d.seed = float(dt), int(nsteps), int(precision), int(seed)
        d.steps_per_launch = int(steps_per_launch) if steps_per_launch else int(nsteps)
        d.block_size, d.grid_blocks, d.tally_mode = int(block_size), int(grid_blocks), int(tally_mode)
        keep = []
        if replay is not None:
            words, offsets = replay
            words = np.ascontiguousarray(words, dtype=np.uint32)
            offsets = np.ascontiguousarray(offsets, dtype=np.int64)
            keep += [words, offsets]
            d.replay_words = words.ctypes.data_as(C.POINTER(C.c_uint32))
            d.replay_offsets = offsets.ctypes.data_as(C.POINTER(C.c_int64))
        log = None
        if log_cap:
            log = np.zeros((log_phonons, log_cap, 12))
            counts = np.zeros(log_phonons, dtype=np.int64)
            keep += [log, counts]
            d.log = _dp(log)
            d.log_counts = counts.ctypes.data_as(C.POINTER(C.c_int64))
            d.log_cap, d.log_phonons = int(log_cap), int(log_phonons)
            log = (log, counts)
        d.stream = stream
        d.schedule, d.compact_interval = int(schedule), int(compact_interval)
        d.cum_size = int(self.size)
        return d, keep, log

    def solve(self, *, dt, nsteps, seed=0, precision=32, steps_per_launch=0, block_size=0,
              grid_blocks=0, tally_mode=TALLY_AUTO, replay=None, log_cap=0, log_phonons=0, schedule=0,
              compact_interval=0):
        """Run every phonon on the GPU; returns the rows x cols field
        (power * postProc(tally) / cellVol, montecarlo/problem.cpp:439-444).
        With log_cap, ``self.log`` holds (records, counts)."""
        d, keep, log = self.desc(dt=dt, nsteps=nsteps, seed=seed, precision=precision,
                                 steps_per_launch=steps_per_launch, block_size=block_size,
                                 grid_blocks=grid_blocks, tally_mode=tally_mode, replay=replay,
                                 log_cap=log_cap, log_phonons=log_phonons, schedule=schedule,
                                 compact_interval=compact_interval)
        out = np.zeros(self.rows() * self.handle.cols)
        st = _lib.Stats()
        _lib.check(_lib.lib().mc_solve(self.mat.h, self.handle.h, C.byref(d), _dp(out), C.byref(st)))
        self.stats = st.as_dict()
        if log is not None:
            n = min(len(log[1]), st.nemit)
            self.log = (log[0][:n], log[1][:n])
        del keep
        return out.reshape(self.rows(), self.handle.cols, order="F")

    def solve_replicas(self, nsim, *, dt, nsteps, seed=0, precision=32, steps_per_launch=0, schedule=0):
        """solveField(prob, nsim) + calcStats (montecarlo/main.cpp:181-210):
        nsim solves with seeds seed, seed + 1, ...; returns the cell-by-cell
        mean and sample standard deviation (rows x cols each)."""
        d, keep, _ = self.desc(dt=dt, nsteps=nsteps, seed=seed, precision=precision,
                               steps_per_launch=steps_per_launch, schedule=schedule)
        n = self.rows() * self.handle.cols
        mean, sd = np.zeros(n), np.zeros(n)
        st = _lib.Stats()
        _lib.check(_lib.lib().mc_solve_replicas(self.mat.h, self.handle.h, C.byref(d), int(nsim), _dp(mean), _dp(sd),
                                                C.byref(st)))
        self.stats = st.as_dict()
        del keep
        shape = (self.rows(), self.handle.cols)
        return mean.reshape(shape, order="F"), sd.reshape(shape, order="F")

    def session(self, **kw):
        return Session(self, **kw)


class TempProblem(FieldProblem):
    kind = TEMP


class FluxProblem(FieldProblem):
    kind = FLUX


class MultiProblem(FieldProblem):
    kind = MULTI


class _CumProblem(FieldProblem):
    """CumTempProblem / CumFluxProblem(mat, dom, nemit, size, maxscat,
    maxloop=0) (montecarlo/problem.h:205-239): the field binned by the
    scatter count before each flight into size + 1 bins of
    ceil((maxscat - 1) / size) scatters, returned as cumulative sums over the
    bins (the last bin holds the Temp / Flux field)."""

    def __init__(self, mat: Material, dom, nemit: int, size: int, maxscat: int, maxloop: int = 0):
        if size < 1 or maxscat < 2:
            raise ValueError("Invalid problem arguments")
        super().__init__(mat, dom, nemit, maxscat, maxloop)
        self.size = int(size)

    def step(self):
        return -(-(self.maxscat - 1) // self.size)


class CumTempProblem(_CumProblem):
    kind = CUMTEMP


class CumFluxProblem(_CumProblem):
    kind = CUMFLUX


class Session:
    """Device-resident run: emit once, advance in windows, read back."""

    def __init__(self, prob: FieldProblem, **kw):
        self.prob = prob
        d, self._keep, self._log = prob.desc(**kw)
        self.desc = d
        h = C.c_void_p()
        _lib.check(_lib.lib().mc_session_create(prob.mat.h, prob.handle.h, C.byref(d), C.byref(h)))
        self.h = h

    def emit(self):
        _lib.check(_lib.lib().mc_session_emit(self.h))

    def advance(self, nlaunch: int) -> bool:
        done = C.c_int(0)
        _lib.check(_lib.lib().mc_session_advance(self.h, int(nlaunch), C.byref(done)))
        return bool(done.value)

    def run(self):
        self.emit()
        while not self.advance(1 << 20):
            pass

    def result(self, field=True):
        st = _lib.Stats()
        out = np.zeros(self.prob.rows() * self.prob.handle.cols) if field else None
        _lib.check(_lib.lib().mc_session_result(self.h, _dp(out) if field else None, C.byref(st)))
        r = out.reshape(self.prob.rows(), self.prob.handle.cols, order="F") if field else None
        return r, st.as_dict()

    def state_bytes(self):
        return _lib.lib().mc_session_state_bytes(self.h)

    def snapshot(self) -> bytearray:
        """Everything the session needs to continue, as host bytes."""
        n = _lib.lib().mc_session_snapshot_bytes(self.h)
        buf = bytearray(n)
        cbuf = (C.c_char * n).from_buffer(buf)
        _lib.check(_lib.lib().mc_session_snapshot(self.h, cbuf, n))
        return buf

    def restore(self, buf):
        """Load a snapshot of a session of the same problem; advance()
        then continues it exactly."""
        b = bytearray(buf)
        cbuf = (C.c_char * len(b)).from_buffer(b)
        _lib.check(_lib.lib().mc_session_restore(self.h, cbuf, len(b)))

    def close(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.mc_session_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def kappa_from_flux(field: np.ndarray, dom, axis: int = 0, flux_row0: int = 0) -> float:
    """kappa = -<q_axis> / gradT_axis, volume-weighted over the cells."""
    vols = _handle(dom).cell_volumes()
    q = float(np.sum(field[flux_row0 + axis] * vols) / np.sum(vols))
    g = float(dom.ppeds[0].gradT[axis])
    return -q / g
