"""ctypes wrapper of the CPU oracle (oracle/_build/libmc_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product package. Parity of the
oracle against the original montecarlocpp binary is unpinned (see
mc_oracle.h); it is pinned by known answers in tests/test_oracle.py.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmc_oracle.so")

TEMP, FLUX, MULTI, CUMTEMP, CUMFLUX = 0, 1, 2, 3, 4
RNG_MT, RNG_PHILOX, RNG_REPLAY = 0, 1, 2
LOG_FIELDS = ("loop", "sdom", "face", "sdom_after", "cell", "x", "y", "z",
              "time", "nscat", "w", "p")


class Pped(C.Structure):
    _fields_ = [("o", C.c_double * 3), ("M", C.c_double * 9), ("div", C.c_long * 3),
                ("gradT", C.c_double * 3), ("kind", C.c_int * 6), ("T", C.c_double * 6)]


class SdomS(C.Structure):
    _fields_ = [("shape", C.c_int), ("ncols", C.c_int), ("o", C.c_double * 3), ("mat", C.c_double * 27),
                ("div", C.c_long * 3), ("gradT", C.c_double * 3), ("kind", C.c_int * 11), ("T", C.c_double * 11)]


class PairS(C.Structure):
    _fields_ = [("kind", C.c_int), ("sdom1", C.c_int), ("face1", C.c_int),
                ("sdom2", C.c_int), ("face2", C.c_int), ("transl", C.c_double * 3),
                ("rot", C.c_double * 9)]


class Problem(C.Structure):
    _fields_ = [("problem", C.c_int), ("nemit", C.c_long), ("maxscat", C.c_long),
                ("maxloop", C.c_long), ("dt", C.c_double), ("horizon", C.c_double),
                ("rng", C.c_int), ("seed", C.c_uint64), ("nchunk", C.c_int),
                ("nthreads", C.c_int),
                ("replay_words", C.POINTER(C.c_uint32)), ("replay_offsets", C.POINTER(C.c_int64)),
                ("record_words", C.POINTER(C.c_uint32)), ("record_counts", C.POINTER(C.c_int64)),
                ("record_cap", C.c_long),
                ("log", C.POINTER(C.c_double)), ("log_counts", C.POINTER(C.c_int64)),
                ("log_cap", C.c_long), ("log_phonons", C.c_long), ("cum_size", C.c_long)]


class Stats(C.Structure):
    _fields_ = [("nemit", C.c_long), ("power", C.c_double), ("rows", C.c_long),
                ("cols", C.c_long), ("phonon_steps", C.c_double), ("events", C.c_long),
                ("scatters", C.c_long), ("escapes", C.c_long), ("horizon_stops", C.c_long),
                ("maxscat_stops", C.c_long), ("absorbed", C.c_long),
                ("replay_exhausted", C.c_long), ("seconds", C.c_double), ("threads", C.c_long)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, OpenMP)."""
    src = os.path.join(HERE, "mc_oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        L.orc_material_load.restype = C.c_void_p
        L.orc_material_load.argtypes = [C.c_char_p, C.c_char_p, C.c_double]
        L.orc_material_from_tables.restype = C.c_void_p
        L.orc_material_from_tables.argtypes = [P(C.c_double), C.c_long, C.c_long, P(C.c_double), C.c_double]
        L.orc_material_free.argtypes = [C.c_void_p]
        L.orc_material_sums.argtypes = [C.c_void_p, P(C.c_double)]
        L.orc_material_draw.argtypes = [C.c_void_p, C.c_int, C.c_uint32, C.c_uint32, P(C.c_long), P(C.c_long)]
        L.orc_material_tables.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double)]
        L.orc_domain_create.restype = C.c_void_p
        L.orc_domain_create.argtypes = [P(Pped), C.c_int, P(PairS), C.c_int]
        L.orc_domain_create_shapes.restype = C.c_void_p
        L.orc_domain_create_shapes.argtypes = [P(SdomS), C.c_int, P(PairS), C.c_int]
        L.orc_domain_cell_volumes.argtypes = [C.c_void_p, P(C.c_double)]
        L.orc_domain_sdom_volume.restype = C.c_double
        L.orc_domain_sdom_volume.argtypes = [C.c_void_p, C.c_int]
        L.orc_domain_emitters.restype = C.c_long
        L.orc_domain_emitters.argtypes = [C.c_void_p, P(C.c_double), P(C.c_int), P(C.c_int)]
        L.orc_domain_draw_positions.argtypes = [C.c_void_p, C.c_long, C.c_uint64, C.c_long, P(C.c_double)]
        L.orc_domain_is_inside.restype = C.c_int
        L.orc_domain_is_inside.argtypes = [C.c_void_p, C.c_int, P(C.c_double)]
        L.orc_domain_film.restype = C.c_void_p
        L.orc_domain_film.argtypes = [C.c_double, C.c_double, C.c_double, C.c_long, C.c_double]
        L.orc_domain_bulk.restype = C.c_void_p
        L.orc_domain_bulk.argtypes = [C.c_double, C.c_long, C.c_double]
        L.orc_domain_free.argtypes = [C.c_void_p]
        L.orc_domain_cols.restype = C.c_long
        L.orc_domain_cols.argtypes = [C.c_void_p]
        L.orc_accumulate.argtypes = [C.c_void_p, C.c_int, P(C.c_double), P(C.c_double), P(C.c_double),
                                     C.c_long, P(C.c_double)]
        L.orc_solve.restype = C.c_int
        L.orc_solve.argtypes = [C.c_void_p, C.c_void_p, P(Problem), P(C.c_double), P(Stats)]
        L.orc_philox4x32_10.argtypes = [P(C.c_uint32), P(C.c_uint32), P(C.c_uint32)]
        L.orc_mt19937_nth.restype = C.c_uint32
        L.orc_mt19937_nth.argtypes = [C.c_uint32, C.c_long]
        L.orc_draw_iso.argtypes = [C.c_uint32, C.c_uint32, P(C.c_double)]
        L.orc_draw_aniso.argtypes = [C.c_uint32, C.c_uint32, C.c_int, P(C.c_double)]
        L.orc_rot_z_to.argtypes = [P(C.c_double), P(C.c_double)]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OMaterial:
    def __init__(self, disp=None, relax=None, T=300.0, paths=None):
        L = lib()
        if paths is not None:
            h = L.orc_material_load(paths[0].encode(), paths[1].encode(), T)
        else:
            disp = np.ascontiguousarray(disp, dtype=np.float64)
            relax = np.ascontiguousarray(relax, dtype=np.float64)
            self._keep = (disp, relax)
            h = L.orc_material_from_tables(_dp(disp), disp.shape[0], (disp.shape[1] - 2) // 2, _dp(relax), T)
        if not h:
            raise ValueError("oracle material construction failed")
        self.h = h
        self.T = T

    def sums(self):
        out = np.zeros(4)
        lib().orc_material_sums(self.h, _dp(out))
        return dict(energySum=out[0], fluxSum=out[1], scatSum=out[2], cond=out[3])

    def draw(self, which, x1, x2):
        w, p = C.c_long(), C.c_long()
        lib().orc_material_draw(self.h, which, x1, x2, C.byref(w), C.byref(p))
        return w.value, p.value

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_material_free(self.h)
            self.h = None


def domain_structs(dom):
    """Pack a montecarlocpp_gb300.domains.Domain description (subdomains of
    any shape) for orc_domain_create_shapes."""
    n = len(dom.ppeds)
    ps = (SdomS * n)()
    for i, p in enumerate(dom.ppeds):
        cols = np.asarray(p.columns(), dtype=np.float64)
        ps[i].shape = int(p.shape_kind)
        ps[i].ncols = int(cols.shape[1])
        ps[i].o[:] = [float(x) for x in p.o]
        ps[i].mat[:cols.size] = [float(x) for x in cols.reshape(-1, order="F")]
        ps[i].div[:] = [int(x) for x in p.divisions()]
        ps[i].gradT[:] = [float(x) for x in p.gradT]
        ps[i].kind[:len(p.kinds)] = [int(k) for k in p.kinds]
        ps[i].T[:len(p.T)] = [float(t) for t in p.T]
    m = len(dom.pairs)
    qs = (PairS * max(m, 1))()
    for i, q in enumerate(dom.pairs):
        qs[i].kind, qs[i].sdom1, qs[i].face1, qs[i].sdom2, qs[i].face2 = q.kind, q.s1, q.f1, q.s2, q.f2
        qs[i].transl[:] = [float(x) for x in q.transl]
        qs[i].rot[:] = [float(x) for x in np.asarray(q.rot).reshape(-1)]
    return ps, n, qs, m


class ODomain:
    def __init__(self, dom=None, handle=None):
        L = lib()
        if handle is not None:
            self.h = handle
        else:
            ps, n, qs, m = domain_structs(dom)
            self.h = L.orc_domain_create_shapes(ps, n, qs, m)
            if not self.h:
                raise ValueError("oracle domain construction failed")
        self.cols = L.orc_domain_cols(self.h)

    @classmethod
    def film(cls, Lx, Ly, Lz, divy, dT):
        return cls(handle=lib().orc_domain_film(Lx, Ly, Lz, divy, dT))

    @classmethod
    def bulk(cls, L, divx, dT):
        return cls(handle=lib().orc_domain_bulk(L, divx, dT))

    def cell_volumes(self):
        out = np.zeros(self.cols)
        lib().orc_domain_cell_volumes(self.h, _dp(out))
        return out

    def sdom_volume(self, s):
        return lib().orc_domain_sdom_volume(self.h, s)

    def emitters(self):
        n = lib().orc_domain_emitters(self.h, None, None, None)
        w = np.zeros(n)
        sd = (C.c_int * max(n, 1))()
        fc = (C.c_int * max(n, 1))()
        lib().orc_domain_emitters(self.h, _dp(w), sd, fc)
        return w, list(sd[:n]), list(fc[:n])

    def draw_positions(self, e, seed, n):
        out = np.zeros((n, 3))
        lib().orc_domain_draw_positions(self.h, e, seed, n, _dp(out))
        return out

    def is_inside(self, s, x):
        return bool(lib().orc_domain_is_inside(self.h, s, _dp(np.ascontiguousarray(x, dtype=np.float64))))

    def accumulate(self, sdom, bpos, epos, amount, data):
        amount = np.ascontiguousarray(amount, dtype=np.float64)
        buf = np.asfortranarray(data, dtype=np.float64).reshape(-1, order="F").copy()
        lib().orc_accumulate(self.h, sdom, _dp(np.asarray(bpos, dtype=np.float64)),
                             _dp(np.asarray(epos, dtype=np.float64)), _dp(amount), amount.size, _dp(buf))
        return buf.reshape(data.shape, order="F")

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_domain_free(self.h)
            self.h = None


def solve(mat, dom, problem=MULTI, nemit=1000, maxscat=1000, maxloop=0, dt=0.0,
          horizon=0.0, rng=RNG_PHILOX, seed=0, nchunk=1, nthreads=0,
          replay=None, record_cap=0, log_cap=0, log_phonons=0, size=0):
    """Run the oracle. Returns (out rows x cols, stats dict, extras).
    `size` is the bin count of CUMTEMP / CUMFLUX."""
    L = lib()
    P = Problem()
    P.problem, P.nemit, P.maxscat, P.maxloop = problem, nemit, maxscat, maxloop
    P.cum_size = size
    P.dt, P.horizon, P.rng, P.seed = dt, horizon, rng, seed
    P.nchunk, P.nthreads = nchunk, nthreads
    extras = {}
    # the problem's phonon count is only known after rounding; allocate for
    # nemit + number of emitters (each emitter rounds up by at most one)
    cap_n = nemit + 4096
    if replay is not None:
        words, offsets = replay
        words = np.ascontiguousarray(words, dtype=np.uint32)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        extras["_keep"] = (words, offsets)
        P.replay_words = words.ctypes.data_as(C.POINTER(C.c_uint32))
        P.replay_offsets = offsets.ctypes.data_as(C.POINTER(C.c_int64))
    if record_cap:
        rw = np.zeros((cap_n, record_cap), dtype=np.uint32)
        rc = np.zeros(cap_n, dtype=np.int64)
        P.record_words = rw.ctypes.data_as(C.POINTER(C.c_uint32))
        P.record_counts = rc.ctypes.data_as(C.POINTER(C.c_int64))
        P.record_cap = record_cap
    if log_cap:
        nlp = min(log_phonons, cap_n)
        lg = np.full((nlp, log_cap, 12), np.nan)
        lc = np.zeros(nlp, dtype=np.int64)
        P.log = _dp(lg)
        P.log_counts = lc.ctypes.data_as(C.POINTER(C.c_int64))
        P.log_cap, P.log_phonons = log_cap, nlp
    rows = {TEMP: 1, FLUX: 3, MULTI: 4, CUMTEMP: size + 1, CUMFLUX: 3 * (size + 1)}[problem]
    out = np.zeros(rows * dom.cols)
    st = Stats()
    rc_ = L.orc_solve(mat.h, dom.h, C.byref(P), _dp(out), C.byref(st))
    if rc_ != 0:
        raise RuntimeError(f"oracle solve failed ({rc_})")
    n = st.nemit
    if record_cap:
        if (rc[:n] > record_cap).any():
            raise RuntimeError("record capacity exceeded")
        extras["record"] = (rw[:n], rc[:n])
    if log_cap:
        extras["log"] = (lg[:min(nlp, n)], lc[:min(nlp, n)])
    return out.reshape(rows, dom.cols, order="F"), st.as_dict(), extras


def record_to_replay(record, pad=0, seed=12345):
    """Turn recorded per-phonon words into (flat words, offsets). `pad`
    extra words (a fixed pseudo-random sequence) follow each phonon's
    record, so that a replay whose trajectory parts from the recorded one
    (an FP32 rounding flips a discrete choice) can run on past it."""
    rw, rc = record
    rc = np.asarray(rc, dtype=np.int64)
    offsets = np.zeros(len(rc) + 1, dtype=np.int64)
    offsets[1:] = np.cumsum(rc + pad)
    extra = np.random.default_rng(seed).integers(0, 2**32, size=pad, dtype=np.uint64).astype(np.uint32)
    parts = []
    for i in range(len(rc)):
        parts.append(rw[i, :rc[i]])
        if pad:
            parts.append(extra)
    words = np.concatenate(parts) if parts else np.zeros(0, np.uint32)
    return words.astype(np.uint32), offsets


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return list(o)


def mt19937_nth(seed, n):
    return lib().orc_mt19937_nth(seed, n)


def draw_iso(x1, x2):
    o = np.zeros(3)
    lib().orc_draw_iso(x1, x2, _dp(o))
    return o


def draw_aniso(x1, x2, bidir):
    o = np.zeros(3)
    lib().orc_draw_aniso(x1, x2, int(bidir), _dp(o))
    return o


def rot_z_to(n):
    n = np.asarray(n, dtype=np.float64)
    R = np.zeros(9)
    lib().orc_rot_z_to(_dp(n), _dp(R))
    return R.reshape(3, 3)
