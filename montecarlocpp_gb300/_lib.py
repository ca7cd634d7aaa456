"""ctypes binding of the C ABI in include/mc_gb300.h (libmc_gb300.so).

The shared library is built in-tree by montecarlocpp_gb300/build.py. There is
no fallback: if the library is missing or no CUDA device is present, calls
raise.
"""

from __future__ import annotations

import ctypes as C
import os

from . import build as _build

MC_OK = 0
ERRORS = {
    -1: "invalid argument", -2: "CUDA error", -3: "no CUDA device", -4: "unsupported geometry",
    -5: "I/O error", -6: "replay stream exhausted", -7: "non-finite state", -8: "busy", -9: "device wait timeout",
    -10: "cancelled",
}
MC_ERR_ARG, MC_ERR_BUSY, MC_ERR_CANCELLED = -1, -8, -10


class PpedDesc(C.Structure):
    _fields_ = [("o", C.c_double * 3), ("M", C.c_double * 9), ("div", C.c_long * 3),
                ("gradT", C.c_double * 3), ("kind", C.c_int * 6), ("T", C.c_double * 6)]


MAX_SDOM_COLS, MAX_SDOM_FACES = 9, 11


class SdomDesc(C.Structure):
    _fields_ = [("shape", C.c_int), ("ncols", C.c_int), ("o", C.c_double * 3),
                ("mat", C.c_double * (3 * MAX_SDOM_COLS)), ("div", C.c_long * 3), ("gradT", C.c_double * 3),
                ("kind", C.c_int * MAX_SDOM_FACES), ("T", C.c_double * MAX_SDOM_FACES)]


class PairDesc(C.Structure):
    _fields_ = [("kind", C.c_int), ("sdom1", C.c_int), ("face1", C.c_int), ("sdom2", C.c_int),
                ("face2", C.c_int), ("transl", C.c_double * 3), ("rot", C.c_double * 9)]


class ProblemDesc(C.Structure):
    _fields_ = [("problem", C.c_int), ("nemit", C.c_long), ("maxscat", C.c_long),
                ("maxloop", C.c_long), ("dt", C.c_double), ("nsteps", C.c_long),
                ("precision", C.c_int), ("seed", C.c_uint64), ("steps_per_launch", C.c_int),
                ("block_size", C.c_int), ("grid_blocks", C.c_int), ("tally_mode", C.c_int),
                ("replay_words", C.POINTER(C.c_uint32)), ("replay_offsets", C.POINTER(C.c_int64)),
                ("log", C.POINTER(C.c_double)), ("log_counts", C.POINTER(C.c_int64)),
                ("log_cap", C.c_long), ("log_phonons", C.c_long), ("stream", C.c_void_p),
                ("schedule", C.c_int), ("compact_interval", C.c_int), ("cum_size", C.c_long)]


class Stats(C.Structure):
    _fields_ = [("nemit", C.c_long), ("power", C.c_double), ("rows", C.c_long), ("cols", C.c_long),
                ("phonon_steps", C.c_double), ("events", C.c_long), ("scatters", C.c_long),
                ("escapes", C.c_long), ("horizon_stops", C.c_long), ("maxscat_stops", C.c_long),
                ("maxloop_stops", C.c_long), ("absorbed", C.c_long), ("nonfinite", C.c_long),
                ("status", C.c_uint), ("kernel_ms", C.c_double), ("launches", C.c_int),
                ("checksum", C.c_double * 4)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["checksum"] = list(self.checksum)
        return d


class BatchDesc(C.Structure):
    _fields_ = [("dt", C.c_double), ("nsteps", C.c_long), ("precision", C.c_int),
                ("steps_per_launch", C.c_int), ("block_size", C.c_int), ("grid_blocks", C.c_int),
                ("use_graph", C.c_int), ("stream", C.c_void_p)]


class ServerDesc(C.Structure):
    _fields_ = [("dt", C.c_double), ("nsteps", C.c_long), ("precision", C.c_int), ("hbm_budget", C.c_size_t),
                ("max_active", C.c_int), ("groups", C.c_int), ("target_rel_se", C.c_double),
                ("min_rounds", C.c_int), ("max_rounds", C.c_int), ("block_size", C.c_int),
                ("steps_per_window", C.c_int)]


class Request(C.Structure):
    _fields_ = [("mat", C.c_void_p), ("dom", C.c_void_p), ("problem", C.c_int), ("nemit", C.c_long),
                ("maxscat", C.c_long), ("maxloop", C.c_long), ("seed", C.c_uint64), ("axis", C.c_int),
                ("volume", C.c_double), ("gradient", C.c_double), ("field", C.c_int), ("max_rounds", C.c_int)]


class Result(C.Structure):
    _fields_ = [("kappa", C.c_double), ("kappa_se", C.c_double), ("rounds", C.c_long), ("phonons", C.c_long),
                ("phonon_steps", C.c_double), ("t_submit", C.c_double), ("t_admit", C.c_double),
                ("t_done", C.c_double), ("status", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerCounters(C.Structure):
    _fields_ = [("submitted", C.c_long), ("admitted", C.c_long), ("completed", C.c_long), ("queued", C.c_long),
                ("active", C.c_long), ("ticks", C.c_long), ("busy_s", C.c_double), ("uptime_s", C.c_double),
                ("phonon_steps", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# every symbol declared in include/mc_gb300.h
SYMBOLS = [
    "mc_last_error", "mc_version",
    "mc_material_create", "mc_material_load", "mc_material_sums", "mc_material_tables",
    "mc_material_destroy", "mc_material_create_many", "mc_material_thresholds",
    "mc_domain_create", "mc_domain_create_shapes", "mc_domain_cols", "mc_domain_cell_volumes", "mc_domain_destroy",
    "mc_solve", "mc_solve_noalloc", "mc_solve_replicas", "mc_check_bounded_wait",
    "mc_session_create", "mc_session_emit", "mc_session_advance", "mc_session_result",
    "mc_session_state_bytes", "mc_session_destroy", "mc_session_snapshot_bytes", "mc_session_snapshot",
    "mc_session_restore",
    "mc_batch_create", "mc_batch_run", "mc_batch_result", "mc_batch_stats", "mc_batch_state_bytes",
    "mc_batch_destroy",
    "mc_server_create", "mc_server_submit", "mc_server_cancel", "mc_server_poll", "mc_server_wait",
    "mc_server_stats",
    "mc_server_clock", "mc_server_destroy",
]

_lib = None


class McError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, 'error')} ({code}): {msg}")
        self.code = code


def lib(build_if_missing: bool = True):
    """Load libmc_gb300.so (building it with nvcc if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: run montecarlocpp_gb300.build.build()")
        _build.build()
    L = C.CDLL(path)
    P = C.POINTER
    L.mc_last_error.restype = C.c_char_p
    L.mc_version.restype = C.c_char_p
    L.mc_material_create.argtypes = [P(C.c_double), C.c_long, C.c_long, P(C.c_double), C.c_double, P(C.c_void_p)]
    L.mc_material_load.argtypes = [C.c_char_p, C.c_char_p, C.c_double, P(C.c_void_p)]
    L.mc_material_sums.argtypes = [C.c_void_p, P(C.c_double)]
    L.mc_material_create_many.argtypes = [P(C.c_double), C.c_long, C.c_long, P(C.c_double), P(C.c_double), C.c_int,
                                          P(C.c_void_p)]
    L.mc_material_thresholds.argtypes = [C.c_void_p] + [P(C.c_uint64)] * 4
    L.mc_material_tables.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double)]
    L.mc_material_destroy.argtypes = [C.c_void_p]
    L.mc_domain_create.argtypes = [P(PpedDesc), C.c_int, P(PairDesc), C.c_int, P(C.c_void_p)]
    L.mc_domain_create_shapes.argtypes = [P(SdomDesc), C.c_int, P(PairDesc), C.c_int, P(C.c_void_p)]
    L.mc_domain_cols.restype = C.c_long
    L.mc_domain_cols.argtypes = [C.c_void_p]
    L.mc_domain_cell_volumes.argtypes = [C.c_void_p, P(C.c_double)]
    L.mc_domain_destroy.argtypes = [C.c_void_p]
    L.mc_solve.argtypes = [C.c_void_p, C.c_void_p, P(ProblemDesc), P(C.c_double), P(Stats)]
    L.mc_solve_noalloc.argtypes = [C.c_void_p, C.c_void_p, P(ProblemDesc), P(C.c_double), P(Stats)]
    L.mc_check_bounded_wait.argtypes = [C.c_double, P(C.c_uint), P(C.c_double)]
    L.mc_solve_replicas.argtypes = [C.c_void_p, C.c_void_p, P(ProblemDesc), C.c_long, P(C.c_double),
                                    P(C.c_double), P(Stats)]
    L.mc_session_create.argtypes = [C.c_void_p, C.c_void_p, P(ProblemDesc), P(C.c_void_p)]
    L.mc_session_emit.argtypes = [C.c_void_p]
    L.mc_session_advance.argtypes = [C.c_void_p, C.c_int, P(C.c_int)]
    L.mc_session_result.argtypes = [C.c_void_p, P(C.c_double), P(Stats)]
    L.mc_session_snapshot_bytes.restype = C.c_size_t
    L.mc_session_snapshot_bytes.argtypes = [C.c_void_p]
    L.mc_session_snapshot.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
    L.mc_session_restore.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
    L.mc_session_state_bytes.restype = C.c_size_t
    L.mc_session_state_bytes.argtypes = [C.c_void_p]
    L.mc_session_destroy.argtypes = [C.c_void_p]
    L.mc_batch_create.argtypes = [C.c_int, P(C.c_void_p), P(C.c_void_p), P(ProblemDesc), P(BatchDesc),
                                  P(C.c_void_p)]
    L.mc_batch_run.argtypes = [C.c_void_p]
    L.mc_batch_result.argtypes = [C.c_void_p, C.c_int, P(C.c_double), P(Stats)]
    L.mc_batch_stats.argtypes = [C.c_void_p, P(Stats)]
    L.mc_batch_state_bytes.restype = C.c_size_t
    L.mc_batch_state_bytes.argtypes = [C.c_void_p]
    L.mc_batch_destroy.argtypes = [C.c_void_p]
    L.mc_server_create.argtypes = [P(ServerDesc), P(C.c_void_p)]
    L.mc_server_submit.argtypes = [C.c_void_p, P(Request), P(C.c_long)]
    L.mc_server_poll.argtypes = [C.c_void_p, C.c_long, P(Result), P(C.c_double)]
    L.mc_server_cancel.argtypes = [C.c_void_p, C.c_long]
    L.mc_server_wait.argtypes = [C.c_void_p, C.c_long, C.c_double, P(Result), P(C.c_double)]
    L.mc_server_stats.argtypes = [C.c_void_p, P(ServerCounters)]
    L.mc_server_clock.restype = C.c_double
    L.mc_server_clock.argtypes = [C.c_void_p]
    L.mc_server_destroy.argtypes = [C.c_void_p]
    _lib = L
    return L


def check(rc: int):
    if rc != MC_OK:
        raise McError(rc, lib().mc_last_error().decode(errors="replace"))
