"""Snapshot and resume of device-resident sessions: a session restored from
a snapshot taken half way continues exactly as the original (every
phonon's random numbers depend only on its id and event index); only the
order of the FP64 atomics that add the blocks' fields differs."""

import numpy as np
import pytest

import montecarlocpp_gb300 as M
from montecarlocpp_gb300 import _lib

pytestmark = pytest.mark.gpu

KEYS = ("events", "scatters", "absorbed", "horizon_stops", "phonon_steps", "escapes", "nonfinite")


def field_err(a, b):
    scale = np.abs(a).max(axis=1, keepdims=True)
    scale[scale == 0] = 1
    return float((np.abs(a - b) / scale).max())


@pytest.mark.parametrize("schedule,K", [(1, 1), (2, 25)])
@pytest.mark.parametrize("prec", [32, 64])
def test_snapshot_resume_continues_exactly(schedule, K, prec, gmat):
    dom = M.CrossPlaneFilmDomain(1e-7, 1e-7, 20)  # isothermal walls absorb: live counts shrink
    P = M.TempProblem(gmat, dom, 20000, 10**6)
    kw = dict(dt=1e-12, nsteps=400, precision=prec, steps_per_launch=K, schedule=schedule, seed=8)
    a = P.session(**kw)
    a.emit()
    a.advance(200 // K)
    snap = a.snapshot()
    a.advance(1 << 20)
    fa, sa = a.result()
    b = P.session(**kw)
    b.restore(snap)
    assert b.advance(1 << 20)
    fb, sb = b.result()
    c = P.session(**kw)
    c.run()
    fc, sc = c.result()
    for k in KEYS:
        assert sa[k] == sb[k] == sc[k], k
    assert sa["absorbed"] > 0
    assert field_err(fa, fb) < 1e-13 and field_err(fa, fc) < 1e-13


def test_restore_refuses_another_problem(gmat):
    dom = M.FilmDomain.from_cli(1e-7, 1e-7, 20)
    a = M.MultiProblem(gmat, dom, 3000, 10**6).session(dt=0.5e-12, nsteps=100, precision=32, steps_per_launch=10)
    a.emit()
    snap = a.snapshot()
    b = M.MultiProblem(gmat, dom, 4000, 10**6).session(dt=0.5e-12, nsteps=100, precision=32, steps_per_launch=10)
    with pytest.raises(_lib.McError):
        b.restore(snap)
    with pytest.raises(_lib.McError):
        b.restore(b"not a snapshot" * 8)


def test_restore_refuses_another_seed_or_window(gmat):
    """A snapshot only restores into a session with the same Philox key,
    time step, horizon and window; otherwise it would continue silently on
    other random numbers or another window."""
    dom = M.FilmDomain.from_cli(1e-7, 1e-7, 20)
    P = M.MultiProblem(gmat, dom, 3000, 10**6)
    kw = dict(dt=0.5e-12, nsteps=100, precision=32, steps_per_launch=10, seed=4)
    a = P.session(**kw)
    a.emit()
    a.advance(3)
    snap = a.snapshot()
    for change in (dict(seed=5), dict(dt=0.25e-12), dict(nsteps=120), dict(steps_per_launch=20)):
        b = P.session(**dict(kw, **change))
        with pytest.raises(_lib.McError):
            b.restore(snap)


def test_truncated_snapshot_leaves_session_unchanged(gmat):
    """A restore that fails for a short buffer changes nothing: the session
    continues as if the call had not been made."""
    dom = M.CrossPlaneFilmDomain(1e-7, 1e-7, 20)
    P = M.TempProblem(gmat, dom, 8000, 10**6)
    kw = dict(dt=1e-12, nsteps=200, precision=64, steps_per_launch=10, schedule=1, seed=9)
    ref = P.session(**kw)
    ref.run()
    fr, sr = ref.result()
    a = P.session(**kw)
    a.emit()
    a.advance(4)
    snap = a.snapshot()
    b = P.session(**kw)
    b.emit()
    b.advance(7)  # another cursor and parity than the snapshot's
    with pytest.raises(_lib.McError):
        b.restore(snap[: len(snap) - 16])
    assert b.advance(1 << 20)
    fb, sb = b.result()
    for k in KEYS:
        assert sb[k] == sr[k], k
    assert field_err(fr, fb) < 1e-13
