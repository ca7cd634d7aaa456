"""The serving loop: completion by the stopping rule, isolation (a result is
the same alone and in the mix), continuous batching (a request submitted
while another runs joins it at the next window), HBM-budget admission,
per-request failures (oversized, out of rounds, cancelled, invalid host
inputs) that leave the other requests' results unchanged, kappa-only
requests, growing rounds, and kappa against the FP64 oracle."""

import time

import numpy as np
import pytest

import montecarlocpp_gb300 as M
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DT, NSTEPS = 0.5e-12, 1000


@pytest.fixture(scope="module")
def mats():
    return {T: M.Material.silicon(T) for T in (150.0, 300.0)}


def test_one_round_equals_single_solve(mats):
    dom = M.FilmDomain.from_cli(1e-7, 1e-7, 50)
    srv = M.Server(dt=DT, nsteps=NSTEPS, precision=64, groups=4, min_rounds=1, max_rounds=1)
    t = srv.submit(mats[300.0], dom, 20000, problem=M.MULTI, seed=77)
    r = srv.wait(t)
    srv.close()
    assert r["rounds"] == 1
    P = M.MultiProblem(mats[300.0], dom, 20000, 10**6)
    f = P.solve(dt=DT, nsteps=NSTEPS, precision=64, seed=77, steps_per_launch=NSTEPS // 8)
    kappa = M.kappa_from_flux(f, dom, 0, flux_row0=1)
    assert r["kappa"] == pytest.approx(kappa, rel=1e-9)
    assert np.allclose(r["field"], f, rtol=1e-9, atol=1e-9 * np.abs(f).max())


def _requests(mats):
    return [
        (mats[300.0], M.FilmDomain.from_cli(1e-7, 1e-7, 50), 60000, 1),
        (mats[150.0], M.FilmDomain.from_cli(1e-7, 3e-8, 30), 40000, 2),
        (mats[300.0], M.PoreCellDomain(5e-7, 2.5e-7, (4, 8, 4)), 50000, 3),
        (mats[150.0], M.FilmDomain.from_cli(1e-7, 5e-7, 100), 30000, 4),
    ]


def test_isolation_alone_and_in_the_mix(mats):
    reqs = _requests(mats)
    kw = dict(dt=DT, nsteps=NSTEPS, precision=32, groups=8, target_rel_se=0.03, min_rounds=1, max_rounds=50)
    alone = []
    for mat, dom, n, seed in reqs:
        srv = M.Server(**kw)
        alone.append(srv.wait(srv.submit(mat, dom, n, seed=seed)))
        srv.close()
    srv = M.Server(**kw)
    tickets = [srv.submit(mat, dom, n, seed=seed) for mat, dom, n, seed in reqs]
    mixed = [srv.wait(t) for t in tickets]
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs)
    for a, b in zip(alone, mixed):
        assert a["status"] == b["status"] == 0
        assert a["rounds"] == b["rounds"]
        # same phonons, same trajectories; only the FP64 atomic order differs
        assert b["kappa"] == pytest.approx(a["kappa"], rel=1e-9)
        assert b["kappa_se"] <= 0.03 * abs(b["kappa"])


def test_hbm_budget_queues_and_completes(mats):
    reqs = _requests(mats)
    # room for about one request's phonon state at a time
    srv = M.Server(dt=DT, nsteps=NSTEPS, precision=32, hbm_budget=70000 * 48, groups=4, target_rel_se=0.05,
                   max_rounds=40)
    tickets = [srv.submit(mat, dom, n, seed=seed) for mat, dom, n, seed in reqs]
    res = [srv.wait(t) for t in tickets]
    st = srv.stats()
    srv.close()
    assert all(r["status"] == 0 for r in res)
    assert st["admitted"] == st["completed"] == len(reqs)
    # admission was serial: each request was admitted after the previous finished
    ends = sorted(r["t_done"] for r in res)
    admits = sorted(r["t_admit"] for r in res)
    assert all(a >= e - 1e-6 for a, e in zip(admits[1:], ends[:-1]))


def test_kappa_against_fp64_oracle(mats):
    dom = M.FilmDomain.from_cli(1e-7, 1e-7, 20)
    srv = M.Server(dt=DT, nsteps=NSTEPS, precision=32, groups=8, target_rel_se=0.01, max_rounds=200)
    r = srv.wait(srv.submit(mats[300.0], dom, 100000, seed=5))
    srv.close()
    assert r["status"] == 0 and r["kappa_se"] <= 0.01 * r["kappa"]
    omat = O.OMaterial(*M.silicon_tables(), 300.0)
    od = O.ODomain(dom)
    ks = []
    for s in range(8):
        o, _, _ = O.solve(omat, od, O.FLUX, nemit=40000, maxscat=10**6, dt=DT, horizon=DT * NSTEPS, rng=O.RNG_MT,
                          nchunk=8, seed=1000 * s)
        ks.append(M.kappa_from_flux(o, dom, 0, flux_row0=0))
    ks = np.array(ks)
    se = np.sqrt(ks.var(ddof=1) / len(ks) + r["kappa_se"] ** 2)
    assert abs(ks.mean() - r["kappa"]) < 3 * se


def test_kappa_only_requests(mats):
    """field=False skips the cell split; kappa comes from the same per-flight
    sums. On a film (1-D field) the trajectories are those of a field
    request, so kappa agrees to the FP64 summation order; on the pore cell
    (3-D walk) the moves round differently, so kappa agrees statistically."""
    kw = dict(dt=DT, nsteps=NSTEPS, precision=64, groups=8, target_rel_se=0.05, min_rounds=1, max_rounds=20)
    film = M.FilmDomain.from_cli(1e-7, 1e-7, 50)
    pore = M.PoreCellDomain(5e-7, 2.5e-7, (4, 8, 4))
    out = {}
    for field in (True, False):
        srv = M.Server(**kw)
        tf = srv.submit(mats[300.0], film, 30000, problem=M.MULTI, seed=11, field=field)
        tp = srv.submit(mats[300.0], pore, 30000, problem=M.MULTI, seed=12, field=field, volume=(5e-7) ** 3)
        out[field] = (srv.wait(tf), srv.wait(tp))
        srv.close()
    (fa, pa), (fb, pb) = out[True], out[False]
    assert fb["field"] is None and fa["field"] is not None
    assert fa["rounds"] == fb["rounds"]
    assert fb["kappa"] == pytest.approx(fa["kappa"], rel=1e-9)
    assert pa["status"] == pb["status"] == 0
    assert abs(pa["kappa"] - pb["kappa"]) < 3 * np.hypot(pa["kappa_se"], pb["kappa_se"])


def test_rounds_grow_to_the_target(mats):
    """A small first round is followed by a round sized for the target: the
    solve needs far fewer rounds than repeats of its first round would."""
    srv = M.Server(dt=DT, nsteps=NSTEPS, precision=32, groups=8, target_rel_se=0.01, min_rounds=1, max_rounds=100)
    r = srv.wait(srv.submit(mats[300.0], M.FilmDomain.from_cli(1e-7, 1e-7, 50), 2000, seed=3, field=False))
    srv.close()
    assert r["status"] == 0 and r["kappa_se"] <= 0.01 * abs(r["kappa"])
    assert r["rounds"] <= 4 and r["phonons"] > 20 * 2000


def test_shape_domains_alone_and_in_the_mix(mats):
    """Requests on the reference's hex rod and L-junction (kernels with the
    general face code) served beside a film: each result is the same alone
    and in the mix, and a one-round hex request equals the single solve."""
    reqs = [
        (mats[300.0], M.HexDomain.from_cli(1e-7, 4e-8), 30000, 5),
        (mats[150.0], M.FilmDomain.from_cli(1e-7, 1e-7, 50), 30000, 6),
        (mats[300.0], M.JctDomain.from_cli(1e-7, 5e-8), 30000, 7),
    ]
    kw = dict(dt=DT, nsteps=NSTEPS, precision=32, groups=8, target_rel_se=0.05, min_rounds=1, max_rounds=20)
    alone = []
    for mat, dom, n, seed in reqs:
        srv = M.Server(**kw)
        alone.append(srv.wait(srv.submit(mat, dom, n, seed=seed)))
        srv.close()
    srv = M.Server(**kw)
    tickets = [srv.submit(mat, dom, n, seed=seed) for mat, dom, n, seed in reqs]
    mixed = [srv.wait(t) for t in tickets]
    srv.close()
    for a, b in zip(alone, mixed):
        assert a["status"] == b["status"] == 0
        assert a["rounds"] == b["rounds"]
        assert b["kappa"] == pytest.approx(a["kappa"], rel=1e-9)
    dom = M.HexDomain.from_cli(1e-7, 4e-8)
    srv = M.Server(dt=DT, nsteps=NSTEPS, precision=64, groups=4, min_rounds=1, max_rounds=1)
    r = srv.wait(srv.submit(mats[300.0], dom, 20000, problem=M.MULTI, seed=78))
    srv.close()
    f = M.MultiProblem(mats[300.0], dom, 20000, 10**6).solve(dt=DT, nsteps=NSTEPS, precision=64, seed=78)
    assert r["kappa"] == pytest.approx(M.kappa_from_flux(f, dom, 0, flux_row0=1), rel=1e-9)


def _solo(kw, mat, dom, n, seed, **req):
    srv = M.Server(**kw)
    r = srv.wait(srv.submit(mat, dom, n, seed=seed, **req))
    srv.close()
    return r


def _wait_for(cond, timeout=60.0):
    t0 = time.monotonic()
    while not cond():
        assert time.monotonic() - t0 < timeout
        time.sleep(0.0005)


def test_request_joins_while_another_runs(mats):
    """Continuous batching: B is submitted after A's first window has run on
    the device; B is admitted before A completes (it joins A's windows), and
    both results equal their solo runs."""
    kw = dict(dt=DT, nsteps=NSTEPS, precision=32, groups=8, target_rel_se=0.01, min_rounds=2, max_rounds=40,
              steps_per_window=NSTEPS // 10)
    A = (mats[300.0], M.PoreCellDomain(5e-7, 2.5e-7, (4, 8, 4)), 400000, 21)
    B = (mats[150.0], M.FilmDomain.from_cli(1e-7, 3e-8, 30), 20000, 22)
    a_solo, b_solo = _solo(kw, *A), _solo(kw, *B)
    srv = M.Server(**kw)
    ta = srv.submit(*A[:3], seed=A[3])
    _wait_for(lambda: srv.stats()["ticks"] >= 1)
    tb = srv.submit(*B[:3], seed=B[3])
    rb = srv.wait(tb)
    ra = srv.wait(ta)
    srv.close()
    assert ra["status"] == rb["status"] == 0
    assert rb["t_submit"] > ra["t_admit"]
    assert rb["t_admit"] < ra["t_done"]  # B joined while A was on the device
    for solo, mixed in ((a_solo, ra), (b_solo, rb)):
        assert mixed["rounds"] == solo["rounds"]
        assert mixed["kappa"] == pytest.approx(solo["kappa"], rel=1e-9)


def test_failures_stay_with_their_request(mats):
    """Host-side fault injection in a mix: a request cancelled while it runs
    (MC_ERR_CANCELLED), one larger than the HBM budget (MC_ERR_BUSY, no
    rounds), one that runs out of rounds (MC_ERR_BUSY after its limit), one
    cancelled while queued, and two with a non-finite host input (refused at
    submit). The healthy requests' results equal their solo runs."""
    budget_phonons = 400000
    kw = dict(dt=DT, nsteps=NSTEPS, precision=32, hbm_budget=budget_phonons * 48, groups=8, target_rel_se=0.02,
              min_rounds=1, max_rounds=40, steps_per_window=NSTEPS // 50)
    good = [(mats[300.0], M.FilmDomain.from_cli(1e-7, 1e-7, 50), 30000, 31),
            (mats[150.0], M.PoreCellDomain(5e-7, 2.5e-7, (4, 8, 4)), 30000, 32)]
    solo = [_solo(kw, *g) for g in good]
    film = M.FilmDomain.from_cli(1e-7, 1e-7, 20)
    srv = M.Server(**kw)
    t_run = srv.submit(mats[150.0], film, 200000, seed=35)  # 50 windows per round
    _wait_for(lambda: srv.stats()["ticks"] >= 1)
    assert srv.cancel(t_run)
    t_good0 = srv.submit(*good[0][:3], seed=good[0][3])
    t_big = srv.submit(mats[300.0], film, 2 * budget_phonons, seed=33)
    t_rounds = srv.submit(mats[300.0], film, 2000, seed=34, max_rounds=1)
    with pytest.raises(M._lib.McError):
        srv.submit(mats[300.0], film, 10000, seed=36, gradient=float("nan"))
    with pytest.raises(M._lib.McError):
        srv.submit(mats[300.0], film, 10000, seed=37, volume=float("inf"))
    t_good1 = srv.submit(*good[1][:3], seed=good[1][3])
    t_queued = srv.submit(mats[300.0], film, 350000, seed=38)  # waits for slots behind the others
    assert srv.cancel(t_queued)
    res = {t: srv.wait(t) for t in (t_run, t_good0, t_big, t_rounds, t_good1, t_queued)}
    assert srv.cancel(t_good0) is False  # already complete
    st = srv.stats()
    srv.close()
    assert res[t_run]["status"] == M._lib.MC_ERR_CANCELLED and res[t_run]["rounds"] == 0
    assert res[t_big]["status"] == M._lib.MC_ERR_BUSY and res[t_big]["rounds"] == 0
    assert res[t_rounds]["status"] == M._lib.MC_ERR_BUSY and res[t_rounds]["rounds"] == 1
    assert res[t_queued]["status"] == M._lib.MC_ERR_CANCELLED and res[t_queued]["rounds"] == 0
    assert st["completed"] == 6 and st["submitted"] == 6
    for t, s in zip((t_good0, t_good1), solo):
        r = res[t]
        assert r["status"] == s["status"] == 0
        assert r["rounds"] == s["rounds"]
        assert r["kappa"] == pytest.approx(s["kappa"], rel=1e-9)
