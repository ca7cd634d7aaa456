"""GPU parity tests: the sm_103a kernels, called through the C ABI, against
the CPU oracle on the same inputs.

Tolerances (stated per test):
* trajectories, FP64 flight: loop index, subdomains, face hit, cell, nscat,
  w, p identical; positions within 1e-12 of the domain size; times 1e-12
  relative;
* trajectories, FP32 flight: the same discrete fields identical except in
  as many trajectories as the measured FP32 discrete-mismatch rate allows
  (test_gpu_statistics.mismatch_allowance); positions within 1e-5 of the
  domain size;
* fields, FP64 flight: within 1e-9 of each row's largest magnitude;
* statistics: kappa within 3 standard errors of the oracle.
"""

import numpy as np
import pytest

import montecarlocpp_gb300 as M
from oracle import oracle as O
from test_gpu_statistics import mismatch_allowance

pytestmark = pytest.mark.gpu

DISCRETE = [0, 1, 2, 3, 4, 9, 10, 11]


def domains():
    return {
        "film": M.FilmDomain.from_cli(1e-7, 1e-7, 100),
        "cross": M.CrossPlaneFilmDomain(1e-7, 1e-7, 20),
        "bulk": M.BulkDomain.from_cli(1e-6, 10),
        "pore": M.PoreCellDomain(5e-7, 2.5e-7),
    }


CASES = {
    "film": (M.MULTI, 2000, 0.5e-12, 400),
    "cross": (M.TEMP, 2000, 1e-12, 2000),
    "bulk": (M.FLUX, 2000, 0.5e-12, 400),
    "pore": (M.MULTI, 1500, 0.5e-12, 400),
}
PROBLEM = {M.TEMP: M.TempProblem, M.FLUX: M.FluxProblem, M.MULTI: M.MultiProblem}


def run_pair(gmat, omat, dom, kind, nemit, dt, nsteps, prec, K, seed=7, maxscat=10**6, log_cap=512,
             nlog=96, rng=O.RNG_PHILOX, replay=None, oracle_kw=None, **kw):
    od = O.ODomain(dom)
    o_out, o_st, ex = O.solve(omat, od, kind, nemit=nemit, maxscat=maxscat, dt=dt, horizon=dt * nsteps,
                              rng=rng, seed=seed, log_cap=log_cap, log_phonons=nlog, **(oracle_kw or {}))
    P = PROBLEM[kind](gmat, dom, nemit, maxscat)
    if replay == "from_oracle":
        replay = O.record_to_replay(ex["record"])
    g_out = P.solve(dt=dt, nsteps=nsteps, seed=seed, precision=prec, steps_per_launch=K, log_cap=log_cap,
                    log_phonons=nlog, replay=replay, **kw)
    return (o_out, o_st, ex["log"]), (g_out, P.stats, P.log)


def compare_logs(olog, glog, L, pos_tol, allow_mismatch=0, pos_quantile=1.0, pos_cap=None):
    """Discrete fields (loop index, subdomains, face, cell, nscat, w, p) must
    be identical in all but `allow_mismatch` trajectories. Positions of the
    matching trajectories: within pos_tol * L for a fraction pos_quantile of
    the records and within pos_cap * L for all. Times: 1e-12 relative in
    FP64."""
    (a_rec, a_cnt), (b_rec, b_cnt) = olog, glog
    bad = 0
    errs = []
    for i in range(min(len(a_cnt), len(b_cnt))):
        n = int(min(a_cnt[i], b_cnt[i], a_rec.shape[1]))
        a, b = a_rec[i, :n], b_rec[i, :n]
        ok = a_cnt[i] == b_cnt[i] and np.array_equal(a[:, DISCRETE], b[:, DISCRETE])
        if not ok:
            bad += 1
            continue
        if n:
            # FP32: positions at events; a record at the time horizon is a
            # position sampled at a fixed time, where an event-time error
            # (a position error over a slow segment's velocity) reappears
            # multiplied by the current velocity
            ev = a[:, 2] >= -1 if pos_tol > 1e-12 else np.ones(n, bool)
            errs.extend((np.abs(a[ev, 5:8] - b[ev, 5:8]).max(axis=1) / L).tolist())
            if pos_tol <= 1e-12:
                assert np.allclose(a[:, 8], b[:, 8], rtol=1e-12, atol=0)
    assert bad <= allow_mismatch, f"{bad} trajectories differ"
    errs = np.array(errs) if errs else np.zeros(1)
    assert np.quantile(errs, pos_quantile) <= pos_tol, (np.quantile(errs, pos_quantile), errs.max())
    if pos_cap is not None:
        assert errs.max() <= pos_cap, errs.max()
    return bad, float(errs.max())


def field_err(a, b):
    scale = np.abs(a).max(axis=1, keepdims=True)
    scale[scale == 0] = 1
    return float((np.abs(a - b) / scale).max())


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("K", [1, 50, 100000])
def test_fp64_trajectories_and_field(name, K, gmat, omat):
    dom = domains()[name]
    kind, nemit, dt, nsteps = CASES[name]
    (oo, ost, olog), (go, gst, glog) = run_pair(gmat, omat, dom, kind, nemit, dt, nsteps, 64, K)
    assert gst["nemit"] == ost["nemit"]
    assert gst["events"] == ost["events"]
    assert gst["scatters"] == ost["scatters"]
    assert gst["absorbed"] == ost["absorbed"]
    assert gst["horizon_stops"] == ost["horizon_stops"]
    assert gst["phonon_steps"] == ost["phonon_steps"]
    compare_logs(olog, glog, dom.max_dim(), 1e-12)
    assert field_err(oo, go) < 1e-9


@pytest.mark.parametrize("name", list(CASES))
def test_fp32_trajectories(name, gmat, omat):
    dom = domains()[name]
    kind, nemit, dt, nsteps = CASES[name]
    (oo, ost, olog), (go, gst, glog) = run_pair(gmat, omat, dom, kind, nemit, dt, nsteps, 32, 50)
    # FP32 directions carry ~1e-7 relative rounding; a wall reached at a
    # grazing angle a turns a transverse error d into d / a along the wall.
    # Trajectories that part from the FP64 ones: at most as many as the
    # measured FP32 mismatch rate over this horizon allows
    allow = mismatch_allowance(name, dt * nsteps, len(olog[1]))
    bad, _ = compare_logs(olog, glog, dom.max_dim(), 1e-5, allow_mismatch=allow, pos_quantile=0.99, pos_cap=1e-3)
    # the per-result FP32 error of the field against the FP64 oracle
    assert field_err(oo, go) < 5e-3


@pytest.mark.parametrize("prec,tol", [(64, 1e-12), (32, 1e-5)])
def test_replay_of_reference_stream(prec, tol, gmat, omat):
    """The oracle runs the reference's uniform scheme (mt19937 engines over
    static phonon chunks, montecarlo/main.cpp:29-39,155-160), records the
    32-bit words each phonon consumed; the GPU replays them."""
    dom = domains()["film"]
    (oo, ost, olog), (go, gst, glog) = run_pair(
        gmat, omat, dom, M.MULTI, 1000, 0.5e-12, 300, prec, 37, seed=0, rng=O.RNG_MT, replay="from_oracle",
        oracle_kw=dict(nchunk=4, record_cap=8192))
    assert gst["status"] == 0
    if prec == 64:
        compare_logs(olog, glog, dom.max_dim(), tol)
    else:
        allow = mismatch_allowance("film", 0.5e-12 * 300, len(olog[1]))
        compare_logs(olog, glog, dom.max_dim(), tol, allow_mismatch=allow, pos_quantile=0.99, pos_cap=1e-3)
    if prec == 64:
        assert gst["events"] == ost["events"]
        assert field_err(oo, go) < 1e-9


def test_replay_exhausted_is_an_error(gmat):
    dom = domains()["film"]
    P = M.MultiProblem(gmat, dom, 100, 10**6)
    n = 100
    words = np.arange(3 * n, dtype=np.uint32) * 2654435761
    offsets = np.arange(n + 1, dtype=np.int64) * 3
    with pytest.raises(M.problem._lib.McError) as e:
        P.solve(dt=0.5e-12, nsteps=200, precision=64, replay=(words, offsets))
    assert e.value.code == -6


@pytest.mark.parametrize("name", ["cross", "pore"])
def test_schedules_agree(name, gmat):
    """Static passes (front/back compaction), dynamic lane refill in place,
    and dynamic with periodic compaction give the same trajectories."""
    dom = domains()[name]
    kind, nemit, dt, nsteps = CASES[name]
    P = PROBLEM[kind](gmat, dom, 4 * nemit, 10**6)
    kw = dict(dt=dt, nsteps=nsteps, precision=64, steps_per_launch=20, seed=21)
    a = P.solve(schedule=1, **kw)
    sa = dict(P.stats)
    b = P.solve(schedule=2, **kw)
    sb = dict(P.stats)
    c = P.solve(schedule=2, compact_interval=2, **kw)
    sc = dict(P.stats)
    for k in ("events", "scatters", "absorbed", "horizon_stops", "phonon_steps"):
        assert sa[k] == sb[k] == sc[k], k
    assert field_err(a, b) < 1e-12 and field_err(a, c) < 1e-12


def test_tally_layouts_agree(gmat):
    dom = domains()["film"]
    P = M.MultiProblem(gmat, dom, 5000, 10**6)
    a = P.solve(dt=0.5e-12, nsteps=300, precision=64, steps_per_launch=30, tally_mode=0, seed=3)
    b = P.solve(dt=0.5e-12, nsteps=300, precision=64, steps_per_launch=30, tally_mode=1, seed=3)
    assert field_err(a, b) < 1e-12


def test_launch_shape_does_not_change_results(gmat):
    dom = domains()["pore"]
    P = M.MultiProblem(gmat, dom, 3000, 10**6)
    a = P.solve(dt=0.5e-12, nsteps=200, precision=64, steps_per_launch=200, block_size=256, seed=4)
    ea = P.stats["events"]
    b = P.solve(dt=0.5e-12, nsteps=200, precision=64, steps_per_launch=7, block_size=64, grid_blocks=13, seed=4)
    assert P.stats["events"] == ea
    assert field_err(a, b) < 1e-12


def test_checksum_partition_of_unity_full_size(gmat):
    """At the full in-plane film size (1e7 phonons, 4000 steps of 0.5 ps)
    the raw tally summed over cells equals the sum over every flight of its
    amount (the cell split loses nothing), and no phonon is lost."""
    dom = M.FilmDomain.from_cli(1e-7, 1e-7, 100)
    P = M.MultiProblem(gmat, dom, 10_000_000, 10**6)
    out = P.solve(dt=0.5e-12, nsteps=4000, precision=32, steps_per_launch=200, seed=11)
    st = P.stats
    assert st["horizon_stops"] == st["nemit"] and st["escapes"] == 0 and st["nonfinite"] == 0
    assert st["phonon_steps"] == 4000 * st["nemit"]
    vol = P.handle.cell_volumes()
    raw = out * vol / st["power"]
    raw[0] *= gmat.energySum()
    for r in range(4):
        # the shared layout splits each flight's int64 amount exactly; the
        # two sides differ only by the FP64 rounding of the conversions
        assert raw[r].sum() == pytest.approx(st["checksum"][r], rel=1e-12, abs=1e-12 * abs(raw[r]).sum())
    kappa = M.kappa_from_flux(out, dom, 0, flux_row0=1)
    assert 20 < kappa < 120


def test_checksum_fp64(gmat):
    dom = M.PoreCellDomain(5e-7, 2.5e-7)
    P = M.MultiProblem(gmat, dom, 20000, 10**6)
    out = P.solve(dt=0.5e-12, nsteps=500, precision=64, steps_per_launch=100, seed=12)
    st = P.stats
    raw = out * P.handle.cell_volumes() / st["power"]
    raw[0] *= gmat.energySum()
    for r in range(4):
        assert raw[r].sum() == pytest.approx(st["checksum"][r], rel=1e-11, abs=1e-11 * abs(raw[r]).sum())


def test_kappa_statistical_parity(gmat, omat):
    """FP32 GPU (Philox) against the FP64 oracle run with the reference's
    mt19937 scheme on the 100 nm film, 8 independent replicas each:
    * kappa within 3 standard errors;
    * the per-cell temperature profile (row 0) and x-flux profile (row 1):
      every cell's difference of means within 5 standard errors of that cell
      (Welch, 14 degrees of freedom), and the mean squared z over the 40
      cells below 2.5 (its expectation is about 1.2 for equal means)."""
    dom = M.FilmDomain.from_cli(1e-7, 1e-7, 20)
    od = O.ODomain(dom)
    dt, nsteps, n, R = 0.5e-12, 1000, 15000, 8
    ko, kg, fo, fg = [], [], [], []
    for s in range(R):
        o, _, _ = O.solve(omat, od, O.MULTI, nemit=n, maxscat=10**6, dt=dt, horizon=dt * nsteps,
                          rng=O.RNG_MT, nchunk=8, seed=100 * s)
        ko.append(M.kappa_from_flux(o, dom, 0, flux_row0=1))
        fo.append(np.asarray(o)[:2])
    P = M.MultiProblem(gmat, dom, n, 10**6)
    for s in range(R):
        g = P.solve(dt=dt, nsteps=nsteps, precision=32, steps_per_launch=100, seed=1000 + s)
        kg.append(M.kappa_from_flux(g, dom, 0, flux_row0=1))
        fg.append(np.asarray(g)[:2])
    ko, kg = np.array(ko), np.array(kg)
    se = np.sqrt(ko.var(ddof=1) / R + kg.var(ddof=1) / R)
    assert abs(ko.mean() - kg.mean()) < 3 * se
    fo, fg = np.array(fo), np.array(fg)                      # replicas x 2 rows x cells
    se = np.sqrt(fo.var(axis=0, ddof=1) / R + fg.var(axis=0, ddof=1) / R)
    z = (fo.mean(axis=0) - fg.mean(axis=0)) / se
    assert np.abs(z).max() < 5, np.abs(z).max(axis=1)
    assert (z ** 2).mean() < 2.5, (z ** 2).mean(axis=1)


def test_edge_cases(gmat, omat):
    film = domains()["film"]
    # one requested phonon
    P = M.TempProblem(gmat, film, 1, 10)
    P.solve(dt=1e-12, nsteps=5, precision=64)
    assert P.stats["nemit"] == 1
    # maxscat = 1 stops every phonon at its first scatter
    P = M.FluxProblem(gmat, film, 500, 1)
    P.solve(dt=1e-12, nsteps=10**6, precision=64, steps_per_launch=10**6)
    st = P.stats
    assert st["maxscat_stops"] + st["maxloop_stops"] == st["nemit"]
    # one step only
    P = M.MultiProblem(gmat, film, 500, 10**6)
    P.solve(dt=1e-12, nsteps=1, precision=32)
    assert P.stats["phonon_steps"] == P.stats["nemit"] == P.stats["horizon_stops"]
    # isothermal walls absorb everything given time
    cross = domains()["cross"]
    P = M.TempProblem(gmat, cross, 2000, 10**6)
    P.solve(dt=1e-12, nsteps=200000, precision=32, steps_per_launch=5000)
    st = P.stats
    assert st["absorbed"] + st["horizon_stops"] == st["nemit"] and st["absorbed"] > 0.99 * st["nemit"]


def test_determinism(gmat):
    dom = domains()["pore"]
    P = M.MultiProblem(gmat, dom, 20000, 10**6)
    a = P.solve(dt=0.5e-12, nsteps=300, precision=32, steps_per_launch=30, seed=9)
    ea = P.stats["events"]
    b = P.solve(dt=0.5e-12, nsteps=300, precision=32, steps_per_launch=30, seed=9)
    assert P.stats["events"] == ea
    assert field_err(a, b) < 1e-10


@pytest.mark.parametrize("name", ["film", "cross", "bulk"])
@pytest.mark.parametrize("prec", [32, 64])
def test_lean_flight_matches_the_walker(name, prec, gmat):
    """The per-step static kernel takes a lean straight-line flight for the
    phonons with no event in the window when the field is 1-D along one
    axis and no event log is kept; with a log it runs the walker for every
    phonon. The two must agree: the lean flight repeats the walker's
    arithmetic and each block's fixed-point field is exact, so counters are
    equal and fields differ only by the order of the FP64 atomics that add
    the blocks' fields (1e-13 of each row's scale)."""
    dom = domains()[name]
    kind, nemit, dt, nsteps = CASES[name]
    P = PROBLEM[kind](gmat, dom, 4 * nemit, 10**6)
    kw = dict(dt=dt, nsteps=min(nsteps, 300), precision=prec, steps_per_launch=1, schedule=1, seed=31)
    lean = P.solve(**kw)
    sl = dict(P.stats)
    walker = P.solve(log_cap=4, log_phonons=1, **kw)
    sw = dict(P.stats)
    for k in ("events", "scatters", "absorbed", "horizon_stops", "phonon_steps", "nonfinite", "escapes"):
        assert sl[k] == sw[k], k
    assert field_err(walker, lean) < 1e-13
    assert np.allclose(sl["checksum"], sw["checksum"], rtol=1e-13, atol=0)


@pytest.mark.parametrize("name", ["film", "cross"])
def test_fp64_plain_kernel_against_oracle_without_log(name, gmat, omat):
    """The per-step kernel with the lean flight in FP64 against the oracle:
    event counts exact, field within 1e-9 of each row's scale."""
    dom = domains()[name]
    kind, nemit, dt, nsteps = CASES[name]
    o, ost, _ = O.solve(omat, O.ODomain(dom), kind, nemit=nemit, maxscat=10**6, dt=dt, horizon=dt * nsteps,
                        rng=O.RNG_PHILOX, seed=7)
    P = PROBLEM[kind](gmat, dom, nemit, 10**6)
    g = P.solve(dt=dt, nsteps=nsteps, precision=64, steps_per_launch=1, schedule=1, seed=7)
    assert P.stats["events"] == ost["events"]
    assert P.stats["phonon_steps"] == ost["phonon_steps"]
    assert field_err(o, g) < 1e-9


CUM = {M.CUMTEMP: M.CumTempProblem, M.CUMFLUX: M.CumFluxProblem}


@pytest.mark.parametrize("kind", [M.CUMTEMP, M.CUMFLUX])
@pytest.mark.parametrize("K,schedule", [(1, 1), (40, 2), (100000, 0)])
def test_cum_problems_fp64_against_oracle(kind, K, schedule, gmat, omat):
    """CumTemp / CumFlux (montecarlo/problem.cpp:553-648): the field binned
    by the scatter count before each flight, cumulative over the bins. FP64
    flight against the oracle in the static (lean flight), dynamic and
    whole-horizon schedules: event counts exact, field within 1e-9."""
    dom = domains()["film"]
    nemit, dt, nsteps, size, maxscat = 2000, 0.5e-12, 400, 4, 21
    o, ost, _ = O.solve(omat, O.ODomain(dom), kind, nemit=nemit, maxscat=maxscat, dt=dt, horizon=dt * nsteps,
                        rng=O.RNG_PHILOX, seed=9, size=size)
    P = CUM[kind](gmat, dom, nemit, size, maxscat)
    g = P.solve(dt=dt, nsteps=nsteps, precision=64, steps_per_launch=K, schedule=schedule, seed=9)
    assert g.shape == o.shape == (P.rows(), dom_cols(dom))
    for k in ("events", "scatters", "maxscat_stops", "phonon_steps"):
        assert P.stats[k] == ost[k], k
    assert field_err(o, g) < 1e-9


def dom_cols(dom):
    return M.problem._handle(dom).cols


def test_cum_flux_pore_cell_fp64_and_fp32(gmat, omat):
    """CumFlux on the 3-D pore cell (FP64 global atomics at the flight's bin
    rows) against the oracle, and the FP32 field's error."""
    dom = M.PoreCellDomain(5e-7, 2.5e-7, (4, 8, 4))
    nemit, dt, nsteps, size, maxscat = 1500, 0.5e-12, 300, 3, 31
    o, ost, _ = O.solve(omat, O.ODomain(dom), M.CUMFLUX, nemit=nemit, maxscat=maxscat, dt=dt,
                        horizon=dt * nsteps, rng=O.RNG_PHILOX, seed=4, size=size)
    P = M.CumFluxProblem(gmat, dom, nemit, size, maxscat)
    g = P.solve(dt=dt, nsteps=nsteps, precision=64, steps_per_launch=50, seed=4)
    assert P.stats["events"] == ost["events"]
    assert field_err(o, g) < 1e-9
    g32 = P.solve(dt=dt, nsteps=nsteps, precision=32, steps_per_launch=50, seed=4)
    assert field_err(o, g32) < 5e-3


def test_cum_last_bin_is_the_plain_field(gmat):
    """The last cumulative bin of CumTemp / CumFlux is the Temp / Flux field
    of the same phonons (FP32 flight, same Philox streams; bins few enough
    that every field stays in the blocks' shared fixed-point layout)."""
    dom = domains()["film"]
    kw = dict(dt=0.5e-12, nsteps=300, precision=32, steps_per_launch=300, seed=17)
    t = M.TempProblem(gmat, dom, 20000, 25).solve(**kw)
    f = M.FluxProblem(gmat, dom, 20000, 25).solve(**kw)
    ct = M.CumTempProblem(gmat, dom, 20000, 6, 25).solve(**kw)
    cf = M.CumFluxProblem(gmat, dom, 20000, 4, 25).solve(**kw)
    assert field_err(t, ct[-1:]) < 1e-12
    assert field_err(f, cf[-3:]) < 1e-12


def test_cum_problem_arguments(gmat):
    dom = domains()["film"]
    with pytest.raises(ValueError):
        M.CumTempProblem(gmat, dom, 100, 0, 10)
    with pytest.raises(ValueError):
        M.CumFluxProblem(gmat, dom, 100, 3, 1)


def test_replica_statistics(gmat):
    """mc_solve_replicas: nsim solves with seeds seed + i and their
    Welford mean and sample standard deviation (montecarlo/field.cpp:226-262,
    montecarlo/main.cpp:181-210), against numpy over the same solves run
    one at a time."""
    dom = M.FilmDomain.from_cli(1e-7, 1e-7, 20)
    P = M.MultiProblem(gmat, dom, 5000, 10**6)
    kw = dict(dt=0.5e-12, nsteps=200, precision=64, steps_per_launch=200)
    mean, sd = P.solve_replicas(5, seed=40, **kw)
    st = dict(P.stats)
    runs = []
    ev = 0
    for i in range(5):
        runs.append(P.solve(seed=40 + i, **kw))
        ev += P.stats["events"]
    runs = np.array(runs)
    assert st["events"] == ev
    assert field_err(runs.mean(axis=0), mean) < 1e-12
    ref_sd = runs.std(axis=0, ddof=1)
    assert np.allclose(sd, ref_sd, rtol=1e-9, atol=1e-12 * np.abs(ref_sd).max())
    one, sd1 = P.solve_replicas(1, seed=40, **kw)
    assert field_err(runs[0], one) < 1e-12 and not sd1.any()


@pytest.mark.parametrize("nemit,block,grid", [(1, 0, 0), (300, 0, 0), (5000, 32, 3), (20000, 64, 7), (20000, 256, 1)])
@pytest.mark.parametrize("prec", [32, 64])
def test_static_regions_in_unusual_launch_shapes(nemit, block, grid, prec, gmat):
    """The per-step static kernel cuts the state into one region per block
    and streams it in tiles of block_size slots: fewer phonons than blocks
    (empty regions), one phonon, tiles of one warp, a few large regions, one
    block. Absorbing walls make regions shrink. Results match the dynamic
    schedule on the same phonons (identical trajectories)."""
    dom = domains()["cross"]
    P = M.TempProblem(gmat, dom, nemit, 10**6)
    kw = dict(dt=1e-12, nsteps=300, precision=prec, seed=19)
    s = P.solve(steps_per_launch=1, schedule=1, block_size=block, grid_blocks=grid, **kw)
    ss = dict(P.stats)
    d = P.solve(steps_per_launch=30, schedule=2, **kw)
    sd = dict(P.stats)
    for k in ("events", "scatters", "absorbed", "horizon_stops", "escapes"):
        assert ss[k] == sd[k], k
    # phonon-steps count the windows a phonon was alive at the start of; in
    # FP32 an absorption within rounding of a dt boundary can fall on either
    # side of it depending on how the windows cut the flight
    if prec == 64:
        assert ss["phonon_steps"] == sd["phonon_steps"]
    else:
        assert abs(ss["phonon_steps"] - sd["phonon_steps"]) <= 1e-5 * sd["phonon_steps"] + 1
    assert ss["status"] == 0
    tol = 1e-12 if prec == 64 else 1e-5
    assert field_err(d, s) < tol


def test_static_lean_kernel_with_more_phonons_than_one_wave_holds(gmat):
    """4.2e7 phonons of the in-plane film: more per resident block than the
    lean flights' carry-free field holds in one launch (2^18 on 152 SMs), so
    the per-step kernel runs whole extra waves of blocks. The trajectories
    equal the dynamic schedule's (counters) and the fields agree to FP32
    flight precision."""
    dom = M.FilmDomain.from_cli(1e-7, 1e-7, 100)
    P = M.MultiProblem(gmat, dom, 42_000_000, 10**6)
    kw = dict(dt=0.5e-12, nsteps=12, precision=32, seed=23)
    s = P.solve(steps_per_launch=1, schedule=1, **kw)
    ss = dict(P.stats)
    d = P.solve(steps_per_launch=12, schedule=2, **kw)
    sd = dict(P.stats)
    assert ss["status"] == 0 and sd["status"] == 0
    for k in ("events", "scatters", "absorbed", "escapes"):
        assert ss[k] == sd[k], k
    assert abs(ss["phonon_steps"] - sd["phonon_steps"]) <= 1e-5 * sd["phonon_steps"] + 1
    assert field_err(d, s) < 1e-5


def test_launch_wide_slot_counter_matches_static_schedule(gmat):
    """FP32 flight with windows of 2000 dt-steps: the fused kernel's blocks
    claim slots from one launch-wide counter (windows of 1024 steps or more)
    while the static schedule streams block-owned regions through the same
    windows. Same phonons and windows, same trajectories: equal counters;
    the fields differ only by the order of the FP64 adds of the blocks'
    fixed-point fields."""
    dom = M.FilmDomain.from_cli(1e-7, 1e-7, 100)
    P = M.MultiProblem(gmat, dom, 300_000, 10**6)
    kw = dict(dt=0.5e-12, nsteps=2000, precision=32, steps_per_launch=2000, seed=29)
    a = P.solve(schedule=2, **kw)
    sa = dict(P.stats)
    c = P.solve(schedule=1, **kw)
    sc = dict(P.stats)
    for k in ("events", "scatters", "absorbed", "escapes", "horizon_stops", "phonon_steps"):
        assert sa[k] == sc[k], k
    assert sa["status"] == sc["status"] == 0
    assert field_err(a, c) < 1e-12
