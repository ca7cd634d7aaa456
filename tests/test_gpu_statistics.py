"""Statistical parity and the FP32 discrete-mismatch rate.

Statistical parity: the GPU (Philox streams) against the FP64 oracle run
with the reference's uniform scheme (mt19937 engines over static phonon
chunks, montecarlo/main.cpp:29-39,155-166), R = 8 independent replicas on
each side, on the cross-plane film (config 0), the in-plane film (config 1)
and the pore cell (config 2, on a coarser grid). Each compared quantity is a
difference of replica means over its Welch standard error; the Welch t is
turned into the equivalent standard-normal z through the t distribution
(Welch-Satterthwaite degrees of freedom), so that under equal means each z
is N(0, 1). The rule:

* kappa: |z| <= 3;
* a profile of m cells (temperature, x-flux): every cell within
  max(3, z_(1 - 0.005 / m)) standard errors -- the 3-SE criterion with a
  Bonferroni correction for m cells at a family-wise 1% false-failure
  probability, which holds however the cells are correlated (the flux of a
  film is nearly the same random number in every cell); and, for profiles
  of 100 cells or more, at most 1% of the cells beyond 3 SE (0.27%
  expected).

The seeds are fixed, so a run is reproducible.

Mismatch rate: the fraction of FP32 trajectories whose discrete fields
(cells, subdomains, faces, event counts, scatter counts, frequency bins,
branches) differ from the FP64 oracle's at or before a horizon, with both
fed the same uniform words (replay of the oracle's mt19937 stream), on
10^4 phonons of the in-plane film, the pore cell and the cross-plane film.
"""

import numpy as np
import pytest

import montecarlocpp_gb300 as M
from montecarlocpp_gb300.logs import divergence_times, mismatch_rate
from oracle import oracle as O

pytestmark = pytest.mark.gpu

R = 8


def welch_z(a, b):
    """Equivalent standard-normal z of the Welch t of the means of replicas
    a and b (first axis), elementwise."""
    from scipy import stats
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    va, vb = a.var(axis=0, ddof=1) / len(a), b.var(axis=0, ddof=1) / len(b)
    se = np.sqrt(va + vb)
    d = a.mean(axis=0) - b.mean(axis=0)
    with np.errstate(divide="ignore", invalid="ignore"):
        t = np.where(se > 0, d / se, np.where(d == 0, 0.0, np.inf))
        nu = np.where(se > 0, (va + vb) ** 2 / (va ** 2 / (len(a) - 1) + vb ** 2 / (len(b) - 1)), 1.0)
    p = stats.t.sf(np.abs(t), np.maximum(nu, 1.0))
    return np.sign(t) * stats.norm.isf(p)


def check_profile(z, what):
    from scipy import stats
    z = np.ravel(z)
    m = z.size
    bound = max(3.0, float(stats.norm.isf(0.005 / m)))
    assert np.abs(z).max() <= bound, f"{what}: max |z| {np.abs(z).max():.2f} above {bound:.2f} ({m} cells)"
    frac = float(np.mean(np.abs(z) > 3))
    if m >= 100:
        assert frac <= 0.01, f"{what}: {frac:.2%} of {m} cells beyond 3 SE"
    return frac, float(np.abs(z).max())


def replicas(gmat, omat, dom, kind, n, dt, nsteps, prec, K):
    """R oracle (mt19937) and R GPU (Philox) solves of the same problem."""
    od = O.ODomain(dom)
    o = [O.solve(omat, od, kind, nemit=n, maxscat=10**6, dt=dt, horizon=dt * nsteps, rng=O.RNG_MT, nchunk=16,
                 seed=100 * s + 1)[0] for s in range(R)]
    P = {M.MULTI: M.MultiProblem, M.FLUX: M.FluxProblem}[kind](gmat, dom, n, 10**6)
    g = [P.solve(dt=dt, nsteps=nsteps, precision=prec, steps_per_launch=K, seed=5000 + s) for s in range(R)]
    return np.array(o), np.array(g)


def kappa_of(fields, dom, grad):
    vols = M.problem._handle(dom).cell_volumes()
    return np.array([-float(np.sum(f[1] * vols) / np.sum(vols)) / grad for f in fields])


@pytest.mark.parametrize("prec", [64, 32])
def test_cross_plane_film_statistics(prec, gmat, omat):
    """Config 0: 100 nm cross-plane film between isothermal walls at +1 K and
    -1 K about 300 K, 20 cells, 1e5 phonons, dt 1 ps x 2000 steps; kappa is
    the x-flux over the applied gradient -2 K / 100 nm."""
    dom = M.CrossPlaneFilmDomain(1e-7, 1e-7, 20)
    o, g = replicas(gmat, omat, dom, M.MULTI, 100_000, 1e-12, 2000, prec, 100)
    grad = -2.0 / 1e-7
    zk = welch_z(kappa_of(o, dom, grad), kappa_of(g, dom, grad))
    assert abs(zk) <= 3, zk
    check_profile(welch_z(o[:, 0], g[:, 0]), "temperature")
    check_profile(welch_z(o[:, 1], g[:, 1]), "x-flux")


def test_in_plane_film_statistics(gmat, omat):
    """Config 1 (FP32 flight), 20 cells across the 100 nm film, 15000 phonons,
    dt 0.5 ps x 1000 steps."""
    dom = M.FilmDomain.from_cli(1e-7, 1e-7, 20)
    o, g = replicas(gmat, omat, dom, M.MULTI, 15_000, 0.5e-12, 1000, 32, 100)
    grad = dom.ppeds[0].gradT[0]
    zk = welch_z(kappa_of(o, dom, grad), kappa_of(g, dom, grad))
    assert abs(zk) <= 3, zk
    check_profile(welch_z(o[:, 0], g[:, 0]), "temperature")
    check_profile(welch_z(o[:, 1], g[:, 1]), "x-flux")


def test_pore_cell_statistics(gmat, omat):
    """Config 2 (FP32 flight): the 500 nm periodic cell with the 250 nm pore,
    divisions 4 / 8 / 4 per block (16^3 - 8^3 = 3584 cells), 50000 phonons,
    dt 0.5 ps x 2000 steps; every cell of the temperature and x-flux fields,
    and the x-flux profile along the gradient (cells summed over y and z)."""
    dom = M.PoreCellDomain(5e-7, 2.5e-7, (4, 8, 4))
    o, g = replicas(gmat, omat, dom, M.MULTI, 50_000, 0.5e-12, 2000, 32, 100)
    grad = dom.ppeds[0].gradT[0]
    zk = welch_z(kappa_of(o, dom, grad), kappa_of(g, dom, grad))
    assert abs(zk) <= 3, zk
    assert o.shape[2] == 3584
    check_profile(welch_z(o[:, 0], g[:, 0]), "temperature")
    check_profile(welch_z(o[:, 1], g[:, 1]), "x-flux")
    # the profile along x: each x slab's volume-weighted x-flux
    vols = M.problem._handle(dom).cell_volumes()
    xs = slab_index(dom)
    prof = lambda f: np.array([[np.sum(r[1][xs == i] * vols[xs == i]) for i in range(xs.max() + 1)] for r in f])
    check_profile(welch_z(prof(o), prof(g)), "x-flux profile")


def slab_index(dom, nslab=16):
    """The x slab of every field column of a PoreCellDomain whose cells are
    all side / nslab wide along x (4 / 8 / 4 divisions): columns follow the
    subdomains in order, x fastest within one (montecarlo/field.cpp:87-90)."""
    out = []
    for p in dom.ppeds:
        d = [int(x) for x in p.divisions()]
        M_ = p.columns()
        xc = p.o[0] + (np.arange(d[0]) + 0.5) * M_[0, 0] / d[0]
        ii = np.tile(np.floor(xc / (dom.side / nslab)).astype(int), d[1] * d[2])
        out.append(ii)
    out = np.concatenate(out)
    assert out.size == M.problem._handle(dom).cols
    return out


# ----------------------------------------------------------- mismatch rate
# Measured FP32 discrete-mismatch rates: the fraction of trajectories that
# parted from the FP64 trajectory of the same uniform words at or before
# each horizon, the larger of two measurements on 10^4 phonons each (replay
# of the oracle's mt19937 stream over 2000 and over 4000 steps of 0.5 ps;
# the bench's `precision.discrete_mismatch` measures the same against the
# FP64 kernels over the whole 4000-step horizon). A rate measured as zero
# is taken as 1 / 10^4. Keys: the horizon in ns. These rates set the
# allowance of every FP32 trajectory comparison (test_gpu_parity.py).
MISMATCH_RATE = {
    "film": {0.125: 1e-4, 0.25: 2e-4, 0.5: 1.4e-3, 1.0: 6.5e-3, 1.5: 2.0e-2, 2.0: 4.3e-2},
    "pore": {0.125: 1e-4, 0.25: 1e-4, 0.5: 4e-4, 1.0: 1.1e-3, 1.5: 1.6e-3, 2.0: 3.1e-3},
    "cross": {0.25: 1e-4, 0.5: 1e-4, 1.0: 1e-4, 2.0: 1e-4},
}
MISMATCH_CASES = {  # domain, dt, dt-steps of each measured horizon
    "film": (lambda: M.FilmDomain.from_cli(1e-7, 1e-7, 100), 0.5e-12, (250, 500, 1000, 2000)),
    "pore": (lambda: M.PoreCellDomain(5e-7, 2.5e-7), 0.5e-12, (250, 500, 1000, 2000)),
    "cross": (lambda: M.CrossPlaneFilmDomain(1e-7, 1e-7, 20), 1e-12, (250, 500, 1000, 2000)),
}


def mismatch_allowance(name, horizon_s, n):
    """Trajectories of n that may differ over a horizon of horizon_s
    seconds: the 99.9% quantile of Binomial(n, measured rate), the rate of
    the first measured horizon at or beyond it (the film's for domains
    without a measurement of their own)."""
    from scipy import stats
    rates = MISMATCH_RATE.get(name, MISMATCH_RATE["film"])
    ns = horizon_s * 1e9
    h = min([x for x in rates if x >= ns * (1 - 1e-9)] or [max(rates)])
    return int(stats.binom.ppf(0.999, n, rates[h]))


@pytest.mark.parametrize("name", list(MISMATCH_CASES))
def test_fp32_discrete_mismatch_rate(name, gmat, omat):
    make, dt, horizons = MISMATCH_CASES[name]
    dom = make()
    n, nsteps, cap = 10_000, max(horizons), 320
    od = O.ODomain(dom)
    _, ost, ex = O.solve(omat, od, O.MULTI, nemit=n, maxscat=10**6, dt=dt, horizon=dt * nsteps, rng=O.RNG_MT,
                         nchunk=16, seed=3, record_cap=4096, log_cap=cap, log_phonons=n)
    olog = ex["log"]
    assert olog[1].max() < cap
    P = M.MultiProblem(gmat, dom, n, 10**6)
    # the words each phonon consumed in FP64, then padding: an FP32
    # trajectory that parts from it may draw more
    P.solve(dt=dt, nsteps=nsteps, precision=32, steps_per_launch=100,
            replay=O.record_to_replay(ex["record"], pad=4096), log_cap=cap, log_phonons=n)
    assert P.stats["status"] == 0
    tdiv = divergence_times(olog, P.log)
    rates = mismatch_rate(tdiv, [h * dt for h in horizons])
    print(f"{name}: FP32 mismatch rate at {horizons} steps of {dt:g} s: {rates}")
    for h, r in zip(horizons, rates):
        # the measured rate, with the binomial spread of 10^4 trajectories
        assert r * n <= mismatch_allowance(name, h * dt, n), (h, r)
    # the FP64 path replays the same words without a single mismatch
    P.solve(dt=dt, nsteps=nsteps, precision=64, steps_per_launch=100, replay=O.record_to_replay(ex["record"]),
            log_cap=cap, log_phonons=n)
    assert np.isinf(divergence_times(olog, P.log)).all()
