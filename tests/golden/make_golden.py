"""Generate the golden fixtures of the oracle (tests/golden/*.json).

The reference (montecarlocpp) cannot be built here (it needs Eigen 3 and
Boost) and ships no golden vectors, so these fixtures record the oracle's own
outputs on small cases: the field, the stop counters and the first phonons'
event logs. The GPU tests compare against the oracle directly; these files
pin the oracle itself across compilers and machines.

Run:  python tests/golden/make_golden.py
"""

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

CASES = {
    "oracle_film_multi": dict(domain="film", problem=2, nemit=400, maxscat=10**6, dt=0.5e-12, nsteps=300,
                              rng=0, seed=0, nchunk=2),
    "oracle_cross_temp": dict(domain="cross", problem=0, nemit=400, maxscat=10**6, dt=1e-12, nsteps=2000,
                              rng=1, seed=11, nchunk=1),
    "oracle_pore_multi": dict(domain="pore", problem=2, nemit=300, maxscat=10**6, dt=0.5e-12, nsteps=200,
                              rng=1, seed=5, nchunk=1),
}


def domain(name):
    import montecarlocpp_gb300 as M
    if name == "film":
        return M.FilmDomain.from_cli(1e-7, 1e-7, 20)
    if name == "cross":
        return M.CrossPlaneFilmDomain(1e-7, 1e-7, 20)
    if name == "pore":
        return M.PoreCellDomain(5e-7, 2.5e-7, (3, 6, 3))
    raise KeyError(name)


def run_case(c, omat):
    from oracle import oracle as O
    od = O.ODomain(domain(c["domain"]))
    out, st, ex = O.solve(omat, od, c["problem"], nemit=c["nemit"], maxscat=c["maxscat"], dt=c["dt"],
                          horizon=c["dt"] * c["nsteps"], rng=c["rng"], seed=c["seed"], nchunk=c["nchunk"],
                          nthreads=2, log_cap=64, log_phonons=8)
    log, counts = ex["log"]
    return {"case": c, "field": out.tolist(),
            "stats": {k: st[k] for k in ("nemit", "events", "scatters", "absorbed", "horizon_stops",
                                          "maxscat_stops", "escapes", "phonon_steps")},
            "log_counts": [int(x) for x in counts],
            "log": [[r for r in log[i, :min(int(counts[i]), 64)].tolist()] for i in range(len(counts))]}


def main():
    from montecarlocpp_gb300 import silicon_tables
    from oracle import oracle as O
    omat = O.OMaterial(*silicon_tables(), 300.0)
    for name, c in CASES.items():
        r = run_case(c, omat)
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump(r, f)
        print(name, r["stats"])


if __name__ == "__main__":
    main()
