"""Project autotuner for the advance kernel's launch parameters.

Searches dt-steps per launch (the compaction / sort interval), block size and
tally layout on a reduced copy of the workload (fewer phonons, a shortened
horizon), timing device-resident solves with CUDA events, and returns the
fastest. Results are cached per workload signature for the process.
"""

from __future__ import annotations

import itertools
import time

_cache = {}


def _time_config(prob, W, stream, nemit, nsteps, K, block, tally, precision=32, reps=2):
    import torch

    from .problem import MultiProblem
    p = MultiProblem(prob.mat, prob.dom, nemit, W["maxscat"])
    s = p.session(dt=W["dt"], nsteps=nsteps, precision=precision, steps_per_launch=K, seed=99,
                  block_size=block, tally_mode=tally, stream=stream.cuda_stream)
    s.run()
    s.result(field=False)
    best = None
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.run()
        e1.record(stream)
        torch.cuda.synchronize()
        _, st = s.result(field=False)
        rate = st["phonon_steps"] / (e0.elapsed_time(e1) * 1e-3)
        best = rate if best is None else max(best, rate)
    s.close()
    return best


def tune(prob, W, stream, Ks=(50, 200, 1000, 4000), blocks=(128, 256), tallies=(0,),
         nemit=None, nsteps=None, precision=32, budget_s=60.0):
    """Return (best config dict, list of (config, rate))."""
    key = (type(prob.dom).__name__, tuple(sorted((k, str(v)) for k, v in W.items())), precision)
    if key in _cache:
        return _cache[key]
    nemit = nemit or min(W["nemit"], 1_000_000)
    nsteps = nsteps or W["nsteps"]
    results = []
    t0 = time.time()
    for K, b, t in itertools.product(Ks, blocks, tallies):
        if K > nsteps:
            continue
        r = _time_config(prob, W, stream, nemit, nsteps, K, b, t, precision)
        results.append(({"steps_per_launch": K, "block_size": b, "tally_mode": t}, r))
        if time.time() - t0 > budget_s:
            break
    best = max(results, key=lambda x: x[1])[0]
    _cache[key] = (best, results)
    return best, results


def best_steps_per_launch(prob, W, stream):
    best, _ = tune(prob, W, stream, blocks=(256,))
    return best["steps_per_launch"]
