"""Project autotuner for the advance kernels' launch parameters.

tune(): dt-steps per launch (the compaction / sort interval), block size and
tally layout of a single solve, on a reduced copy of the workload (fewer
phonons), timing device-resident solves with CUDA events.
tune_batch(): block size and dt-steps per launch of a batched solve, on a
copy of the batch with a fraction of each instance's phonons, timing the
replayed CUDA graph.
Both return the fastest configuration; results are cached per workload
signature for the process.
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


def tune_batch(problems, *, dt, nsteps, precision=32, blocks=(128, 256), Ks=(0, 1000), scale=0.1,
               min_nemit=1000, reps=2):
    """Return (best {"block_size", "steps_per_launch"}, list of (config,
    phonon-steps/s)) for a batch of the given problems (steps_per_launch 0:
    the whole horizon in one launch)."""
    import torch

    from .batch import Batch
    from .problem import CUMFLUX, CUMTEMP, FLUX, MULTI, TEMP, CumFluxProblem, CumTempProblem, FluxProblem, \
        MultiProblem, TempProblem
    key = ("batch", tuple((type(p.dom).__name__, p.nemit_requested, p.kind) for p in problems), dt, nsteps,
           precision)
    if key in _cache:
        return _cache[key]
    cls = {TEMP: TempProblem, FLUX: FluxProblem, MULTI: MultiProblem}
    small = []
    for p in problems:
        n = max(min_nemit, int(p.nemit_requested * scale))
        if p.kind in (CUMTEMP, CUMFLUX):
            c = CumTempProblem if p.kind == CUMTEMP else CumFluxProblem
            small.append(c(p.mat, p.dom, n, p.size, p.maxscat, p.maxloop))
        else:
            small.append(cls[p.kind](p.mat, p.dom, n, p.maxscat, p.maxloop))
    results = []
    for b, K in itertools.product(blocks, Ks):
        if K > nsteps:
            continue
        B = Batch(small, dt=dt, nsteps=nsteps, precision=precision, steps_per_launch=K, block_size=b,
                  use_graph=True)
        B.run()
        torch.cuda.synchronize()
        best = None
        for _ in range(reps):
            t0 = time.perf_counter()
            B.run()
            st = B.stats()  # synchronises
            rate = st["phonon_steps"] / (time.perf_counter() - t0)
            best = rate if best is None else max(best, rate)
        B.close()
        results.append(({"block_size": b, "steps_per_launch": K}, best))
    cfg = max(results, key=lambda x: x[1])[0]
    _cache[key] = (cfg, results)
    return cfg, results
