"""Autotuner of the solver schedule for a channel or a batched ensemble.

The knobs are the multigrid V-cycle's depth and work and the shape of its
kernels:
- mg_coarse_max: the largest level solved directly;
- mg_nu1 / mg_nu2 / mg_nu_coarse: the sweeps on the finest and the coarser
  levels;
- mg_quads: four points of a line per thread, or one;
- mg_fused_sweep: a 7-point level's two colour phases as one kernel over
  64 x 8 x 8 shared-memory tiles with a halo, or one grid-stride launch per
  phase;
- mg_fused_coarse: the coarse end of the V-cycle as one persistent
  cooperative kernel (from the first level of at most that many points), or
  one launch per phase. On small grids, whose phases are bound by launch
  latency, the fused forms can win; on the 640x128x128 channel they do not.
Every candidate solves to the same tolerances, so the choice changes the time
per step and nothing else. It is measured on the GPU: host wall time of
graph-captured steps, each waiting for its results, from the context's own
fields, which are restored after every trial.

An ensemble is tuned by size class. Instances are bucketed by cell count
(log-spaced buckets), the median instance of each bucket is tuned, and the
winner applies to the whole bucket. A cache keyed by grid shape and precision
(JSON on disk, optional) skips tuning a shape that was tuned before.
"""
from __future__ import annotations

import copy
import json
import os
import time
from typing import Iterable, Optional

import numpy as np

CANDIDATES = (
    dict(mg_coarse_max=2560, mg_nu1=3, mg_nu2=3, mg_nu_coarse=2, mg_quads=1),
    dict(mg_coarse_max=640, mg_nu1=3, mg_nu2=3, mg_nu_coarse=2, mg_quads=1),
    dict(mg_coarse_max=2560, mg_nu1=2, mg_nu2=2, mg_nu_coarse=2, mg_quads=1),
    dict(mg_coarse_max=2560, mg_nu1=2, mg_nu2=2, mg_nu_coarse=1, mg_quads=1),
    dict(mg_coarse_max=2560, mg_nu1=3, mg_nu2=3, mg_nu_coarse=2, mg_quads=0),
    dict(mg_coarse_max=2560, mg_nu1=3, mg_nu2=3, mg_nu_coarse=2, mg_quads=1, mg_fused_sweep=1),
    dict(mg_coarse_max=2560, mg_nu1=3, mg_nu2=3, mg_nu_coarse=2, mg_quads=1, mg_fused_coarse=1 << 30),
    dict(mg_coarse_max=2560, mg_nu1=3, mg_nu2=3, mg_nu_coarse=2, mg_quads=1, mg_fused_sweep=1,
         mg_fused_coarse=1 << 30),
)


def with_overrides(params, overrides: dict):
    p = copy.copy(params)
    for k, v in overrides.items():
        if not hasattr(p, k):
            raise AttributeError(f"SolverParams has no field {k!r}")
        setattr(p, k, v)
    return p


def tune(solver, candidates: Iterable[dict] = CANDIDATES, steps: int = 3, warmup: int = 1, ramp: float = 1.0):
    """Times each candidate on the solver's context and leaves the fastest
    one set. Returns (best overrides, [(ms per step, overrides, worst status,
    pressure iterations)]). Candidates whose steps fail are never chosen."""
    base = copy.copy(solver.params)
    fields = solver.fields()
    trials = []
    for cand in candidates:
        solver.set_params(with_overrides(base, cand))
        solver.set_fields(*fields)
        worst, p_iters = 0, 0
        try:
            for _ in range(warmup):
                solver.step(ramp)
            t0 = time.perf_counter()
            for _ in range(steps):
                st = solver.step(ramp)
                if worst >= 0:  # an error (negative) outranks IBM_NOT_CONVERGED (1)
                    worst = st.status if st.status < 0 else max(worst, st.status)
                p_iters = st.p.iters
            ms = (time.perf_counter() - t0) / steps * 1e3
        except RuntimeError:
            ms, worst = float("inf"), -1
        trials.append((ms, dict(cand), worst, p_iters))
    ok = [t for t in trials if t[2] == 0]
    best = min(ok, key=lambda t: t[0])[1] if ok else {}
    solver.set_params(with_overrides(base, best))
    solver.set_fields(*fields)
    return best, trials


class TuneCache:
    """Tuned overrides keyed by (nx, ny, nz, precision); optional JSON file."""

    def __init__(self, path: Optional[str] = None):
        self.path = path
        self.entries: dict = {}
        if path and os.path.exists(path):
            with open(path) as f:
                self.entries = json.load(f)

    @staticmethod
    def key(shape, precision) -> str:
        return "x".join(str(int(s)) for s in shape) + f"/p{int(precision)}"

    def get(self, shape, precision):
        return self.entries.get(self.key(shape, precision))

    def put(self, shape, precision, overrides: dict) -> None:
        self.entries[self.key(shape, precision)] = dict(overrides)
        if self.path:
            with open(self.path, "w") as f:
                json.dump(self.entries, f, indent=1, sort_keys=True)


def size_classes(cells, nbuckets: int = 4):
    """Bucket index of each instance: log-spaced buckets over the cell counts."""
    cells = np.asarray(cells, dtype=np.float64)
    lo, hi = np.log(cells.min()), np.log(cells.max())
    if hi - lo < 1e-12:
        return np.zeros(cells.size, dtype=int)
    return np.minimum(((np.log(cells) - lo) / (hi - lo) * nbuckets).astype(int), nbuckets - 1)


def tune_batch(solvers, nbuckets: int = 4, cache: Optional[TuneCache] = None, **kw):
    """Tunes an ensemble by size class (the solvers of a Batch, or any list).
    Returns the overrides applied to each instance and the per-class trials."""
    shapes = [s.case.shape for s in solvers]
    cells = [int(np.prod(sh)) for sh in shapes]
    cls = size_classes(cells, nbuckets)
    applied = [None] * len(solvers)
    report = {}
    for b in sorted(set(cls.tolist())):
        members = [i for i in range(len(solvers)) if cls[i] == b]
        rep = sorted(members, key=lambda i: cells[i])[len(members) // 2]
        prec = solvers[rep].params.precision
        best = cache.get(shapes[rep], prec) if cache else None
        trials = None
        if best is None:
            best, trials = tune(solvers[rep], **kw)
            if cache:
                cache.put(shapes[rep], prec, best)
        for i in members:
            solvers[i].set_params(with_overrides(solvers[i].params, best))
            applied[i] = best
        report[int(b)] = {"representative": list(shapes[rep]), "instances": len(members), "chosen": best,
                          "trials": None if trials is None else
                          [{"ms": t[0], "overrides": t[1], "status": t[2], "p_iters": t[3]} for t in trials]}
    return applied, report
