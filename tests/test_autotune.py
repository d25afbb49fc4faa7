"""Autotuner logic on the CPU (no GPU): candidate selection with a fake
solver and clock, failing candidates never chosen, size classes, the cache.
The GPU side (tuning real contexts) is in tests/test_gpu_batch.py."""
import importlib

import numpy as np
import pytest


@pytest.fixture(scope="module")
def at():
    return importlib.import_module("ibm-3d-fpc_gb300.autotune")


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t


class FakeSolver:
    """Step cost = a function of the multigrid knobs; mg_coarse_max 640 fails."""

    def __init__(self, ibm, clock, shape=(96, 16, 16)):
        self.ibm = ibm
        self.clock = clock
        self.params = ibm._native.SolverParams()
        self.params.precision = 2
        self.case = type("C", (), {"shape": shape})()
        self.state = 0.0

    def set_params(self, p):
        self.params = p

    def fields(self):
        return (self.state,)

    def set_fields(self, *f):
        self.state = f[0]

    def step(self, ramp):
        p = self.params
        self.clock.t += 1e-3 * (p.mg_nu1 + p.mg_nu2 + 0.5 * p.mg_nu_coarse + (2 if not p.mg_quads else 0))
        self.state += 1.0
        st = self.ibm.StepStats()
        if p.mg_coarse_max == 640:
            st.status = -3
        return st


def test_tune_picks_the_fastest_valid_candidate(ibm, at, monkeypatch):
    clock = FakeClock()
    monkeypatch.setattr(at.time, "perf_counter", clock)
    s = FakeSolver(ibm, clock)
    s.state = 5.0
    best, trials = at.tune(s)
    assert best == dict(mg_coarse_max=2560, mg_nu1=2, mg_nu2=2, mg_nu_coarse=1, mg_quads=1)
    assert len(trials) == len(at.CANDIDATES)
    assert [t[2] for t in trials].count(-3) == 1
    # the chosen overrides are set and the fields restored
    assert (s.params.mg_nu1, s.params.mg_nu2, s.params.mg_nu_coarse) == (2, 2, 1)
    assert s.state == 5.0
    assert s.params.precision == 2


def test_size_classes_and_cache(ibm, at, tmp_path, monkeypatch):
    cls = at.size_classes([96 * 16 * 16, 128 * 16 * 16, 256 * 48 * 48, 240 * 48 * 32, 160 * 32 * 32], 4)
    assert cls.min() == 0 and cls.max() == 3
    assert cls[0] <= cls[1] <= cls[4] <= cls[3] <= cls[2]
    assert at.size_classes([1000, 1000], 4).tolist() == [0, 0]
    path = str(tmp_path / "tune.json")
    c = at.TuneCache(path)
    c.put((96, 16, 16), 2, {"mg_nu1": 2})
    assert at.TuneCache(path).get((96, 16, 16), 2) == {"mg_nu1": 2}
    assert at.TuneCache(path).get((96, 16, 16), 0) is None
    # tune_batch: one representative per class, a cached shape is not re-tuned
    clock = FakeClock()
    monkeypatch.setattr(at.time, "perf_counter", clock)
    solvers = [FakeSolver(ibm, clock, sh) for sh in ((96, 16, 16), (96, 16, 16), (256, 48, 48))]
    applied, report = at.tune_batch(solvers, nbuckets=2, cache=c)
    assert applied[0] == {"mg_nu1": 2} == applied[1]  # from the cache
    assert report[0]["trials"] is None
    assert applied[2]["mg_nu_coarse"] == 1 and report[1]["trials"] is not None
    assert at.TuneCache(path).get((256, 48, 48), 2) == applied[2]
