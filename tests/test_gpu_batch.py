"""Batching extension (ibm_batch_*): independent channels stepped together.

Each instance of a batch is a full context on its own stream; a batch step
queues every instance's step before waiting for any. The instances' results
must equal those of the same contexts stepped alone, bit for bit, whatever
mix of graph-captured and host-driven instances the batch holds, and an
instance that fails must not hide the others' results.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


def instances(ibm):
    # sizes in multiples of 16 with different cylinders and inflows, as the
    # ensemble workload draws them
    specs = [((96, 16, 16), dict(Um=0.8, Rcirc=0.04, ycirc=0.18)),
             ((128, 32, 16), dict(Um=1.6, Rcirc=0.06, ycirc=0.22)),
             ((64, 16, 32), dict(Um=0.3, Rcirc=0.05, ycirc=0.2))]
    return [ibm.Case(ibm.channel_params(*shape, dt=1e-3, **kw)) for shape, kw in specs]


def params(ibm, graph, precision=2):
    return ibm.solver_params(vel_tol=1e-10, p_tol=1e-10, precision=precision, use_graph=graph,
                             p_pc_rap_type=0, p_pc_relax_type=2, mg_omega=1.0, mg_group_ratio=1.5)


@pytest.mark.parametrize("graphs", [(1, 1, 1), (1, 0, 1)])
def test_batch_equals_instances_alone(ibm, graphs):
    cases = instances(ibm)
    prm = [params(ibm, g) for g in graphs]
    batch = ibm.Batch(cases, prm)
    alone = [ibm.Solver(c, p) for c, p in zip(cases, prm)]
    assert len(batch) == 3
    for step in range(1, 5):
        ramp = min(1.0, step / 3.0)
        sb = batch.step([ramp] * 3)
        for s, solver in zip(sb, alone):
            sa = solver.step(ramp)
            assert s.status == sa.status == ibm.IBM_OK
            for f in "uvwp":
                assert getattr(s, f).iters == getattr(sa, f).iters, f
            assert s.div_l2 == sa.div_l2
    for bs, solver in zip(batch.solvers, alone):
        for x, y, name in zip(bs.fields(), solver.fields(), "uvwp"):
            assert bits_equal(x, y), name
    batch.close()


def test_batch_reports_a_failing_instance(ibm):
    cases = instances(ibm)
    batch = ibm.Batch(cases, params(ibm, 1))
    u, v, w, p = cases[1].initial_fields()
    u = u.copy()
    nx, ny, nz = cases[1].shape
    i, j, k = 3 * nx // 4, ny // 2, nz // 2  # a fluid face far downstream of the cylinder
    u[(k * ny + j) * (nx + 1) + i] = np.nan
    batch.solvers[1].set_fields(u, v, w, p)
    with pytest.raises(ibm.IBMError) as e:
        batch.step(1.0)
    assert "instance 1" in str(e.value)
    # the other instances stepped and can step again
    for i in (0, 2):
        st = batch.solvers[i].step(1.0)
        assert st.status == ibm.IBM_OK
    batch.close()


def test_autotuned_batch_converges_to_the_same_fields(ibm):
    """The autotuner changes the multigrid schedule, not the tolerance: the
    tuned instances step to the untuned fields within the solves' tolerance."""
    import importlib
    at = importlib.import_module("ibm-3d-fpc_gb300.autotune")
    cases = instances(ibm)
    prm = [params(ibm, 1) for _ in cases]
    tuned = ibm.Batch(cases, prm)
    plain = ibm.Batch(cases, prm)
    applied, report = at.tune_batch(tuned.solvers, nbuckets=2, steps=2, warmup=1)
    assert all(a is not None for a in applied)
    assert any(r["trials"] for r in report.values())
    for _ in range(3):
        for st in tuned.step([1.0] * 3) + plain.step([1.0] * 3):
            assert st.status == ibm.IBM_OK
    for a, b in zip(tuned.solvers, plain.solvers):
        for x, y, name in zip(a.fields(), b.fields(), "uvwp"):
            assert np.abs(x - y).max() <= 1e-7 * max(np.abs(y).max(), 1e-30), name
    tuned.close()
    plain.close()
