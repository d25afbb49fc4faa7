"""The multi-GPU form of bench.py runs independent replicas (a single channel
does not shard): each rank times its own steps, the job's time is the max
over ranks, and the whole-job value is ranks x steps over that time. This
checks the aggregation with two gloo ranks on the CPU, and that the
reference arm leaves ranks other than 0 idle."""
import importlib.util
import os
import socket
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=ws)
    try:
        b = _bench()
        ms = b.reduce_max_ms(10.0 * (rank + 1), ws, "cpu")
        out[rank] = (ms, b.replica_throughput(5, ms, ws))
    finally:
        dist.destroy_process_group()


def test_replica_timing_takes_the_slowest_rank():
    ws = 2
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(ws, _free_port(), out), nprocs=ws, join=True)
    for r in range(ws):
        ms, value = out[r]
        assert ms == 20.0
        assert value == pytest.approx(ws * 5 / 0.020)


def test_single_rank_is_unchanged():
    b = _bench()
    assert b.reduce_max_ms(7.5, 1, "cpu") == 7.5
    assert b.replica_throughput(4, 8.0, 1) == pytest.approx(500.0)


def test_reference_arm_idle_on_other_ranks(monkeypatch, capsys):
    b = _bench()
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"])
    b.reference_arm(b.parse())
    assert capsys.readouterr().out == ""


@pytest.mark.parametrize("ws", [1, 2, 3, 8])
def test_ensemble_shards_cover_every_instance_once(ws):
    """The batched ensemble shards by instance: every instance lands on
    exactly one rank and the cell counts are balanced to within the largest
    instance."""
    b = _bench()
    specs = b.ensemble_cases(None, 32)
    shards = [b.shard_by_cells(specs, ws, r) for r in range(ws)]
    flat = sorted(i for s in shards for i in s)
    assert flat == list(range(len(specs)))
    cells = [sum(specs[i][0] * specs[i][1] * specs[i][2] for i in s) for s in shards]
    largest = max(nx * ny * nz for nx, ny, nz, *_ in specs)
    assert max(cells) - min(cells) <= largest
    for nx, ny, nz, d, yc, um in specs:
        assert 96 <= nx <= 256 and 16 <= ny <= 48 and 16 <= nz <= 48
        assert nx % 16 == ny % 16 == nz % 16 == 0
        assert 0.06 <= d <= 0.14 and 0.15 <= yc <= 0.26 and 0.2 <= um <= 2.25


def test_ensemble_accuracy_summary():
    """The ensemble's accuracy record: per-instance velocity differences
    relative to the reference set's largest velocity, against FP64 at the
    same tolerances and both forms against the tighter truth."""
    import numpy as np
    b = _bench()
    rng = np.random.default_rng(3)
    truth = [[rng.standard_normal(50) for _ in range(4)] for _ in range(3)]
    fp64 = [[x + d for x in t] for t, d in zip(truth, (1e-7, 5e-6, 2e-7))]
    mixed = [[x + d for x in t] for t, d in zip(truth, (3e-7, 2e-6, 4e-6))]
    acc = b.ensemble_accuracy(mixed, fp64, truth)
    scale = [max(float(np.abs(x).max()) for x in t[:3]) for t in truth]
    assert np.allclose(acc["mixed_vs_fp64_tight"], [3e-7 / scale[0], 2e-6 / scale[1], 4e-6 / scale[2]])
    assert np.allclose(acc["fp64_vs_fp64_tight"], [1e-7 / scale[0], 5e-6 / scale[1], 2e-7 / scale[2]])
    assert acc["mixed_vs_fp64_tight_max"] == max(acc["mixed_vs_fp64_tight"])
    assert len(acc["velocity_rel_err_vs_fp64"]) == 3
    # instance 0: within 1e-6; 1: within FP64's own error; 2: neither
    assert acc["instances_mixed_within_fp64_error"] == 2
    # the pressure (index 3) does not enter the velocity differences
    mixed[0][3] = mixed[0][3] + 1.0
    assert b.ensemble_accuracy(mixed, fp64, truth)["mixed_vs_fp64_tight"][0] == acc["mixed_vs_fp64_tight"][0]
