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
