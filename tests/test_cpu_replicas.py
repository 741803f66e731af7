"""The multi-GPU form is replicas: bench.py under torchrun runs one
independent box per rank and reports the whole job's updates/s timed by the
slowest rank.  The rank aggregation runs here as two gloo processes on CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank: int, world: int, port: int, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = [7.5, 9.25][rank]                     # the second replica is slower
    got = bench.max_over_ranks(ms, dist, "cpu")
    out[rank] = (got, bench.replica_value(1000, world, got))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_time_by_slowest_rank():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
    for r in range(world):
        got, value = out[r]
        assert got == 9.25
        assert value == pytest.approx(world * 1000 / 9.25e-3)


def test_single_process_passes_through():
    assert bench.max_over_ranks(3.0, None, "cpu") == 3.0
    assert bench.replica_value(2_097_152, 1, 6.0) == pytest.approx(2_097_152 / 6e-3)


def test_batched_cpu_baseline_spreads_tubes_over_processes():
    """The batched workload's host baseline: every sampled tube is stepped
    once by one process, and the rate counts each tube's particles x steps."""
    from ndspmhd_gb300 import configs
    counts = [200, 300, 450]
    res = bench.cpu_batched_baseline(counts, 4, 1, ntubes=3)
    n = sum(configs.brio_wu_tube(c)[1]["x"].shape[0] for c in counts)
    assert res["kind"] == "port" and res["cores"] >= 1 and res["value"] > 0
    assert f"({n} particles)" in res["sample"]
    upd, el = bench._cpu_tube_worker(([counts[0]], 4, 1))
    assert upd == configs.brio_wu_tube(counts[0])[1]["x"].shape[0] * 4 and el > 0


def test_reference_arm_line(monkeypatch, capsys):
    """`bench.py --impl reference` prints one JSON line with the native arm's
    metric and unit, its CPU sample described in cpu_baseline and an e2e
    object with no host-device bytes; ranks other than 0 print nothing."""
    import argparse
    import json
    monkeypatch.setattr(bench, "CPU_SAMPLE_N1D", 8)
    monkeypatch.setattr(bench.os, "cpu_count", lambda: 2)
    args = argparse.Namespace(gpus=2, steps=1, warmup=0)
    monkeypatch.setenv("RANK", "1")
    bench.reference_arm(args)
    assert capsys.readouterr().out == ""
    monkeypatch.setenv("RANK", "0")
    bench.reference_arm(args)
    lines = [ln for ln in capsys.readouterr().out.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["higher_is_better"] is True and d["n_gpus"] == 2
    assert d["value"] > 0 and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["cores"] == 2 and d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"] == {"value": d["value"], "unit": bench.UNIT, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
