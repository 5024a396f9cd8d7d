"""Multi-GPU form of bench.py (replicas only), checked on CPU: two gloo ranks
agree on the slowest rank's time, the whole-job value counts every rank's
transforms, and the reference arm runs on rank 0 alone."""
import os
import socket
import sys
import types

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import bench
    import torch.distributed as dist
    ws, r, _ = bench.dist_setup("gloo")
    ms = 10.0 + 5.0 * r                    # rank 1 is the slow one
    out[r] = (ws, bench.max_over_ranks(ms, ws))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_max():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert dict(out) == {0: (2, 15.0), 1: (2, 15.0)}


def test_replica_value_counts_all_ranks():
    import bench
    assert bench.replica_value(500.0, 100, 4) == pytest.approx(800.0)
    assert bench.max_over_ranks(3.0, 1) == 3.0


def test_reference_arm_only_on_rank_zero(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = types.SimpleNamespace(gpus=2, steps=5, warmup=3)
    assert bench.reference_arm(args, bench.WORKLOADS["plain"]) is None
    assert capsys.readouterr().out == ""


def test_reference_arm_line_has_contract_keys(monkeypatch, capsys):
    """Rank 0 of `bench.py --impl reference` prints one JSON line with the
    contract's keys: the reference's CPU pipeline (the oracle's restatement)
    timed on the host, its cpu_baseline description and an e2e object
    without device copies, on the plain workload (N = 1e4, a few seconds)."""
    import json
    import bench
    monkeypatch.setenv("RANK", "0")
    monkeypatch.setenv("WORLD_SIZE", "1")
    args = types.SimpleNamespace(gpus=1, steps=3, warmup=1)
    bench.reference_arm(args, bench.WORKLOADS["plain"])
    out = [l for l in capsys.readouterr().out.splitlines() if l.startswith("{")]
    assert len(out) == 1
    line = json.loads(out[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["value"] > 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
