"""The N > 1 host path of bench.py on CPU: two ranks over gloo (127.0.0.1).

The hot path does not shard (replicas only): every rank advances its own
seeded mesh, and the ranks meet only at the barriers around the timed region,
in the maximum of their times, and in rank 0's single output line. These
tests run that host logic with world size 2 and no GPU.
"""
from __future__ import annotations

import json
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import bench
    r, w, local = bench.dist_info()
    bench.init_replicas(w)
    import torch.distributed as dist
    backend = dist.get_backend()
    bench.barrier(w)
    # rank r "took" 10 + 5 r ms: every rank sees the slowest
    slowest = bench.max_over_ranks(10.0 + 5.0 * r, w)
    # whole-job value: the units of all ranks over the slowest rank's time
    cells, steps = 1000, 4
    value = cells * steps * w / (slowest * 1e-3)
    printed = bench.emit({"rank": r, "value": value}, r)
    bench.barrier(w)
    bench.finish_replicas(w)
    Path(out_dir, f"rank{r}.json").write_text(json.dumps(
        {"rank": r, "world": w, "local": local, "backend": backend, "slowest": slowest, "value": value,
         "printed": printed}))


def test_two_replicas_over_gloo(tmp_path):
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    res = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(world)]
    assert [x["rank"] for x in res] == [0, 1] and all(x["world"] == 2 for x in res)
    assert [x["local"] for x in res] == [0, 1]
    assert all(x["backend"] == "gloo" for x in res)
    assert all(x["slowest"] == 15.0 for x in res)
    assert res[0]["value"] == res[1]["value"] == pytest.approx(1000 * 4 * 2 / 15e-3)
    assert [x["printed"] for x in res] == [True, False]


def test_single_process_needs_no_group(capsys):
    sys.path.insert(0, str(ROOT))
    import bench
    bench.init_replicas(1)
    bench.barrier(1)
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.emit({"x": 1}, 0) is True
    assert bench.emit({"x": 2}, 1) is False
    out = capsys.readouterr().out.strip().splitlines()
    assert out == ['{"x": 1}']
    bench.finish_replicas(1)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    """Under torchrun the reference arm's other ranks exit without work."""
    sys.path.insert(0, str(ROOT))
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    args = bench.parse()
    bench.run_reference(args)
    assert capsys.readouterr().out == ""
