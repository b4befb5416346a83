"""bench.py with N > 1 ranks runs N independent replicas of the workload (the
solve path does not shard): rank 0 reports N solves per step over the slowest
rank's time per step.  The aggregation is checked with two gloo ranks on CPU."""
import json
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_path):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = [20.0, 25.0][rank]
    line = {"metric": "m", "value": 1e3 / ms, "unit": "solves/s", "n_gpus": 1, "steps": 10, "ms_per_step": ms,
            "p50_ms": ms, "p99_ms": ms + 1, "e2e": {"value": 1e3 / (ms + 0.5), "unit": "solves/s"},
            "config": {"workload": "w", "parallelism": "replicas only"}, "cpu_baseline": {"value": 0.3}}
    out = bench.combine_replicas(line)
    if rank == 0:
        with open(out_path, "w") as f:
            json.dump(out, f)
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank(tmp_path):
    out_path = str(tmp_path / "line.json")
    mp.start_processes(_rank, args=(2, _free_port(), out_path), nprocs=2, join=True, start_method="spawn")
    line = json.load(open(out_path))
    assert line["n_gpus"] == 2
    assert line["ms_per_step"] == 25.0 and line["p99_ms"] == 26.0
    assert line["value"] == pytest.approx(2 * 1e3 / 25.0, rel=1e-3)
    assert line["e2e"]["value"] == pytest.approx(2 * 1e3 / 25.5, rel=1e-3)
    assert line["per_rank_value"] == pytest.approx([50.0, 40.0])
    assert line["cpu_baseline"] is None
    assert "2 independent replicas" in line["config"]["parallelism"]
