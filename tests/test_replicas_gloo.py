"""bench.py's multi-process path (replicas) on two gloo ranks, on the CPU.

The render-and-fit path runs as independent replicas, one per GPU; what bench.py adds
for N > 1 is host logic: the process group from the torchrun environment, the barrier
around the timed region, the maximum of the ranks' times, rank 0 alone printing, and the
reference arm running on rank 0 only while the other ranks exit without work.
"""

from __future__ import annotations

import json
import os
import socket
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, folder):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))  # fmt: skip
    sys.path.insert(0, str(ROOT))
    import bench
    import torch

    calls = []

    def fake_baseline(threads=None):
        calls.append(threads)
        return {"value": 0.5, "unit": "steps/s", "cores": 1, "kind": "port", "sample": "stub"}

    bench.full_refit_baseline = fake_baseline
    got_world, got_rank, local = bench._distributed()
    bench._barrier(got_world)
    slowest = bench._max_over_ranks(1.5 + got_rank, got_world, torch.device("cpu"))
    args = bench.argparse.Namespace(steps=3, warmup=1, cpu_threads=None)
    result = bench.run_reference(args, got_world, got_rank)
    bench._barrier(got_world)
    torch.distributed.destroy_process_group()
    record = {"world": got_world, "rank": got_rank, "local": local, "slowest": slowest, "calls": len(calls),
              "result": result}  # fmt: skip
    (Path(folder) / f"rank{rank}.json").write_text(json.dumps(record))


@pytest.mark.timeout(300)
def test_two_gloo_replicas_share_the_slowest_time_and_rank0_reports(tmp_path):
    world = 2
    mp.start_processes(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn",
                       join=True)  # fmt: skip
    records = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(world)]
    for r, record in enumerate(records):
        assert record["world"] == world and record["rank"] == r and record["local"] == r
        assert record["slowest"] == 2.5  # max over ranks of 1.5 + rank
    assert records[0]["calls"] == 1 and records[1]["calls"] == 0  # the CPU arm runs once, on rank 0
    assert records[1]["result"] is None
    line = records[0]["result"]
    assert line["impl"] == "reference" and line["n_gpus"] == world and line["value"] == 0.5
    assert line["e2e"] == {"value": 0.5, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
