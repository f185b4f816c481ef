"""The multi-rank path of bench.py on CPU: two gloo ranks reduce their step
times to the slowest one, the job rate counts every rank's instances, and the
reference arm runs on rank 0 only."""
import os
import sys
from pathlib import Path

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _worker(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = bench.max_over_ranks(dist, [10.0 + rank, 5.0 - rank], "cpu")
    out[rank] = ms + [bench.job_rate(world, 256, ms[0])]
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_to_slowest():
    world = 2
    port = 29500 + os.getpid() % 1000
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        assert res[r][0] == 11.0 and res[r][1] == 5.0
        assert res[r][2] == pytest.approx(2 * 256 / 0.011)


def test_reference_arm_is_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, str(ROOT))
    import bench

    class Args:
        workload, batch, cpu_threads, warmup, steps, ref_max_steps = "film2d", 1, 1, 0, 1, 1

    called = []
    monkeypatch.setattr(bench, "cpu_sample", lambda *a, **k: called.append(1) or (1.0, 1.0))
    bench.run_reference(Args, rank=1, world=2)
    assert not called and capsys.readouterr().out == ""


def test_reference_arm_line(tmp_path):
    """bench.py --impl reference times the CPU restatement of SCFT.c and prints
    the contract's line: the same metric and unit, a cpu_baseline describing
    the run, and an e2e with no host-device bytes."""
    import json
    import subprocess
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "bulk2d",
                          "--batch", "2", "--steps", "1", "--warmup", "0", "--cpu-threads", "2"],
                         cwd=ROOT, capture_output=True, text=True, timeout=300, check=True).stdout
    line = json.loads(out.strip().splitlines()[-1])
    import bench
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC
    assert line["value"] > 0 and line["unit"] == "instance-iterations/s" and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] == 2
    assert line["cpu_baseline"]["value"] == line["value"]
    # the line states the steps it timed
    assert line["steps"] == 1 and line["warmup"] == 0
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
