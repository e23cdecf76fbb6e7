"""Replica bookkeeping of bench.py at world size 2 (gloo, CPU ranks).

The path does not shard across GPUs with a collective: N GPUs run N
independent replicas, and the job's time is the slowest rank's.  This covers
the host-side reduction that every rank runs, and that ranks other than 0
print nothing for the reference arm.
"""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.replica_max_ms(10.0 + 5.0 * rank, world)
    val = bench.job_tflops(2.0e12, world, ms)
    dist.destroy_process_group()
    Path(out, f"r{rank}.json").write_text(json.dumps({"ms": ms, "value": val}))


def test_max_over_ranks_and_whole_job_value(tmp_path):
    import torch.multiprocessing as mp
    port = 29000 + os.getpid() % 1000
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn")
    res = [json.loads(Path(tmp_path, f"r{r}.json").read_text()) for r in range(2)]
    for r in res:
        assert r["ms"] == 15.0                             # the slower rank's time on both ranks
        assert abs(r["value"] - 2 * 2.0e12 / 15e-3 / 1e12) < 1e-9


def test_reference_arm_prints_only_on_rank_0():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--size", "256",
                        "--steps", "1", "--warmup", "1"], capture_output=True, text=True, env=env, timeout=120)
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""


def test_reference_arm_line_on_rank_0():
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    p = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--size", "256",
                        "--steps", "2", "--warmup", "1"], capture_output=True, text=True, env=env, timeout=300)
    assert p.returncode == 0, p.stderr
    line = json.loads(p.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["value"] > 0
