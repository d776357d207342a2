"""The multi-process (N > 1) paths of bench.py, on the CPU with gloo.

Each GPU runs an independent replica of the workload (the step has no
exchange between grids), so the only collectives are the barrier around the
timed region and the maximum of the per-rank times.  These tests run two
ranks on the CPU:

* max_over_ranks and barrier across two gloo processes;
* the reference arm launched as torch.distributed.run does it: rank 0 runs
  and prints one JSON line, the other rank exits 0 without work.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, values, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(world)
        m = bench.max_over_ranks(values[rank], world)
        bench.barrier(world)
    finally:
        dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(repr(m))


def test_max_over_ranks_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    values = [3.25, 7.5]
    mp.start_processes(_rank_main, args=(2, _free_port(), values, str(tmp_path)), nprocs=2,
                       join=True, start_method="spawn")
    for r in range(2):
        assert float((tmp_path / f"rank{r}.txt").read_text()) == max(values)


def test_reference_arm_under_torchrun(tmp_path):
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
           "--steps", "2", "--warmup", "1", "--size", "64"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    p = subprocess.run(cmd, cwd=str(tmp_path), stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                       text=True, timeout=600, env=env)
    assert p.returncode == 0, p.stderr[-3000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["steps"] == 2
    assert d["value"] > 0 and d["e2e"]["value"] == d["value"]
