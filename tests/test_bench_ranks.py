"""bench.py's multi-rank plumbing on CPU, world size 2 over gloo.

The path is not sharded: under torchrun every rank runs its own lattice, and
the ranks meet only at a barrier and a max over their timings.  These tests
run those helpers on two gloo ranks, and the reference arm under torchrun,
where rank 0 alone measures and prints one JSON line.
"""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, port: int, out_dir: str):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": "2",
                       "RANK": str(rank), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, str(ROOT))
    import bench
    ws, r, local = bench.dist_env()
    bench.dist_init(ws, "gloo")
    bench.dist_barrier(ws)
    mx = bench.dist_max(ws, 1.5 + r)
    sm = bench.dist_sum(ws, 1.5 + r)
    bench.dist_barrier(ws)
    Path(out_dir, f"rank{r}.json").write_text(json.dumps({"ws": ws, "rank": r, "local": local, "max": mx, "sum": sm}))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_dist_helpers_on_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    port = free_port()
    mp.start_processes(_rank_main, args=(port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        d = json.loads((tmp_path / f"rank{r}.json").read_text())
        assert d == {"ws": 2, "rank": r, "local": r, "max": 2.5, "sum": 4.0}


def test_reference_arm_under_torchrun_prints_once_on_rank_0():
    """Two ranks of `bench.py --impl reference`: rank 1 exits 0 without work,
    rank 0 times the CPU implementation and prints the arm's JSON line."""
    pytest.importorskip("torch.distributed.run")
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--cpu-n", "12"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300,
                       env={**os.environ, "OMP_NUM_THREADS": "2"})
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["unit"] == "site-updates/s" and d["higher_is_better"] is True
    assert d["e2e"]["value"] == d["value"] and d["cpu_baseline"]["kind"] == "port"


def test_reference_arm_runs_the_same_config_as_ours():
    """The reference arm times the workload itself: its `config` is the one
    the GPU arm prints for the same lattice."""
    sys.path.insert(0, str(ROOT))
    import bench
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "2", "--warmup", "1",
                        "--cpu-n", "10"], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][0])
    assert d["config"] == bench.bench_config(10, "f64", 1)
    assert d["steps"] == 2 and d["warmup"] == 1 and "10^3 workload itself" in d["cpu_baseline"]["sample"]
