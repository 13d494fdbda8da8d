"""The multi-process host path of bench.py on CPU, world size 2 over gloo on 127.0.0.1:
whole-job timing takes the slowest rank (max over ranks) behind a barrier, and the
reference arm under torchrun prints one line from rank 0 while the other rank exits 0.
Each rank answers its own replica's queries, so no data-path collective exists to test."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      IG_BENCH_BACKEND="gloo")
    sys.path.insert(0, ROOT)
    import bench

    r, world = bench.dist_setup(2)
    bench.barrier(world)
    slowest = bench.max_over_ranks(10.0 * (r + 1), world)
    with open(os.path.join(out_dir, f"rank{r}.txt"), "w") as f:
        f.write(f"{world} {slowest}")


def test_max_over_ranks_gloo(tmp_path):
    torch_mp = pytest.importorskip("torch.multiprocessing")
    torch_mp.start_processes(_rank_main, args=(_free_port(), str(tmp_path)), nprocs=2, start_method="spawn")
    for r in range(2):
        world, slowest = (tmp_path / f"rank{r}.txt").read_text().split()
        assert int(world) == 2 and float(slowest) == 20.0


def test_reference_arm_under_torchrun():
    pytest.importorskip("torch.distributed.run")
    env = dict(os.environ, IG_BENCH_BACKEND="gloo", OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference", "--gpus", "2",
           "--steps", "1", "--warmup", "3"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["value"] > 0 and line["n_gpus"] == 2
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
    # The arm reports the GPU arm's metric, unit and configuration: the same workload.
    sys.path.insert(0, ROOT)
    import bench

    assert line["metric"] == bench.METRIC and line["unit"] == "queries/s" and line["config"] == bench.CONFIG
    assert line["higher_is_better"] is True and line["steps"] == 1 and line["warmup"] == 3
    for key in ("ms_per_step", "scaling", "vs_baseline", "dtype", "data", "step", "execution"):
        assert key in line, key
    assert line["e2e"]["value"] == line["value"] and line["cpu_baseline"]["value"] == line["value"]
