"""The multi-process path of bench.py on the CPU: two ranks over gloo at 127.0.0.1.

The propagation path has no exchange step, so N ranks are N replicas. What must hold across
ranks is host logic: the step time reported is the slowest rank's, every rank propagates
its own parameter sets (weak scaling), and only rank 0 prints a result line."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    slowest = bench.max_over_ranks(1.5 + rank, world, "cpu")
    w = bench.workload("batch_atmos", rank)
    wb = bench.workload("batch_beam", rank)
    m = bench.rank_parameter_set(rank, world)
    mine = (w["sets"][0].theta23, w["sets"][0].dm23sq, tuple(w["grids"][0]),
            wb["sets"][0].dcp, m.theta23, m.dcp)
    every = [None] * world
    dist.all_gather_object(every, mine)
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"slowest": slowest, "every": every}, f)


def test_two_ranks_reduce_the_slowest_time_and_shard_the_parameter_sets(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       start_method="spawn", join=True)
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    for r in res:
        assert r["slowest"] == 2.5  # max over ranks of 1.5 + rank
    every = res[0]["every"]
    assert res[1]["every"] == every
    # every rank propagates different parameter sets (batched and single-grid workloads)
    assert every[0][0] != every[1][0] or every[0][1] != every[1][1]
    assert every[0][3] != every[1][3]
    assert (every[0][4], every[0][5]) != (every[1][4], every[1][5])


def test_rank_zero_keeps_the_configurations_own_sets():
    sys.path.insert(0, ROOT)
    import bench
    from cudaprob3_gb300 import earth
    w0 = bench.workload("batch_atmos", 0)
    ref = earth.gaussian_sets(256, seed=2024)
    assert w0["sets"][0] == ref[0] and w0["sets"][-1] == ref[-1]
    assert bench.rank_parameter_set(0, 4) == earth.NOMINAL


@pytest.mark.parametrize("rank", [0, 1])
def test_reference_arm_prints_on_rank_zero_only(rank):
    env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank),
               MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2",
                        "--workload", "prem4", "--steps", "1", "--warmup", "1",
                        "--cpu-seconds", "0.05"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    if rank == 0:
        assert len(lines) == 1
        d = json.loads(lines[0])
        assert d["impl"] == "reference" and d["value"] > 0 and d["n_gpus"] == 2
        assert d["e2e"]["h2d_bytes_per_step"] == 0
    else:
        assert lines == []
