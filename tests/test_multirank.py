"""The N > 1 path of bench.py on CPU: world-size-2 gloo ranks (127.0.0.1).

Each rank of the batched workload advances its own seeded set of grids (no
data shared, no collective on the data path) and the reported time is the
slowest rank's."""
import os
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "an5d-artifact_gb300"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    specs = bench.rank_specs(16, rank, world, tmax=64)
    ms = bench.max_over_ranks(10.0 + rank, world)
    gathered = [None] * world
    dist.all_gather_object(gathered, specs)
    out[rank] = (ms, gathered)
    dist.destroy_process_group()


def test_two_ranks_shard_and_take_the_slowest():
    port = 29500 + os.getpid() % 1000
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    ms0, g0 = res[0]
    ms1, g1 = res[1]
    assert ms0 == ms1 == 11.0                   # max over ranks, seen by both
    assert g0[0] != g0[1] and g0 == g1          # each rank its own grids
    assert len(g0[0]) == len(g0[1]) == 16       # same count per rank (weak scaling)


def test_single_rank_is_the_standard_set():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.rank_specs(8, 0, 1) == bench.batched_specs(8)
    assert bench.max_over_ranks(3.5, 1) == 3.5


def _bench(args, env_extra=None, drop=("WORLD_SIZE", "RANK", "LOCAL_RANK")):
    import subprocess
    env = {k: v for k, v in os.environ.items() if k not in drop}
    env.update(env_extra or {})
    return subprocess.run([sys.executable, str(ROOT / "bench.py")] + args, capture_output=True, text=True,
                          timeout=600, env=env)


SMALL = ["--impl", "reference", "--workload", "star2d1r", "--n", "128", "--T", "4", "--steps", "1",
         "--warmup", "0", "--cpu-budget", "0.2"]


def test_gpus_flag_launches_one_process_per_rank():
    """bench.py --gpus 2 outside torchrun re-runs itself as two ranks under
    torch.distributed.run (127.0.0.1); rank 0 alone prints the line."""
    import json
    r = _bench(["--gpus", "2"] + SMALL)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["n_gpus"] == 2 and line["impl"] == "reference"


def test_gpus_flag_never_silently_runs_fewer_ranks():
    r = _bench(["--gpus", "2"] + SMALL, env_extra={"WORLD_SIZE": "1", "RANK": "0"})
    assert r.returncode != 0 and "WORLD_SIZE" in r.stderr
