"""The bench's multi-rank path on CPU: one process per rank over gloo
(world size 2, 127.0.0.1), the barrier and the max/sum reductions that turn
per-rank times and work into the whole-job value (replicas: each rank runs
its own copy of the workload, no collective on the data path)."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench

    r, w, local = bench.dist_info()
    assert (r, w, local) == (rank, world, rank)
    dist = bench.init_dist(w)
    bench.barrier(dist)
    t_max = bench.reduce_max(dist, 1.0 + rank)      # per-rank device time
    work = bench.reduce_sum(dist, 100.0 * (rank + 1))  # per-rank tet-iterations
    bench.barrier(dist)
    Path(out_dir, f"rank{rank}.txt").write_text(f"{t_max} {work}")
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_time_and_work(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for rank in range(2):
        t_max, work = (float(x) for x in (tmp_path / f"rank{rank}.txt").read_text().split())
        assert t_max == 2.0 and work == 300.0
    # whole-job value = all ranks' work / the slowest rank's time
    assert 300.0 / 2.0 == 150.0


def test_single_rank_has_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.init_dist(1) is None
    assert bench.reduce_max(None, 3.5) == 3.5 and bench.reduce_sum(None, 2.0) == 2.0
    bench.barrier(None)
