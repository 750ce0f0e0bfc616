"""Multi-GPU path on CPU: replicas on two gloo ranks.

The batch shards by scene with no data-path collective: every rank renders its own
batch (disjoint seeds) and the only collective is the max over ranks of the step time.
These tests run that host logic as two processes on the gloo backend.
"""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank_main(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "pathfinder-cpp_gb300"))
    import bench
    import scenes as S
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seed = bench.replica_first_seed(rank)
        batch = S.batched(n_scenes=3, first_seed=seed, hi_paths=64)
        # a rank's own step time; the job's is the slowest rank's
        mine = 10.0 + 5.0 * rank
        job = bench.max_over_ranks(mine, dist, "cpu")
        sig = [int(s.points[:4].view("uint32").sum()) for s in batch]
        with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
            f.write(f"{seed} {job} {' '.join(map(str, sig))}\n")
        dist.barrier()
    finally:
        dist.destroy_process_group()


def _free_port():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_replicas_render_disjoint_batches_and_agree_on_the_step_time(tmp_path):
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    rows = []
    for r in range(world):
        seed, job, *sig = open(tmp_path / f"rank{r}.txt").read().split()
        rows.append((int(seed), float(job), tuple(sig)))
    (s0, j0, g0), (s1, j1, g1) = rows
    assert s0 != s1 and abs(s1 - s0) >= 3  # seed ranges do not overlap
    assert g0 != g1                        # different scenes on each rank
    assert j0 == j1 == 15.0                # both see the slowest rank's time


def test_one_process_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, None, "cpu") == 12.5
    assert bench.replica_first_seed(0) == 1000
