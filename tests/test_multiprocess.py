"""The N > 1 path of bench.py on CPU: two gloo ranks on 127.0.0.1.

The path shards as replicas (each rank renders its own frame; there is no
data-path collective), so what N > 1 adds is host-side: the rendezvous, the
max of the per-rank times, the sum of the per-rank ray counts, and the
reference arm running on rank 0 alone while the other ranks exit without
work.  Processes start with `spawn`.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import bench
    w, r, local, dist = bench._dist()
    assert (w, r, local) == (world, rank, rank) and dist is not None
    # per-rank frame time and rays: the job time is the slowest rank's, the
    # throughput counts every rank's rays
    ms = 2.0 + rank
    rays = 1000 * (rank + 1)
    t = bench._allmax(dist, ms)
    total = bench._allsum(dist, float(rays))
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{t} {total}\n")
    dist.barrier()
    dist.destroy_process_group()


def _reference_rank(rank, world, port, out_dir):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import bench
    w, r, local, dist = bench._dist()
    if r != 0:
        # ranks other than 0 leave the reference arm at once
        bench.run_reference(None, w, r, local, dist)
        with open(os.path.join(out_dir, f"ref{rank}.txt"), "w") as f:
            f.write("exited\n")
        return
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"ref{rank}.txt"), "w") as f:
        f.write("rank0\n")


def test_two_gloo_ranks_reduce_times_and_rays(tmp_path):
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    lines = [(tmp_path / f"rank{r}.txt").read_text().split() for r in range(2)]
    for t, total in lines:
        assert float(t) == 3.0        # max over ranks
        assert float(total) == 3000.0  # sum over ranks


def test_reference_arm_runs_on_rank0_only(tmp_path):
    port = _free_port()
    mp.start_processes(_reference_rank, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    assert (tmp_path / "ref1.txt").read_text().strip() == "exited"
    assert (tmp_path / "ref0.txt").read_text().strip() == "rank0"
