"""bench.py's replica plumbing across two gloo ranks on the CPU (the N > 1 launch without GPUs): the barrier,
the max-over-ranks timing that the whole-job value is divided by, and the reference arm doing its work on rank
0 only."""
import json
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, outdir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench
    ws, r, local = bench.dist_init()
    assert (ws, r, local) == (2, rank, rank) and dist.get_backend() == "gloo"
    bench.barrier(ws)
    slowest = bench.max_over_ranks(ws, 10.0 + 5.0 * rank)  # rank 1 is the slow one
    ref = bench.run_reference(bench.parse(["--impl", "reference", "--n", "8"]), ws, rank) \
        if rank == 1 else None
    with open(os.path.join(outdir, f"rank{rank}.json"), "w") as f:
        json.dump({"slowest": slowest, "ref_is_none": ref is None}, f)
    bench.barrier(ws)
    dist.destroy_process_group()


def test_two_rank_barrier_and_max(tmp_path):
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(_free_port(), str(tmp_path)), nprocs=2, join=True)
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    assert res[0]["slowest"] == res[1]["slowest"] == 15.0
    assert res[1]["ref_is_none"]  # non-zero ranks of the reference arm exit without work
