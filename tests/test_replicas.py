"""The N > 1 path of bench.py on CPU: two ranks under the gloo backend.

The solve does not shard (each rank runs an independent replica), so the
only cross-rank logic is the harness: the whole job's step time is the
maximum over ranks, the barriers around the timed region, and the reference
arm running on rank 0 alone.  These run here with world size 2 on gloo; the
GPU runs use the same functions with NCCL."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as td

    import bench

    td.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                          world_size=world)
    try:
        bench.dist_barrier()
        v = bench.dist_max(1.5 + rank)
        # the reference arm returns on every rank but 0 without doing work
        ref = bench.run_reference(None, rank, world) if rank != 0 else "rank0"
        bench.dist_barrier()
        out.put((rank, v, ref))
    finally:
        td.destroy_process_group()


def test_two_gloo_ranks_max_and_rank0_only():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.5, 2.5]
    assert res[0][2] == "rank0" and res[1][2] is None


def test_single_process_without_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.dist_max(3.25) == 3.25
    bench.dist_barrier()


if __name__ == "__main__":
    sys.exit(pytest.main([__file__, "-q"]))
