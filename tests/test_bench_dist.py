"""bench.py's multi-rank plumbing on CPU: two gloo ranks on 127.0.0.1, the
max-over-ranks timing reduction and the barrier the timed region is bracketed by.
On a GPU machine the same functions run over NCCL, one rank per GPU, each rank an
independent replica of the product (no data-path collective)."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    r, w, local, dist = bench.dist_init()
    assert (r, w, local) == (rank, ws, rank) and dist is not None
    bench.barrier(dist)
    t = bench.reduce_max(dist, 1.5 + rank, local)
    # the reference arm runs on rank 0 only; other ranks return without work
    skipped = bench.run_reference(None, r, w, dist) is None if r != 0 else True
    bench.barrier(dist)
    dist.destroy_process_group()
    q.put((rank, t, skipped))


def test_two_gloo_ranks_reduce_max_and_barrier():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("with a GPU visible bench picks NCCL, one rank per GPU; this test is the CPU (gloo) form")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
    assert all(p.exitcode == 0 for p in ps)
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert got == [(0, 2.5, True), (1, 2.5, True)]


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK") if k in os.environ}
    try:
        assert bench.dist_init() == (0, 1, 0, None)
        assert bench.reduce_max(None, 3.0, 0) == 3.0
        bench.barrier(None)
    finally:
        os.environ.update(env)
