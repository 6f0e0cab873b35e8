"""The replica set-up of bench.py on two CPU ranks (gloo, world size 2).

bench.py --gpus N runs one independent replica per GPU: no data crosses
between ranks, the ranks only meet at barriers around the timed region and
take the maximum of their times.  This checks that set-up without a GPU:
rendezvous on 127.0.0.1, the barrier, the max-reduce, and that the reference
arm does its work on rank 0 alone.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(ws),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    w, r, local, pg = bench.dist_setup()
    assert (w, r, local) == (ws, rank, rank) and pg is not None
    bench.barrier(pg)
    # rank k reports a time of 10 + k ms; every rank must see the slowest
    got = bench.allmax(pg, 10.0 + rank)
    bench.barrier(pg)

    class Args:  # run_reference returns before any work on ranks other than 0
        steps, warmup, gpus = 1, 0, ws
    if rank != 0:
        bench.run_reference(Args, 8, 4, 4, ws, rank)
    pg.destroy_process_group()
    out.put((rank, got))


def test_two_rank_barrier_and_max():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    codes = [p.exitcode for p in procs]
    for p in procs:
        if p.is_alive():
            p.kill()
    assert codes == [0, 0], codes
    res = dict(q.get(timeout=5) for _ in range(2))
    assert res == {0: 11.0, 1: 11.0}
