"""The multi-rank plumbing of bench.py on CPU: two gloo ranks.

A single instance does not shard (its 3-D FFTs would need all-to-all
transposes), so N GPUs run N independent replicas of the batch: the only
cross-rank operations are the barrier around the timed region and the max of
the per-rank times.  Both, and the rule that only rank 0 runs the reference arm
and prints, are exercised here with world_size 2 over gloo on 127.0.0.1.
"""
import argparse
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    r, w, local = bench.dist_env()
    d = bench.dist_init(w)
    bench.barrier(d)
    # per-rank "timed region" lengths: the job time is the slowest rank's
    m = bench.max_over_ranks(d, 10.0 + 5.0 * r)
    bench.barrier(d)
    ref = None
    if r != 0:
        # the reference arm runs on rank 0 only; other ranks return at once
        ref = bench.run_reference(argparse.Namespace(steps=1, warmup=1, gpus=w))
    q.put((r, w, local, m, ref))
    d.destroy_process_group()


def test_two_gloo_ranks_barrier_max_and_rank0_only():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(i, 2, port, q)) for i in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 and o[2] == o[0] for o in out)
    assert all(o[3] == 15.0 for o in out)
    assert out[1][4] == 0


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.dist_init(1) is None
    bench.barrier(None)
    assert bench.max_over_ranks(None, 3.5) == 3.5
