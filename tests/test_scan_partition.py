"""The effective-potential scan's instance partition across ranks, on CPU.

The scan's instances (the pure droplet and one per impurity position) are
independent, so N GPUs split the list (rank r takes r, r + N, ...) and rank
0 gathers the per-instance energies (host scalars over gloo/NCCL, no
collective on the data path).  Checked with two gloo ranks on 127.0.0.1:
the ranks' shares are disjoint and cover the list, and the gathered V_eff(z)
equals a one-rank run.  The engine here is the CPU FP64 oracle behind the
Batch interface on a tiny grid (the GPU engine is exercised by the GPU
tests); the scan's host logic is the product code.
"""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ZS = [0.0, 1.25, 2.5, 3.75, 5.0]
KW = dict(steps32=3, steps64=2, dt=5e-4, n=16, h=1.0, n4=60.0, seed=1, reference=True, tune=False, refine="fp64")


class OracleBatch:
    """The oracle behind the Batch interface (FP64 only: set_precision is a no-op)."""

    def __init__(self, cfgs):
        from oracle import pyoracle
        self.solvers = [pyoracle.OracleSolver(c) for c in cfgs]

    def __iter__(self):
        return iter(self.solvers)

    def __len__(self):
        return len(self.solvers)

    def steprk(self, dt):
        for s in self.solvers:
            s.steprk(dt)

    def run(self, n, dt, wait=True):
        return [s.run(n, dt) for s in self.solvers]

    def set_precision(self, p):
        pass

    def close(self):
        for s in self.solvers:
            s.close()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import torch.distributed as dist
    from oracle import pyoracle
    from eff_pot_gb300 import scan
    from test_scan_partition import OracleBatch
    pyoracle.set_threads(1)
    dist.init_process_group("gloo")
    res = scan.veff_scan(ZS, rank=rank, world=world, dist=dist, make_batch=OracleBatch, **KW)
    q.put((rank, res))
    dist.destroy_process_group()


def test_partition_covers_the_instance_list_once():
    from eff_pot_gb300 import scan
    inst = scan.instance_list([1.25 * k for k in range(32)])
    for world in (1, 2, 3, 4, 8):
        shares = [scan.partition(inst, r, world) for r in range(world)]
        flat = [x for s in shares for x in s]
        assert sorted(flat, key=str) == sorted(inst, key=str)
        assert len(flat) == len(inst)
        assert max(len(s) for s in shares) - min(len(s) for s in shares) <= 1


def test_two_gloo_ranks_gather_the_one_rank_scan(oracle):
    from eff_pot_gb300 import scan
    oracle.set_threads(1)
    one = scan.veff_scan(ZS, make_batch=OracleBatch, **KW)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(i, 2, port, q)) for i in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[1] is None
    two = out[0]
    assert two["ranks"] == 2 and two["instances"] == len(ZS) + 1
    assert two["E_pure"] == one["E_pure"]
    for a, b in zip(two["rows"], one["rows"]):
        assert a["z"] == b["z"]
        assert a["Veff"] == b["Veff"] and a["E"] == b["E"]
    # the oracle runs FP64 in both passes: the "FP32 + refine" pass equals
    # the FP64 reference pass, so every per-point error is exactly zero
    assert one["max_abs_Veff_err_K"] == 0.0
    # the impurity raises or lowers the energy: V_eff is not identically zero
    assert any(abs(r["Veff"]) > 1e-6 for r in one["rows"])
