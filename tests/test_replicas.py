"""Replica (multi-rank) host logic on CPU: two gloo ranks each run their own
walker-id range and sum their quantity sums once; the result equals one
process running all walkers.  The chains run in the oracle (no GPU here)."""
import math
import os
import socket

import numpy as np
import pytest

PHI, NEEL, L, W, SEED = 0.25 * math.pi, 0.1, 4, 3, 77


def _sums(oracle_mod, first, count):
    tot = np.zeros(4)
    for w in range(first, first + count):
        o = oracle_mod.OracleChain(L, PHI, NEEL, seed=SEED, walker=w)
        o.random_start()
        o.walk(100)
        o.walk(16 * 5, meas=16, mask=oracle_mod.MEAS_PROJHEIS | oracle_mod.MEAS_STAGMAGN)
        pj, n = o.projheis()
        sm, _ = o.stagmagn()
        tot += [pj[0, 0].real, n, sm.real, 1.0]
    return tot


def _rank(rank, world, port, out):
    import torch.distributed as dist
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    sys.path.insert(0, os.path.dirname(here))
    import oracle_lib
    from gpvmc_gb300.replicas import allreduce_sum, walker_base
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    s = allreduce_sum(_sums(oracle_lib, walker_base(rank, W), W))
    if rank == 0:
        np.save(out, s)
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_replicas_equal_single_process(oracle, tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as tmp
    out = str(tmp_path / "sum.npy")
    tmp.spawn(_rank, args=(2, _free_port(), out), nprocs=2, join=True)
    got = np.load(out)
    want = _sums(oracle, 0, 2 * W)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12)
    assert got[1] == 2 * W * 5


def test_walker_base():
    from gpvmc_gb300.replicas import walker_base
    assert [walker_base(r, 2048) for r in range(4)] == [0, 2048, 4096, 6144]
    with pytest.raises(ValueError):
        walker_base(-1, 8)
