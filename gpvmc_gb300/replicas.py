"""Replica partitioning of walkers across ranks (one GPU per rank).

Walkers are independent Markov chains (the reference runs one chain per MPI
rank and never exchanges Monte-Carlo state, vmc.cpp:119-127), so a multi-GPU
run is N replicas: rank r owns walker ids [r*W, (r+1)*W) of the Philox
streams, nothing is exchanged on the data path, and quantity sums are added
once at the end (the reference's offline averaging of per-rank datasets).
"""
import numpy as np


def walker_base(rank, walkers_per_rank):
    """First Philox walker id owned by `rank`."""
    if rank < 0 or walkers_per_rank < 1:
        raise ValueError("rank >= 0 and walkers_per_rank >= 1 required")
    return rank * walkers_per_rank


def allreduce_sum(values, device=None):
    """Sum a float64 array over all ranks of the default torch.distributed
    group (gloo on CPU tensors, NCCL on CUDA tensors); returns numpy."""
    import torch
    import torch.distributed as dist
    t = torch.as_tensor(np.ascontiguousarray(values, dtype=np.float64))
    if device is not None:
        t = t.to(device)
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.cpu().numpy()
