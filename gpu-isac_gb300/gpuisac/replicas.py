"""Host logic of the multi-process (one process per GPU) use of the library.

Particles are independent, so N GPUs run N processes with no collective on
the data path.  The reference splits the particle stack across its GPU ranks
with MPI_start_end (bin/sp_isac_applications.py:4128-4131) and gathers the
ranks' result columns at the root before the group assignment
(wrap_mpi_concat_numpy, bin/sp_isac2_gpu.py:464-500, called at :1029);
`start_end` and `gather_columns` do the same over torch.distributed (NCCL on
GPUs, gloo on CPU).  `max_over_ranks` gives the slowest rank's time for a
whole-job rate.
"""
from __future__ import annotations

import os

import numpy as np


def rank_env() -> tuple[int, int, int]:
    """(world size, rank, local rank) from the launcher's environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def start_end(nima: int, nproc: int, myid: int) -> tuple[int, int]:
    """Particles [start, end) of rank myid out of nproc (the reference's
    MPI_start_end: both ends rounded from nima / nproc * rank)."""
    return int(round(float(nima) / nproc * myid)), int(round(float(nima) / nproc * (myid + 1)))


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def max_over_ranks(x: float, device=None) -> float:
    """The largest x of all ranks (x itself without a process group)."""
    dist = _dist()
    if dist is None or dist.get_world_size() == 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_columns(local: np.ndarray, nima: int, cols_per_particle: int = 1, root: int = 0):
    """Concatenate the ranks' column blocks of a [rows][cols_per_particle * n_local]
    array (peak_list: 4 columns per particle, d: 1) in rank order at `root`;
    rank r holds particles start_end(nima, world, r).  Returns the
    [rows][cols_per_particle * nima] array on root, None elsewhere."""
    dist = _dist()
    local = np.ascontiguousarray(local)
    if dist is None or dist.get_world_size() == 1:
        return local
    world, rank = dist.get_world_size(), dist.get_rank()
    a, b = start_end(nima, world, rank)
    if local.shape[1] != cols_per_particle * (b - a):
        raise ValueError(f"rank {rank} holds {local.shape[1]} columns, expected {cols_per_particle * (b - a)}")
    parts = [None] * world if rank == root else None
    dist.gather_object(local, parts, dst=root)
    if rank != root:
        return None
    return np.concatenate(parts, axis=1)
