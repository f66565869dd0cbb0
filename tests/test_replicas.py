"""The multi-process host logic (gpuisac/replicas.py) on CPU with two gloo
ranks: the reference's particle partition (MPI_start_end), the slowest
rank's time, and the gather of the ranks' result columns at the root
(wrap_mpi_concat_numpy) -- the pieces a one-process-per-GPU run uses."""
import os
import socket
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "gpu-isac_gb300"))

from gpuisac.replicas import start_end  # noqa: E402


def test_partition_covers_every_particle_once():
    for nima in (1, 7, 50000, 99999):
        for nproc in (1, 2, 3, 8):
            edges = [start_end(nima, nproc, r) for r in range(nproc)]
            assert edges[0][0] == 0 and edges[-1][1] == nima
            assert all(edges[r][1] == edges[r + 1][0] for r in range(nproc - 1))
    # the reference's rounding: 10 particles on 4 ranks -> 0-2, 2-5, 5-8, 8-10 (round half to even)
    assert [start_end(10, 4, r) for r in range(4)] == [(0, 2), (2, 5), (5, 8), (8, 10)]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    from gpuisac import replicas
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert replicas.rank_env() == (world, rank, rank)
        # slowest rank's time
        m = replicas.max_over_ranks(10.0 + rank * 3.5)
        # each rank aligns its partition: columns of d [R][n] and peak_list [R][4n]
        nima, R = 23, 5
        full_d = np.arange(R * nima, dtype=np.float32).reshape(R, nima)
        full_pk = np.arange(R * 4 * nima, dtype=np.float32).reshape(R, 4 * nima) * 0.5
        a, b = replicas.start_end(nima, world, rank)
        d = replicas.gather_columns(full_d[:, a:b], nima)
        pk = replicas.gather_columns(full_pk[:, 4 * a:4 * b], nima, cols_per_particle=4)
        ok = m == 10.0 + (world - 1) * 3.5
        if rank == 0:
            ok = ok and np.array_equal(d, full_d) and np.array_equal(pk, full_pk)
        else:
            ok = ok and d is None and pk is None
        with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
            f.write("ok" if ok else "bad")
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    assert [open(tmp_path / f"rank{r}.txt").read() for r in range(world)] == ["ok", "ok"]
    del torch
