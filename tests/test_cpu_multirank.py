"""The multi-rank path on the CPU (gloo, world size 2): the bench's host barrier and
max-over-ranks timing, and the column split the reference distributes over MPI ranks
(benchmark_hpc/benchmark_mpi.c:26-45, src/matchgate_target.c:1336-1338): each rank traces
its own range of basis columns and one sum gives the full f and gradient.  Ranks are
processes on 127.0.0.1; the per-rank traces use the oracle (no GPU here)."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, L, out_path):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank), "WORLD_SIZE": str(world)})
    for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch
    import bench
    import oracle as O
    from conftest import random_gates, brickwall_perms
    dist = bench.Dist(world)
    # max over ranks of the per-rank "time"
    assert dist.max(1.0 + rank) == float(world)
    dist.barrier()
    rng = np.random.default_rng(42)
    ul = random_gates(6, rng, unitary=True)
    uperms = brickwall_perms(L, 6, rng)
    v = random_gates(3, rng, unitary=True)
    perms = brickwall_perms(L, 3, rng)
    t = O.Target("brickwall", L, ulist=ul, uperms=uperms)
    n = 1 << L
    b0, b1 = rank * n // world, (rank + 1) * n // world
    f, dv = O.brickwall_target_and_gradient(t, v, perms, L, col_range=(b0, b1))
    buf = torch.tensor(np.concatenate([[f.real, f.imag], dv.view(np.float64).reshape(-1)]), dtype=torch.float64)
    dist.td.all_reduce(buf)
    if rank == 0:
        f_all, dv_all = O.brickwall_target_and_gradient(t, v, perms, L)
        full = np.concatenate([[f_all.real, f_all.imag], dv_all.view(np.float64).reshape(-1)])
        np.save(out_path, np.stack([buf.numpy(), full]))
    dist.barrier()
    dist.td.destroy_process_group()


def test_two_ranks_column_split(oracle, tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    out = str(tmp_path / "r.npy")
    mp.start_processes(_rank_main, args=(2, _free_port(), 8, out), nprocs=2, join=True, start_method="spawn")
    got, full = np.load(out)
    assert np.max(np.abs(got - full)) < 1e-12 * max(1.0, np.max(np.abs(full)))
