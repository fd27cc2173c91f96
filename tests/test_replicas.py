"""Several ranks (no GPU): signal sharding, max-over-ranks timing and the
rank-0 gather, run as two gloo processes on the CPU.  Each rank integrates its
shard of a small two-compartment workload with the oracle; the gathered
signals must equal the single-process ones bit for bit."""

import importlib
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = "dmri-fem-cloud_gb300"


def test_shard_covers_every_signal_once(pkg):
    rp = importlib.import_module(PKG + ".replicas")
    for n, w in [(0, 1), (1, 3), (7, 2), (512, 8), (2048, 6)]:
        got = np.concatenate([rp.shard(n, r, w) for r in range(w)])
        assert np.array_equal(np.sort(got), np.arange(n))
        sizes = [len(rp.shard(n, r, w)) for r in range(w)]
        assert max(sizes) - min(sizes) <= (1 if n else 0)
    mesh_of = np.array([2, 0, 1, 0, 2, 1, 0, 2])
    parts = [rp.shard(8, r, 3, mesh_of) for r in range(3)]
    flat = np.concatenate(parts)
    assert np.all(np.diff(mesh_of[flat]) >= 0)          # mesh-major
    with pytest.raises(ValueError):
        rp.shard(4, 2, 2)


def _problem():
    sys.path.insert(0, ROOT)
    import oracle
    pkg = importlib.import_module(PKG)
    xyz, tets = pkg.meshgen.kuhn_box(-2.0, 2.0, 3)
    reg = pkg.meshgen.cylinder_regions(xyz, tets, [(0.0, 0.0)], [1.2])
    sd = oracle.duplicated_system(xyz, tets, reg, np.array([2e-3, 3e-3]), 0.0, 1e-4)
    prof = oracle.PGSE(1000, 4000)
    dirs = pkg.meshgen.fibonacci_directions(5)
    sig = [(b, d) for b in (500.0, 1500.0) for d in dirs]
    return oracle, sd, prof, sig


def _solve(idx):
    oracle, sd, prof, sig = _problem()
    out = []
    for i in idx:
        b, d = sig[i]
        q = oracle.bvalue_to_q(b, prof.int4gb())
        r = oracle.solve_duplicated(sd, prof, q, d, 200.0)
        out.append([r.signal / r.S0, i])
    return np.array(out).reshape(len(idx), 2)


def _rank_main(rank, world_size, port, result_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    try:
        sys.path.insert(0, ROOT)
        rp = importlib.import_module(PKG + ".replicas")
        assert rp.world() == (rank, world_size)
        n = len(_problem()[3])
        mine = rp.shard(n, rank, world_size)
        vals = _solve(mine)
        t = rp.max_over_ranks(10.0 + rank)
        allv = rp.gather_signals(mine, vals, n)
        if rank == 0:
            np.save(result_path, allv)
            assert t == 10.0 + world_size - 1
        else:
            assert allv is None
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_match_single_process(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    path = str(tmp_path / "sig.npy")
    mp.start_processes(_rank_main, args=(2, port, path), nprocs=2, join=True, start_method="spawn")
    got = np.load(path)
    ref = _solve(np.arange(10))
    assert np.array_equal(got, ref)
