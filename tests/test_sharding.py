"""Forcing-column sharding (one process per GPU) with world_size 2 on CPU (gloo).

Each rank runs the FOM rank-2 leapfrog of its own column range -- here through the CPU
oracle, which stands in for one GPU's work -- and rank 0 gathers the seismograms; the
result must equal the unsharded run bit for bit, since columns never interact.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from conftest import mesh_dir
from shaw_gb300.sharding import shard_range


def test_shard_range_covers_columns_once():
    for total in (0, 1, 5, 256, 1001):
        for world in (1, 2, 3, 8):
            got = [shard_range(total, r, world) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == total
            assert all(got[i][1] == got[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(4, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _job(M):
    rng = np.random.default_rng(11)
    depths = rng.uniform(300.0, 1500.0, M)
    angles = rng.uniform(10.0, 170.0, M)
    periods = rng.uniform(40.0, 70.0, M)
    return depths, angles, periods


def _run_columns(om, lo, hi, depths, angles, periods, rcv, n):
    gids = [om.map_source(float(depths[j]), float(angles[j])) for j in range(lo, hi)]
    m = hi - lo
    if m == 0:
        return np.zeros((len(rcv), n, 0))
    out = om.fom_run(2, n, 1.0, gids, [2] * m, list(periods[lo:hi]), [20.0] * m, rcv, 1, 0, 0, nthreads=1,
                     want_final=False)
    return out["seis"]


def _worker(rank, world, port, M, n, result_path):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import sys

    here = os.path.dirname(os.path.abspath(__file__))
    for p in (here, os.path.dirname(here)):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch.distributed as dist

    import oracle_lib
    from shaw_gb300.sharding import gather_columns

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        om = oracle_lib.OracleMesh(mesh_dir("fullMesh21x51"))
        om.set_material("unilayer", [([2000.0, 0.0, 0.0], [5000.0, 0.0, 0.0])])
        rcv = [om.map_receiver(a) for a in (15.0, 90.0, 165.0)]
        depths, angles, periods = _job(M)
        lo, hi = shard_range(M, rank, world)
        local = _run_columns(om, lo, hi, depths, angles, periods, rcv, n)
        full = gather_columns(local, M, dist)
        if rank == 0:
            np.save(result_path, full)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("M", [5, 1])
def test_two_rank_column_sharding_matches_unsharded(oracle, tmp_path, M):
    n, world = 60, 2
    result = str(tmp_path / "gathered.npy")
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, M, n, result)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
    for p in procs:
        if p.is_alive():
            p.kill()
            p.join()
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    gathered = np.load(result)
    om = oracle.OracleMesh(mesh_dir("fullMesh21x51"))
    om.set_material("unilayer", [([2000.0, 0.0, 0.0], [5000.0, 0.0, 0.0])])
    rcv = [om.map_receiver(a) for a in (15.0, 90.0, 165.0)]
    depths, angles, periods = _job(M)
    whole = _run_columns(om, 0, M, depths, angles, periods, rcv, n)
    assert gathered.shape == whole.shape == (3, n, M)
    assert np.max(np.abs(whole)) > 0
    assert np.array_equal(gathered, whole)
