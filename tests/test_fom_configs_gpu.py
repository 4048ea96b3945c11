"""FOM parity at the benchmark configurations (FP64, 1e-12 relative to the oracle).

Each test runs the GPU leapfrog through the C ABI on a configuration's own grid,
material, seeded sources and receivers, and the oracle (the CPU restatement of the
reference's CRS leapfrog) on the same inputs:
  * config 1: rank 1, 101 theta x 201 r (and the reference fixture's 201 x 101
    orientation), gaussDer at 640 km on the axis, period 60 s, delay 180 s, the full
    2000 steps, 181 surface receivers;
  * config 2: rank 2, 1000 theta x 2000 r, all M = 256 seeded forcings of the
    benchmark (depth U[200,700] km, period U[30,90] s, delay 180 s);
  * config 5's FOM: rank 2, 2000 theta x 4000 r, M = 64 seeded forcings.
The rank-2 grids are checked twice: from rest (the benchmark's own run: forcing
injection near the sources) and from a random state, which exercises every stencil
coefficient of the grid with O(1) values.  Tolerance: max |gpu - oracle| / max |oracle|
over each compared array <= 1e-12.
"""
import os
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12
MATERIAL = [3300.0, 2300.0 / 2891000.0, 0.0, 4400.0, 2900.0 / 2891000.0, 0.0]
SEED = 20261203  # the benchmark's seed for config 2's draws


def relerr(a, b):
    scale = np.max(np.abs(b))
    return np.max(np.abs(a - b)) / (scale if scale > 0 else 1.0)


def grids(shaw, oracle, nth, nr):
    m = shaw.Mesh.generate(nth, nr)
    m.set_material("unilayer", MATERIAL)
    with tempfile.TemporaryDirectory() as d:
        oracle.write_full_mesh(nth, nr, d)
        om = oracle.OracleMesh(d)
    om.set_material("unilayer", [(MATERIAL[0:3], MATERIAL[3:6])])
    dt = 0.25 * min(m.info[5], m.info[4] * m.info[2]) / (np.sqrt(2.0) * 7300.0)
    return m, om, dt


@pytest.mark.parametrize("nth,nr", [(101, 201), (201, 101)])
def test_config1_full_run(shaw, oracle, nth, nr):
    m, om, dt = grids(shaw, oracle, nth, nr)
    n = 2000
    src = m.map_source(640.0, 0.0)
    assert src == om.map_source(640.0, 0.0)
    rcv = [m.map_receiver(float(a)) for a in range(181)]
    f = shaw.Fom(m, 1, 1)
    f.set_sources([src], "gaussDer", 60.0, 180.0)
    f.set_receivers(rcv, 1, n)
    f.run(dt, n)
    ref = om.fom_run(1, n, dt, [src], [2], [60.0], [180.0], rcv, 1, 0, 0)
    vp, sp = f.get_state()
    seis = f.seismogram()
    f.close()
    assert np.max(np.abs(ref["seis"])) > 0  # the wave has reached the surface receivers
    assert relerr(seis, ref["seis"]) <= RTOL
    assert relerr(vp, ref["final_vp"]) <= RTOL and relerr(sp, ref["final_sp"]) <= RTOL


def rank2_case(shaw, oracle, nth, nr, gids_of, periods, n_rest, n_random, seed):
    m, om, dt = grids(shaw, oracle, nth, nr)
    M = len(periods)
    gids = gids_of(m)
    assert gids == gids_of(om)
    # receivers: every degree at the surface, and every source point (seen from step 1)
    rcv = [m.map_receiver(float(a)) for a in range(181)] + list(gids)
    f = shaw.Fom(m, 2, M)
    f.set_sources(gids, "gaussDer", periods, 180.0)
    # from rest, with the benchmark's sources
    f.set_receivers(rcv, 1, n_rest)
    f.run(dt, n_rest)
    vp, sp = f.get_state()
    seis = f.seismogram()
    ref = om.fom_run(2, n_rest, dt, gids, [2] * M, periods, [180.0] * M, rcv, 1, 0, 0)
    assert np.max(np.abs(ref["seis"])) > 0
    assert relerr(seis, ref["seis"]) <= RTOL
    assert relerr(vp, ref["final_vp"]) <= RTOL and relerr(sp, ref["final_sp"]) <= RTOL
    del vp, sp, ref
    # from a random state: every coefficient of the grid at O(1) values
    rng = np.random.default_rng(seed)
    xv = rng.standard_normal((m.nvp, M))
    xs = rng.standard_normal((m.nsp, M)) * 1e4
    f.set_receivers([], 0, 0)
    f.reset()
    f.set_state(np.asfortranarray(xv), np.asfortranarray(xs))
    f.advance(dt, n_random)
    f.synchronize()
    vp, sp = f.get_state()
    f.close()
    om.fom_advance_forced(xv, xs, 0, n_random, dt, gids, [2] * M, periods, 180.0)
    assert relerr(vp, xv) <= RTOL and relerr(sp, xs) <= RTOL


def test_config2_all_256_forcings(shaw, oracle):
    rng = np.random.default_rng(SEED)
    depths, periods = rng.uniform(200.0, 700.0, 256), rng.uniform(30.0, 90.0, 256)
    rank2_case(shaw, oracle, 1000, 2000, lambda mm: [mm.map_source(float(d), 0.0) for d in depths], periods,
               n_rest=50, n_random=20, seed=21)


def test_config5_fom_64_forcings(shaw, oracle):
    rng = np.random.default_rng(SEED + 5)
    depths = rng.uniform(200.0, 700.0, 64)
    periods = rng.uniform(30.0, 90.0, 64)
    rank2_case(shaw, oracle, 2000, 4000, lambda mm: [mm.map_source(float(d), 0.0) for d in depths], periods,
               n_rest=20, n_random=20, seed=55)
