"""FOM in FP32 (SHAW_MIXED_FP32): FP32 state and stencil values, FP32 FMAs.

Not a parity path: it is held to a stated tolerance against the FP64 path on the
same inputs (relative seismogram error, max |fp32 - fp64| / max |fp64|), and to exact
self-consistency (layouts, graph replay, pieces, observers).
"""
import numpy as np
import pytest

from test_fom_gpu import CFG_MATERIAL, meshes, relerr

pytestmark = pytest.mark.gpu

# measured 8e-7 on the 101 x 201 grid over 2000 steps (FP32 rounding of the state and
# of the stencil values); the bound leaves room for the rank-2 runs below
TOL_FP32 = 3e-6


def test_fp32_fom_config1_within_tolerance(shaw):
    m = shaw.Mesh.generate(101, 201)
    m.set_material("unilayer", CFG_MATERIAL)
    dt = 0.25 * min(m.info[5], m.info[4] * m.info[2]) / (np.sqrt(2.0) * 7300.0)
    n = 2000
    rcv = [m.map_receiver(float(a)) for a in range(181)]
    out = {}
    for p in (shaw.FP64, shaw.MIXED_FP32):
        f = shaw.Fom(m, 1, 1, precision=p)
        f.set_sources([m.map_source(640.0, 0.0)], "gaussDer", 60.0, 180.0)
        f.set_receivers(rcv, 1, n)
        f.run(dt, n)
        out[p] = (f.seismogram(), f.get_state())
        f.close()
    assert np.max(np.abs(out[shaw.FP64][0])) > 0
    assert relerr(out[shaw.MIXED_FP32][0], out[shaw.FP64][0]) <= TOL_FP32
    # the full final state (wavefronts included) carries a little more: 4.6e-6 measured
    assert relerr(out[shaw.MIXED_FP32][1][0], out[shaw.FP64][1][0]) <= 1e-5


@pytest.mark.parametrize("M", [3, 6, 8])  # 1, 2 and 4 columns per thread
def test_fp32_rank2_layouts(shaw, oracle, M):
    m, _ = meshes(shaw, oracle, "fullMesh21x51")
    rng = np.random.default_rng(M)
    gids = [m.map_source(float(d), float(a)) for d, a in zip(rng.uniform(300, 1500, M), rng.uniform(5, 175, M))]
    periods = rng.uniform(30, 60, M)
    rcv = [m.map_receiver(a) for a in (10, 60, 120, 170)]
    n = 400
    out = {}
    for p in (shaw.FP64, shaw.MIXED_FP32):
        f = shaw.Fom(m, 2, M, precision=p)
        f.set_sources(gids, "ricker", periods, 10.0)
        f.set_receivers(rcv, 1, n)
        f.run(1.0, n)
        out[p] = f.seismogram()
        f.close()
    assert relerr(out[shaw.MIXED_FP32], out[shaw.FP64]) <= TOL_FP32
    # each column's arithmetic does not depend on how many columns share a thread
    f1 = shaw.Fom(m, 2, 1, precision=shaw.MIXED_FP32)
    f1.set_sources(gids[:1], "ricker", periods[:1], 10.0)
    f1.set_receivers(rcv, 1, n)
    f1.run(1.0, n)
    assert np.array_equal(f1.seismogram()[:, :, 0], out[shaw.MIXED_FP32][:, :, 0])


def test_fp32_observers_graph_and_pieces(shaw, oracle):
    m, _ = meshes(shaw, oracle, "fullMesh21x51")
    gids = [m.map_source(d, 45.0) for d in (300.0, 600.0, 900.0, 1200.0)]
    rcv = [m.map_receiver(a) for a in (10, 45, 90, 170)]
    n = 200
    seis = []
    for snaps in (False, True):  # snapshots force per-step launches; without them graphs replay
        f = shaw.Fom(m, 2, 4, precision=shaw.MIXED_FP32)
        f.set_sources(gids, "ricker", 40.0, 10.0)
        f.set_receivers(rcv, 2, n)
        if snaps:
            f.set_snapshots(2, 50, n)
        f.run(1.0, n)
        seis.append(f.seismogram())
        if snaps:
            svp, _ = f.snapshots()
            # the vp snapshots hold exactly the seismogram's samples at the receivers
            assert np.array_equal(svp[rcv, :, :], seis[-1])
        f.close()
    assert np.array_equal(seis[0], seis[1])
    f = shaw.Fom(m, 2, 4, precision=shaw.MIXED_FP32)
    f.set_sources(gids, "ricker", 40.0, 10.0)
    f.set_receivers(rcv, 2, n)
    f.reset()
    for k in (1, 63, 64, 72):
        f.advance(1.0, k)
    f.synchronize()
    assert np.array_equal(f.seismogram(), seis[0])


def test_fp32_state_roundtrip(shaw, oracle):
    m, _ = meshes(shaw, oracle, "fullMesh21x51")
    f = shaw.Fom(m, 2, 3, precision=shaw.MIXED_FP32)
    rng = np.random.default_rng(2)
    vp, sp = rng.standard_normal((m.nvp, 3)), rng.standard_normal((m.nsp, 3))
    f.set_state(vp, sp)
    gv, gs = f.get_state()
    assert np.array_equal(gv, vp.astype(np.float32).astype(np.float64))
    assert np.array_equal(gs, sp.astype(np.float32).astype(np.float64))
