"""The single-sweep FOM leapfrog (one kernel per step, TMA-staged tiles, alternating
state buffers) against the oracle and against the two half-step kernels.

  * SHAW_FP64: 1e-12 relative to the oracle (max |gpu - oracle| / max |oracle| per array).
  * SHAW_FP64 and SHAW_MIXED_FP32: the same FMAs in the same order as the two half-step
    kernels, so the states and seismograms are bit-identical to theirs.
Grids cover partial theta strips (nth not a multiple of 16, a strip holding only the
axis point), several r segments, a segment starting on the surface row, sources on the
axis, the CMB and the surface, corner receivers, runs in pieces with odd step counts
(buffer parity), CUDA-graph chunks and snapshots; column counts 32, 64 and 128 cover
one, two and four forcing columns per lane.
"""
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12
MATERIAL = [3300.0, 2300.0 / 2891000.0, 0.0, 4400.0, 2900.0 / 2891000.0, 0.0]


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


def sources(m, M, seed):
    """M sources: axis, CMB, surface, corners and seeded interior points."""
    nth, nr = m.nth, m.nr
    fixed = [0, nth - 1, 5, (nr - 1) * nth + 3, nth * nr - 1, (nr - 1) * nth, nth + 1, nth * (nr // 2) + nth // 2]
    rng = np.random.default_rng(seed)
    rest = list(rng.integers(0, m.nvp, M - len(fixed)))
    return [int(g) for g in fixed + rest]


GRIDS = [(51, 21), (17, 40), (100, 201), (37, 33)]


@pytest.mark.parametrize("nth,nr", GRIDS)
@pytest.mark.parametrize("M", [32, 64])
def test_sweep_fp64_matches_oracle(shaw, oracle, nth, nr, M):
    m, om, dt = grids(shaw, oracle, nth, nr)
    n = 150
    gids = sources(m, M, nth + nr)
    rng = np.random.default_rng(nr)
    periods = rng.uniform(0.5, 3.0, M) * 40 * dt
    kinds = [int(k) for k in rng.integers(0, 3, M)]
    delays = list(rng.uniform(0.0, 20.0 * dt, M))
    rcv = [0, nth - 1, (nr - 1) * nth, m.nvp - 1] + gids[8:16]
    f = shaw.Fom(m, 2, M)
    f.set_schedule(shaw.SCHEDULE_SWEEP)
    f.set_sources(gids, kinds, periods, delays)
    f.set_receivers(rcv, 1, n)
    f.run(dt, n)
    ref = om.fom_run(2, n, dt, gids, kinds, periods, delays, rcv, 1, 0, 0)
    vp, sp = f.get_state()
    assert relerr(vp, ref["final_vp"]) <= RTOL and relerr(sp, ref["final_sp"]) <= RTOL
    assert relerr(f.seismogram(), ref["seis"]) <= RTOL
    # from a random state (every coefficient at O(1) values)
    xv = rng.standard_normal((m.nvp, M))
    xs = rng.standard_normal((m.nsp, M)) * 1e4
    f.set_receivers([], 0, 0)
    f.reset()
    f.set_state(xv, xs)
    f.advance(dt, 37)
    f.synchronize()
    vp, sp = f.get_state()
    om.fom_advance_forced(xv, xs, 0, 37, dt, gids, kinds, periods, delays)
    assert relerr(vp, xv) <= RTOL and relerr(sp, xs) <= RTOL
    f.close()


@pytest.mark.parametrize("nth,nr", GRIDS)
@pytest.mark.parametrize("prec,M", [("fp64", 64), ("fp64", 32), ("fp32", 128), ("fp32", 64), ("fp32", 32)])
def test_sweep_equals_two_half_steps_bitwise(shaw, oracle, nth, nr, prec, M):
    m, _, dt = grids(shaw, oracle, nth, nr)
    n = 140  # 2 graph chunks + 12 single steps
    gids = sources(m, M, 7 * nth)
    rng = np.random.default_rng(nth)
    periods = rng.uniform(0.5, 3.0, M) * 40 * dt
    rcv = [0, nth - 1, (nr - 1) * nth + 1, m.nvp - 1] + gids[:6]
    precision = shaw.FP64 if prec == "fp64" else shaw.MIXED_FP32
    out = []
    for sched in (shaw.SCHEDULE_TWO_PASS, shaw.SCHEDULE_SWEEP):
        f = shaw.Fom(m, 2, M, precision=precision)
        f.set_schedule(sched)
        f.set_sources(gids, "ricker", periods, 10 * dt)
        f.set_receivers(rcv, 1, n)
        f.run(dt, n)
        out.append((f.get_state(), f.seismogram()))
        f.close()
    (a, sa), (b, sb) = out
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.array_equal(sa, sb)
    assert np.max(np.abs(sa)) > 0


def test_sweep_pieces_graphs_and_snapshots(shaw, oracle):
    """Odd step counts between calls (the state buffers alternate each step), graph chunks
    and per-step launches, and snapshots, all equal to one uninterrupted run."""
    m, om, dt = grids(shaw, oracle, 51, 70)
    M, n = 64, 200
    gids = sources(m, M, 3)
    periods = np.linspace(30, 80, M) * dt
    rcv = [m.map_receiver(float(a)) for a in range(0, 181, 15)] + gids[:4]
    f = shaw.Fom(m, 2, M)
    f.set_schedule(shaw.SCHEDULE_SWEEP)
    f.set_sources(gids, "gaussDer", periods, 15 * dt)
    f.set_receivers(rcv, 1, n)
    f.run(dt, n)
    whole_seis = f.seismogram()
    whole = f.get_state()
    f.reset()
    for k in (1, 63, 64, 65, 7):  # crosses graph chunks with both buffer parities
        f.advance(dt, k)
    f.synchronize()
    assert np.array_equal(f.seismogram(), whole_seis)
    vp, sp = f.get_state()
    assert np.array_equal(vp, whole[0]) and np.array_equal(sp, whole[1])
    f.set_snapshots(5, 10, n)
    f.run(dt, n)
    svp, ssp = f.snapshots()
    assert np.array_equal(f.seismogram(), whole_seis)
    ref = om.fom_run(2, n, dt, gids, [2] * M, periods, [15 * dt] * M, rcv, 1, 5, 10)
    assert relerr(svp, ref["snaps_vp"]) <= RTOL and relerr(ssp, ref["snaps_sp"]) <= RTOL
    assert np.array_equal(svp[:, -1, :], whole[0]) and np.array_equal(ssp[:, -1, :], whole[1])
    f.close()


def test_sweep_schedule_errors(shaw, oracle):
    m, _, _ = grids(shaw, oracle, 51, 21)
    f = shaw.Fom(m, 2, 12)  # 12 columns: the two half-step kernels only
    with pytest.raises(shaw.ShawError) as e:
        f.set_schedule(shaw.SCHEDULE_SWEEP)
    assert e.value.code == shaw.ERR_UNSUPPORTED
    with pytest.raises(shaw.ShawError) as e:
        f.set_schedule(7)
    assert e.value.code == shaw.ERR_INVALID_ARG
    f.set_schedule(shaw.SCHEDULE_TWO_PASS)
    f.set_schedule(shaw.SCHEDULE_AUTO)
    f.close()
