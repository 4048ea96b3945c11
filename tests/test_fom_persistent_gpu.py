"""The rank-1 FOM as one persistent cooperative launch (SHAW_FOM_SCHEDULE_PERSISTENT, the
default for rank-1 FP64 handles on grids whose bands fit one CTA per SM): row bands, or
column bands on grids wider than tall (201 x 101, 51 x 21, 7 x 5, 500 x 21, the 21 x 51
fixture).

The band kernel runs the two half-step kernels' FMAs in the same order, so its states
and seismograms must equal theirs bit for bit; it is also held to the oracle (1e-12
relative, max |gpu - oracle| / max |oracle|).  Grids cover bands of one, two and three
rows, a last band shorter than the others, and the reference fixtures; sources and
receivers sit on band boundaries, the axis and the surface; runs in pieces start from
any step, and a run repeated after reset() reuses the exchange words under new tags.
"""
import tempfile

import numpy as np
import pytest
import torch

from conftest import mesh_dir

pytestmark = pytest.mark.gpu

RTOL = 1e-12
MATERIAL = [3300.0, 2300.0 / 2891000.0, 0.0, 4400.0, 2900.0 / 2891000.0, 0.0]


def relerr(a, b):
    scale = np.max(np.abs(b))
    return np.max(np.abs(a - b)) / (scale if scale > 0 else 1.0)


def band_rows(nr):
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    return -(-nr // sms)


def generated(shaw, oracle, nth, nr):
    m = shaw.Mesh.generate(nth, nr)
    m.set_material("unilayer", MATERIAL)
    with tempfile.TemporaryDirectory() as d:
        oracle.write_full_mesh(nth, nr, d)
        om = oracle.OracleMesh(d)
    om.set_material("unilayer", [(MATERIAL[0:3], MATERIAL[3:6])])
    dt = 0.25 * min(m.info[5], m.info[4] * m.info[2]) / (np.sqrt(2.0) * 7300.0)
    return m, om, dt


def run(shaw, m, sched, src, rcv, dt, n, kind="ricker", period=None, delay=None, pieces=None, repeat=False,
        freq=1):
    f = shaw.Fom(m, 1, 1)
    f.set_schedule(sched)
    f.set_sources([src], kind, period, delay)
    f.set_receivers(rcv, freq, n)
    for _ in range(2 if repeat else 1):
        if pieces:
            f.reset()
            for k in pieces:
                f.advance(dt, k)
            f.synchronize()
        else:
            f.run(dt, n)
    out = (f.get_state(), f.seismogram(), f.kernel_launches)
    f.close()
    return out


@pytest.mark.parametrize("nth,nr", [(101, 201), (201, 101), (51, 21), (33, 400), (7, 5), (37, 153)])
def test_persistent_equals_two_half_steps_and_oracle(shaw, oracle, nth, nr):
    m, om, dt = generated(shaw, oracle, nth, nr)
    n = 300
    rows = band_rows(nr)
    # a source on the first row of the second band, receivers on band boundaries, the axis
    # and the surface
    src = min(rows, nr - 1) * nth + nth // 3
    rcv = [m.map_receiver(float(a)) for a in range(0, 181, 12)] + [0, nth - 1, rows * nth + 1,
                                                                    (rows - 1) * nth + 2,
                                                                    (nr - 1) * nth + nth // 2]
    period, delay = 40 * dt, 15 * dt
    (a, sa, la), (b, sb, lb) = (run(shaw, m, s, src, rcv, dt, n, "ricker", period, delay)
                                for s in (shaw.SCHEDULE_TWO_PASS, shaw.SCHEDULE_PERSISTENT))
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.array_equal(sa, sb) and np.max(np.abs(sa)) > 0
    assert lb < la  # one persistent launch (and its forcing table) instead of the half-step kernels
    ref = om.fom_run(1, n, dt, [src], [0], [period], [delay], rcv, 1, 0, 0)
    assert relerr(b[0], ref["final_vp"]) <= RTOL and relerr(b[1], ref["final_sp"]) <= RTOL
    assert relerr(sb, ref["seis"]) <= RTOL


def test_persistent_runs_in_pieces_repeats_and_fixture(shaw, oracle):
    m = shaw.Mesh.load(mesh_dir("fullMesh21x51"))
    m.set_material("unilayer", [2000.0, 0.0, 0.0, 5000.0, 0.0, 0.0])
    src = m.map_source(500.0, 30.0)
    rcv = [m.map_receiver(a) for a in (5, 45, 95, 135)]
    args = (src, rcv, 1.0, 150, "ricker", 40.0, 10.0)
    whole = run(shaw, m, shaw.SCHEDULE_PERSISTENT, *args)
    parts = run(shaw, m, shaw.SCHEDULE_PERSISTENT, *args, pieces=(1, 63, 64, 22))
    again = run(shaw, m, shaw.SCHEDULE_PERSISTENT, *args, pieces=(150,), repeat=True)
    two = run(shaw, m, shaw.SCHEDULE_TWO_PASS, *args)
    for x in (parts, again, two):
        assert np.array_equal(whole[0][0], x[0][0]) and np.array_equal(whole[0][1], x[0][1])
        assert np.array_equal(whole[1], x[1])
    # sampling every third step, with pieces that start at every sampling phase
    for pieces in ((1, 63, 64, 22), (2, 103, 45)):
        a = run(shaw, m, shaw.SCHEDULE_PERSISTENT, *args, pieces=pieces, freq=3)
        b = run(shaw, m, shaw.SCHEDULE_TWO_PASS, *args, pieces=pieces, freq=3)
        assert np.array_equal(a[0][0], b[0][0]) and np.array_equal(a[0][1], b[0][1])
        assert np.array_equal(a[1], b[1]) and np.max(np.abs(a[1])) > 0


def test_persistent_schedule_errors(shaw, oracle):
    m, _, _ = generated(shaw, oracle, 51, 21)
    f = shaw.Fom(m, 2, 4)
    with pytest.raises(shaw.ShawError) as e:
        f.set_schedule(shaw.SCHEDULE_PERSISTENT)
    assert e.value.code == shaw.ERR_UNSUPPORTED
    f.close()
    g = shaw.Fom(m, 1, 1, precision=shaw.MIXED_FP32)
    with pytest.raises(shaw.ShawError) as e:
        g.set_schedule(shaw.SCHEDULE_PERSISTENT)
    assert e.value.code == shaw.ERR_UNSUPPORTED
    g.close()
    # bands of more than 1024 points either way (row bands of 4 x 1100, column bands of
    # 8 x 600 points plus a halo line) keep the two half-step kernels
    wide = shaw.Mesh.generate(1100, 600)
    wide.set_material("unilayer", MATERIAL)
    h = shaw.Fom(wide, 1, 1)
    with pytest.raises(shaw.ShawError) as e:
        h.set_schedule(shaw.SCHEDULE_PERSISTENT)
    assert e.value.code == shaw.ERR_UNSUPPORTED
    h.close()


def test_persistent_handles_of_different_sizes(shaw, oracle):
    """A handle planned for a wide grid (76 KB of shared memory per band) still launches
    after a handle for a narrow grid (24 KB) was planned: the kernel's shared-memory limit
    is set at every launch.  Both equal the two half-step kernels bit for bit."""
    runs = {}
    handles = []
    for nth, nr in ((500, 21), (101, 201)):
        m, _, dt = generated(shaw, oracle, nth, nr)
        f = shaw.Fom(m, 1, 1)
        f.set_schedule(shaw.SCHEDULE_PERSISTENT)
        f.set_sources([(nr // 2) * nth + nth // 2], "ricker", 40 * dt, 10 * dt)
        f.set_receivers([0, (nr - 1) * nth + 3], 1, 120)
        handles.append((nth, nr, m, dt, f))
    for nth, nr, m, dt, f in handles:  # the wide grid runs last-planned-second
        f.run(dt, 120)
        runs[(nth, nr)] = (f.get_state(), f.seismogram())
        f.close()
    for nth, nr, m, dt, _ in handles:
        g = shaw.Fom(m, 1, 1)
        g.set_schedule(shaw.SCHEDULE_TWO_PASS)
        g.set_sources([(nr // 2) * nth + nth // 2], "ricker", 40 * dt, 10 * dt)
        g.set_receivers([0, (nr - 1) * nth + 3], 1, 120)
        g.run(dt, 120)
        (a, sa), b, sb = runs[(nth, nr)], g.get_state(), g.seismogram()
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and np.array_equal(sa, sb)
        g.close()
