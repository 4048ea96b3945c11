"""FOM parity on the GPU: the sm_103a stencil kernels through the C ABI against the
CPU oracle (and, through the input-file driver, against the reference's golds).

Tolerance: FP64 runs must agree with the oracle to 1e-12 relative, measured
normwise (max |gpu - oracle| / max |oracle| over the compared array); the GPU
folds dt into the stencil values and uses FMAs, the oracle rounds as the
reference's CRS kernels do, so bit equality is not expected.
"""
import os
import subprocess

import numpy as np
import pytest

from cases import CASES, as_text_layout, parse_case, read_output, run_case
from conftest import GOLDEN, mesh_dir

pytestmark = pytest.mark.gpu

RTOL = 1e-12
CFG_MATERIAL = [3300.0, 2300.0 / 2891000.0, 0.0, 4400.0, 2900.0 / 2891000.0, 0.0]


def relerr(a, b):
    scale = np.max(np.abs(b))
    return np.max(np.abs(a - b)) / (scale if scale > 0 else 1.0)


def meshes(shaw, oracle, name, mat=("unilayer", [2000.0, 0.0, 0.0, 5000.0, 0.0, 0.0])):
    m = shaw.Mesh.load(mesh_dir(name))
    m.set_material(*mat)
    om = oracle.OracleMesh(mesh_dir(name))
    kind, p = mat
    om.set_material(kind, [(p[0:3], p[3:6])] if kind == "unilayer" else [])
    return m, om


def crs_apply(ptr, ind, val, x):
    rows = np.repeat(np.arange(len(ptr) - 1), np.diff(ptr).astype(np.int64))
    out = np.zeros((len(ptr) - 1, x.shape[1]))
    np.add.at(out, rows, val[:, None] * x[ind.astype(np.int64)])
    return out


@pytest.mark.parametrize("rank,M", [(1, 1), (2, 1), (2, 3), (2, 8)])
def test_half_steps_match_oracle_operators(shaw, oracle, rank, M):
    m, om = meshes(shaw, oracle, "fullMesh21x51")
    f = shaw.Fom(m, rank, M)
    rng = np.random.default_rng(11 + M)
    vp = rng.standard_normal((m.nvp, M))
    sp = rng.standard_normal((m.nsp, M)) * 1e4
    f.set_sources([m.nvp - 1] * M, ["ricker"] * M, [40.0] * M, [1e9] * M)  # signal ~0 at t=0 (exp underflow)
    f.set_state(vp, sp)
    dt = 0.5
    f.update_velocity(dt, 1)
    v1, s1 = f.get_state()
    pv, iv, av = om.crs(0)
    ref_v = vp + dt * crs_apply(pv, iv, av, sp)
    assert relerr(v1, ref_v) <= 1e-13
    assert np.array_equal(s1, sp)
    f.update_stress(dt)
    v2, s2 = f.get_state()
    ps, is_, as_ = om.crs(1)
    ref_s = sp + dt * crs_apply(ps, is_, as_, v1)
    assert relerr(s2, ref_s) <= 1e-13
    assert np.array_equal(v2, v1)


@pytest.mark.parametrize("case", CASES)
def test_runs_match_oracle(shaw, oracle, case):
    c = parse_case(case)
    m, om = meshes(shaw, oracle, c["mesh"])
    ref = run_case(om, c)
    rcv = [m.map_receiver(a) for a in c["receivers"]]
    rank = 1 if c["forcing_size"] is None else 2
    M = 1 if rank == 1 else c["forcing_size"]
    reals = c["realizations"]
    for rid, out in ref.items():
        s = reals[rid * M:(rid + 1) * M] if rank == 2 else [reals[rid]]
        f = shaw.Fom(m, rank, M)
        f.set_sources([m.map_source(d, a) for (d, _, a, _) in s], [c["kind"]] * M, [p for (_, p, _, _) in s],
                      [de for (_, _, _, de) in s])
        f.set_receivers(rcv, c["freq_seis"], c["nsteps"])
        f.set_snapshots(c["freq_vp"], c["freq_sp"], c["nsteps"])
        f.run(c["dt"], c["nsteps"])
        svp, ssp = f.snapshots()
        assert relerr(svp, out["snaps_vp"]) <= RTOL
        assert relerr(ssp, out["snaps_sp"]) <= RTOL
        assert relerr(f.seismogram(), out["seis"]) <= RTOL
        f.close()


@pytest.mark.parametrize("case", CASES)
def test_input_file_driver_matches_reference_golds(shaw, oracle, case, tmp_path):
    """shaw_exe <input.yaml> end to end: files, names, formats and values."""
    c = parse_case(case)
    os.symlink(mesh_dir(c["mesh"]), tmp_path / c["mesh"])
    src = os.path.join(GOLDEN, "cases", case, "input.yaml")
    r = subprocess.run([shaw.EXE_PATH, src], cwd=tmp_path, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    golds = np.load(os.path.join(GOLDEN, "regression_golds.npz"))
    m, om = meshes(shaw, oracle, c["mesh"])
    ref = run_case(om, c)
    rank = 1 if c["forcing_size"] is None else 2
    for rid, out in ref.items():
        for name, arr, hdr in (("snaps_vp", out["snaps_vp"], True), ("snaps_sp", out["snaps_sp"], True),
                               ("seismogram", out["seis"], False)):
            header, mine = read_output(str(tmp_path / ("%s_%d" % (name, rid))), hdr)
            expect = as_text_layout(arr, rank)
            assert mine.shape == expect.shape
            assert relerr(mine, expect) <= RTOL
            if hdr:
                assert header == list(arr.shape[:2]) + ([arr.shape[2]] if rank == 2 else [])
            key = "%s/%s_%d_gold" % (case, name, rid)
            if key in golds.files:
                tol = 1e-10 if name == "snaps_sp" else 1e-13
                assert np.allclose(mine, golds[key], atol=tol, rtol=0)
    assert (tmp_path / "coords_vp.txt").exists() and (tmp_path / "coords_sp.txt").exists()
    # the reference's log lines, in the forms its scaling scripts parse
    # (python_scripts_revise/log_file_extractor.py:9-114)
    import re
    for key in ("aveBandwidth", "minBandwidth", "maxBandwidth"):
        assert float(re.search(key + r"(\D+)\d+.\d+", r.stdout).group().split()[2]) > 0, key
    for key in ("aveGFlop", "aveTime", "flops/bytes", "loopTime", "dataCollectionTime"):
        assert re.search(re.escape(key) + r"(\D+)\d+.\d+", r.stdout), key
    assert int(re.search(r"numGptVp = \d+", r.stdout).group().split()[2]) == m.nvp
    assert int(re.search(r"numSteps(\D+)\d+", r.stdout).group().split()[2]) == c["nsteps"]


@pytest.mark.parametrize("grid", ["small", "large"])
def test_graph_replay_equals_direct_launches(shaw, oracle, grid):
    """Without snapshots a run of >= 64 steps replays CUDA-graph chunks (half-step kernels
    chained by programmatic dependent launch); with snapshots, per-step launches.
    Seismograms and final states agree bit for bit, on a small and a large grid."""
    if grid == "small":
        m, _ = meshes(shaw, oracle, "fullMesh21x51")
        n, M, dt = 200, 4, 1.0  # > one 64-step chunk, with a ragged tail
    else:
        m = shaw.Mesh.generate(1000, 2000)
        m.set_material("unilayer", CFG_MATERIAL)
        n, M = 70, 4
        dt = 0.25 * min(m.info[5], m.info[4] * m.info[2]) / (np.sqrt(2.0) * 7300.0)
    rcv = [m.map_receiver(a) for a in (10, 45, 90, 170)]
    out = []
    for snaps in (False, True):
        f = shaw.Fom(m, 2, M)
        f.set_sources([m.map_source(d, 45.0) for d in (300.0, 600.0, 900.0, 1200.0)], "ricker", 40.0, 10.0)
        f.set_receivers(rcv, 2, n)
        if snaps:
            f.set_snapshots(35 if grid == "large" else 50, 35 if grid == "large" else 50, n)  # per-step launches
        f.run(dt, n)
        out.append((f.seismogram(), f.get_state()))
        f.close()
    assert np.max(np.abs(out[0][1][0])) > 0  # (the large grid's surface receivers are still silent)
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1][0], out[1][1][0]) and np.array_equal(out[0][1][1], out[1][1][1])


def test_generated_large_mesh_rank2(shaw, oracle):
    """The 1000 x 2000 (theta x r) grid of the rank-2 workload, few steps, against the oracle."""
    m = shaw.Mesh.generate(1000, 2000)
    m.set_material("unilayer", CFG_MATERIAL)
    with_dir = os.path.join(os.environ.get("TMPDIR", "/tmp"), "shaw_mesh_1000x2000")
    os.makedirs(with_dir, exist_ok=True)
    m.write(with_dir)
    om = oracle.OracleMesh(with_dir)
    om.set_material("unilayer", [(CFG_MATERIAL[0:3], CFG_MATERIAL[3:6])])
    dt = 0.25 * min(m.info[5], m.info[4] * m.info[2]) / (np.sqrt(2.0) * 7300.0)
    M, n = 4, 12
    rng = np.random.default_rng(3)
    depths = rng.uniform(200, 700, M)
    periods = rng.uniform(30, 90, M)
    gids = [m.map_source(d, 0.0) for d in depths]
    assert gids == [om.map_source(d, 0.0) for d in depths]
    rcv = [m.map_receiver(a) for a in range(0, 181, 10)]
    f = shaw.Fom(m, 2, M)
    f.set_sources(gids, "gaussDer", periods, 1.0)
    f.set_receivers(rcv, 1, n)
    f.run(dt, n)
    vp, sp = f.get_state()
    ref = om.fom_run(2, n, dt, gids, [2] * M, periods, [1.0] * M, rcv, 1, 0, 0)
    assert relerr(vp, ref["final_vp"]) <= RTOL
    assert relerr(sp, ref["final_sp"]) <= RTOL
    assert relerr(f.seismogram(), ref["seis"]) <= RTOL


def test_sources_on_axis_and_surface_and_corner_receivers(shaw, oracle):
    m, om = meshes(shaw, oracle, "fullMesh21x51")
    nth, nr = m.nth, m.nr
    gids = [0, nth - 1, (nr - 1) * nth + 7, 5 * nth + 1, nth * nr - 1]  # axis, axis, surface, interior, corner
    M = len(gids)
    rcv = [0, nth - 1, (nr - 1) * nth, nth * nr - 1, 3]
    n = 40
    f = shaw.Fom(m, 2, M)
    f.set_sources(gids, ["ricker", "sinusoid", "gaussDer", "ricker", "sinusoid"], [30, 35, 40, 45, 50],
                  [5, 0, 10, 2, 0])
    f.set_receivers(rcv, 1, n)
    f.run(1.0, n)
    ref = om.fom_run(2, n, 1.0, gids, [0, 1, 2, 0, 1], [30, 35, 40, 45, 50], [5, 0, 10, 2, 0], rcv, 1, 0, 0)
    vp, sp = f.get_state()
    assert relerr(vp, ref["final_vp"]) <= RTOL
    assert relerr(sp, ref["final_sp"]) <= RTOL
    assert relerr(f.seismogram(), ref["seis"]) <= RTOL


def test_advance_in_pieces_equals_one_run(shaw, oracle):
    m, _ = meshes(shaw, oracle, "fullMesh21x51")
    rcv = [m.map_receiver(a) for a in (5, 95)]
    f = shaw.Fom(m, 1, 1)
    f.set_sources([m.map_source(500.0, 30.0)], "ricker", 40.0, 10.0)
    f.set_receivers(rcv, 1, 150)
    f.run(1.0, 150)
    whole = f.seismogram()
    f.reset()
    for k in (1, 63, 64, 22):  # crosses graph-chunk boundaries
        f.advance(1.0, k)
    f.synchronize()
    assert np.array_equal(f.seismogram(), whole)


def test_error_paths(shaw, oracle):
    m, _ = meshes(shaw, oracle, "fullMesh21x51")
    f = shaw.Fom(m, 1, 1)
    with pytest.raises(shaw.ShawError) as e:
        f.run(1.0, 10)
    assert e.value.code == shaw.ERR_STATE
    f.set_sources([10], "ricker", 40.0, 10.0)
    with pytest.raises(shaw.ShawError) as e:
        f.set_receivers([3], 7, 100)
    assert e.value.code == shaw.ERR_FREQ_DIVISOR
    with pytest.raises(shaw.ShawError) as e:
        f.set_snapshots(3, 7, 20)
    assert e.value.code == shaw.ERR_FREQ_DIVISOR
    with pytest.raises(shaw.ShawError) as e:
        f.set_sources([m.nvp], "ricker", 40.0, 10.0)
    assert e.value.code == shaw.ERR_INVALID_ARG
    # non-finite values reaching a receiver are reported after the run
    f.set_receivers([m.map_receiver(90.0)], 1, 5)
    f.reset()
    vp = np.zeros((m.nvp, 1))
    vp[m.map_receiver(90.0)] = np.nan
    f.set_state(vp, np.zeros((m.nsp, 1)))
    f.advance(1.0, 5)
    with pytest.raises(shaw.ShawError) as e:
        f.synchronize()
    assert e.value.code == shaw.ERR_NONFINITE


def test_config1_both_orientations_match_oracle(shaw, oracle, tmp_path):
    """Config 1 as worded (101 theta x 201 r) and the reference fixture's orientation
    (tests/fullMesh101x201: 201 theta x 101 r), axis source at 640 km, receivers every
    degree: GPU rank-1 run against the oracle."""
    for nth, nr in ((101, 201), (201, 101)):
        m = shaw.Mesh.generate(nth, nr)
        m.set_material("unilayer", CFG_MATERIAL)
        d = str(tmp_path / ("m%dx%d" % (nth, nr)))
        os.makedirs(d)
        m.write(d)
        om = oracle.OracleMesh(d)
        om.set_material("unilayer", [(CFG_MATERIAL[0:3], CFG_MATERIAL[3:6])])
        dt = 0.25 * min(m.info[5], m.info[4] * m.info[2]) / (np.sqrt(2.0) * 7300.0)
        n = 300
        src = m.map_source(640.0, 0.0)
        assert src == om.map_source(640.0, 0.0)
        rcv = [m.map_receiver(float(a)) for a in range(181)]
        f = shaw.Fom(m, 1, 1)
        f.set_sources([src], "gaussDer", 60.0, 20.0)
        f.set_receivers(rcv, 1, n)
        f.run(dt, n)
        ref = om.fom_run(1, n, dt, [src], [2], [60.0], [20.0], rcv, 1, 0, 0)
        vp, sp = f.get_state()
        assert relerr(vp, ref["final_vp"]) <= RTOL and relerr(sp, ref["final_sp"]) <= RTOL
        assert relerr(f.seismogram(), ref["seis"]) <= RTOL
        f.close()
