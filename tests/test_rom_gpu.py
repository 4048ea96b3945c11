"""ROM parity on the GPU against the oracle: FP64 projection of the operators,
rank-1 (cluster-resident persistent kernel) and rank-2 (DGEMM) leapfrogs, the
in-loop ROM seismogram, and the mixed (FP32 hi+lo) rank-1 form against FP64.

Tolerances: FP64 paths 1e-12 relative (normwise) to the oracle; the mixed path
1e-6 relative (normwise, seismogram and states) to the FP64 GPU path.
"""
import numpy as np
import pytest

from conftest import mesh_dir

pytestmark = pytest.mark.gpu

MAT = [2000.0, 0.0, 0.0, 5000.0, 0.0, 0.0]


def relerr(a, b):
    s = np.max(np.abs(b))
    return np.max(np.abs(a - b)) / (s if s > 0 else 1.0)


@pytest.fixture(scope="module")
def setup(shaw, oracle):
    """POD bases of the 21x51 mesh from oracle FOM snapshots (numpy thin SVD)."""
    m = shaw.Mesh.load(mesh_dir("fullMesh21x51"))
    m.set_material("unilayer", MAT)
    om = oracle.OracleMesh(mesh_dir("fullMesh21x51"))
    om.set_material("unilayer", [(MAT[0:3], MAT[3:6])])
    snaps_v, snaps_s = [], []
    for d, a, p in ((400.0, 30.0, 40.0), (900.0, 60.0, 45.0), (1500.0, 120.0, 50.0), (700.0, 150.0, 60.0)):
        out = om.fom_run(1, 600, 1.0, [om.map_source(d, a)], [0], [p], [10.0], [], 0, 3, 3)
        snaps_v.append(out["snaps_vp"][:, :, 0])
        snaps_s.append(out["snaps_sp"][:, :, 0])
    uv = np.linalg.svd(np.hstack(snaps_v), full_matrices=False)[0]
    us = np.linalg.svd(np.hstack(snaps_s), full_matrices=False)[0]
    return m, om, uv, us


def test_projection_matches_oracle(shaw, setup):
    m, om, uv, us = setup
    for kv, ks in ((24, 40), (64, 64), (200, 256)):
        pv, ps = np.asfortranarray(uv[:, :kv]), np.asfortranarray(us[:, :ks])
        f = shaw.Fom(m, 1, 1)
        av, as_ = shaw.rom_project(f, pv, ps)
        ov, os_ = om.rom_operators(pv, ps)
        assert av.shape == (kv, ks) and as_.shape == (ks, kv)
        assert relerr(av, ov) <= 1e-12 and relerr(as_, os_) <= 1e-12
        f.close()


def _rom_inputs(shaw, setup, k, src_specs):
    m, om, uv, us = setup
    pv, ps = np.asfortranarray(uv[:, :k]), np.asfortranarray(us[:, :k])
    av, as_ = om.rom_operators(pv, ps)
    gids = [om.map_source(d, a) for d, a in src_specs]
    b = np.column_stack([om.rom_forcing_vector(pv, g) for g in gids])
    return pv, av, as_, b


@pytest.mark.parametrize("k", [32, 128, 256])
def test_rank1_fp64_matches_oracle(shaw, oracle, setup, k):
    pv, av, as_, b = _rom_inputs(shaw, setup, k, [(1111.0, 88.0)])
    n, dt = 2000, 1.0
    r = shaw.Rom(av, as_, b, rank=1)
    r.set_signals("ricker", 40.0, 10.0)
    r.set_snapshots(5, 5, n)
    rcv = [setup[0].map_receiver(a) for a in (10, 45, 90, 135, 170)]
    r.set_receivers(pv[rcv, :], 5, n)
    r.run(dt, n)
    ref = oracle.rom_run(av, as_, b, n, dt, [0], [40.0], [10.0], 5, 5)
    svp, ssp = r.snapshots()
    assert relerr(svp, ref["snaps_vp"]) <= 1e-12
    assert relerr(ssp, ref["snaps_sp"]) <= 1e-12
    xv, xs = r.get_state()
    assert relerr(xv, ref["final_vp"]) <= 1e-12 and relerr(xs, ref["final_sp"]) <= 1e-12
    seis = r.seismogram()[:, :, 0]
    assert relerr(seis, pv[rcv, :] @ ref["snaps_vp"][:, :, 0]) <= 1e-12
    # forcing table + the whole time loop in one persistent launch + the seismogram GEMM
    assert r.kernel_launches == 3
    r.close()


def stable_system(k, seed):
    """A reduced pair with As = -Av^T and ||dt Av|| < 2: the leapfrog is symplectic and
    bounded over any number of steps, so long runs measure arithmetic, not growth."""
    rng = np.random.default_rng(seed)
    q1 = np.linalg.qr(rng.standard_normal((k, k)))[0]
    q2 = np.linalg.qr(rng.standard_normal((k, k)))[0]
    av = q1 @ np.diag(np.linspace(0.05, 1.0, k)) @ q2.T
    return av, -av.T.copy(), rng.standard_normal(k) * 1e-3


def test_rank1_mixed_within_1e6_of_fp64(shaw):
    k, n, dt = 256, 20000, 0.5
    av, as_, b = stable_system(k, 5)
    pv = np.random.default_rng(6).standard_normal((13, k)) / np.sqrt(k)
    out = {}
    for prec in (shaw.FP64, shaw.MIXED_FP32):
        r = shaw.Rom(av, as_, b, rank=1, precision=prec)
        r.set_signals("gaussDer", 60.0, 180.0)
        r.set_receivers(pv, 1, n)
        r.run(dt, n)
        out[prec] = (r.seismogram(), r.get_state())
        r.close()
    assert np.max(np.abs(out[shaw.FP64][0])) > 0
    assert relerr(out[shaw.MIXED_FP32][0], out[shaw.FP64][0]) <= 1e-6
    assert relerr(out[shaw.MIXED_FP32][1][0], out[shaw.FP64][1][0]) <= 1e-6


def test_rank1_advance_in_pieces(shaw, setup):
    pv, av, as_, b = _rom_inputs(shaw, setup, 64, [(500.0, 45.0)])
    r = shaw.Rom(av, as_, b, rank=1)
    r.set_signals("sinusoid", 40.0, 0.0)
    r.run(1.0, 300)
    whole = r.get_state()
    r.reset()
    for k in (1, 99, 200):
        r.advance(1.0, k)
    r.synchronize()
    part = r.get_state()
    assert np.array_equal(whole[0], part[0]) and np.array_equal(whole[1], part[1])


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_rank1_seismogram_in_pieces(shaw, prec):
    """Seismogram samples (every 3 steps) of a run advanced in uneven pieces equal those
    of one uninterrupted run bit for bit, in both precisions (the mixed form widens each
    launch's samples to FP64 after the launch)."""
    k, n = 96, 300
    av, as_, b = stable_system(k, 12)
    rows = np.random.default_rng(13).standard_normal((9, k)) / np.sqrt(k)
    p = shaw.FP64 if prec == "fp64" else shaw.MIXED_FP32
    r = shaw.Rom(av * 0.5, as_ * 0.5, b, rank=1, precision=p)
    r.set_signals("gaussDer", 40.0, 30.0)
    r.set_receivers(rows, 3, n)
    r.run(0.5, n)
    whole = r.seismogram().copy()
    r.reset()
    for m in (1, 98, 2, 199):
        r.advance(0.5, m)
    r.synchronize()
    assert np.max(np.abs(whole)) > 0
    assert np.array_equal(r.seismogram(), whole)
    r.close()


@pytest.mark.parametrize("M", [1, 5, 16])
def test_rank2_fp64_matches_oracle(shaw, oracle, setup, M):
    rng = np.random.default_rng(M)
    specs = [(float(rng.uniform(200, 1500)), float(rng.uniform(0, 180))) for _ in range(M)]
    pv, av, as_, b = _rom_inputs(shaw, setup, 48, specs)
    periods = rng.uniform(30, 90, M)
    n, dt = 400, 1.0
    r = shaw.Rom(av, as_, b, rank=2)
    r.set_signals("gaussDer", periods, 100.0)
    r.set_snapshots(4, 8, n)
    rcv = [setup[0].map_receiver(a) for a in (20, 80, 160)]
    r.set_receivers(pv[rcv, :], 2, n)
    r.run(dt, n)
    ref = oracle.rom_run(av, as_, b, n, dt, [2] * M, periods, [100.0] * M, 4, 8)
    svp, ssp = r.snapshots()
    assert relerr(svp, ref["snaps_vp"]) <= 1e-12 and relerr(ssp, ref["snaps_sp"]) <= 1e-12
    xv, xs = r.get_state()
    assert relerr(xv, ref["final_vp"]) <= 1e-12 and relerr(xs, ref["final_sp"]) <= 1e-12
    seis = r.seismogram()  # every 2 steps; snapshots every 4: odd seismogram samples are the snapshot steps
    expect = np.einsum("rk,ktm->rtm", pv[rcv, :], ref["snaps_vp"])
    assert relerr(seis[:, 1::2, :], expect) <= 1e-12


def test_rom_error_paths(shaw, setup):
    pv, av, as_, b = _rom_inputs(shaw, setup, 16, [(500.0, 45.0)])
    with pytest.raises(shaw.ShawError) as e:
        shaw.Rom(av, as_, np.column_stack([b, b]), rank=1)
    assert e.value.code == shaw.ERR_INVALID_ARG
    r = shaw.Rom(av, as_, b, rank=1)
    with pytest.raises(shaw.ShawError) as e:
        r.run(1.0, 10)
    assert e.value.code == shaw.ERR_STATE
    with pytest.raises(shaw.ShawError) as e:
        r.set_snapshots(3, 3, 10)
    assert e.value.code == shaw.ERR_FREQ_DIVISOR


def _fp64_vs_mixed(shaw, prec, k_v, k_s, M, n, dt, seed, freq=0, smax=1.0):
    rng = np.random.default_rng(seed)
    kmin = min(k_v, k_s)
    av, as_, _ = stable_system(kmin, seed)
    av, as_ = av * smax, as_ * smax
    if k_v != k_s:  # embed the stable square pair in a rectangular one
        big_v = np.zeros((k_v, k_s))
        big_v[:kmin, :kmin] = av
        big_s = np.zeros((k_s, k_v))
        big_s[:kmin, :kmin] = as_
        av, as_ = big_v, big_s
    b = rng.standard_normal((k_v, M)) * 1e-3
    periods = rng.uniform(30, 90, M)
    out = {}
    for p in (shaw.FP64, prec):
        r = shaw.Rom(av, as_, b, rank=2, precision=p)
        r.set_signals("gaussDer", periods, 40.0)
        if freq:
            r.set_snapshots(freq, freq, n)
        r.run(dt, n)
        out[p] = (r.get_state(), r.snapshots())
        r.close()
    return out[shaw.FP64], out[prec]


def test_rank2_tf32x3_tensor_core_tiny(shaw):
    """One CTA, one 128-mode tile, a few steps: the tcgen05 TF32x3 pipeline end to end.
    The tensor pipe accumulates in FP32 with truncation, so this form is held to 1e-5."""
    ((xv64, xs64), _), ((xvtc, xstc), _) = _fp64_vs_mixed(shaw, shaw.MIXED_TF32X3, 128, 128, 32, 20, 0.5, 1)
    assert np.max(np.abs(xv64)) > 0
    assert relerr(xvtc, xv64) <= 1e-5 and relerr(xstc, xs64) <= 1e-5


@pytest.mark.parametrize("kv,ks,M", [(100, 72, 45), (256, 256, 300), (512, 512, 64)])
def test_rank2_tf32x3_tensor_core_short_runs(shaw, kv, ks, M):
    ((xv64, xs64), (sv64, ss64)), ((xvtc, xstc), (svtc, sstc)) = _fp64_vs_mixed(
        shaw, shaw.MIXED_TF32X3, kv, ks, M, 200, 0.5, kv + M, freq=50, smax=0.2)
    # the truncating FP32 accumulation biases each GEMM by ~1e-6 relative at K = 512
    for a, b in ((xvtc, xv64), (xstc, xs64), (svtc, sv64), (sstc, ss64)):
        assert relerr(a, b) <= 5e-5


def test_rank2_ozaki_tiny(shaw):
    """One CTA, one 128-mode tile, a few steps: BF16 slices with exact accumulation."""
    ((xv64, xs64), _), ((xvoz, xsoz), _) = _fp64_vs_mixed(shaw, shaw.MIXED_OZAKI_BF16, 128, 128, 32, 20, 0.5, 1)
    assert np.max(np.abs(xv64)) > 0
    assert relerr(xvoz, xv64) <= 1e-9 and relerr(xsoz, xs64) <= 1e-9


@pytest.mark.parametrize("kv,ks,M", [(100, 72, 45), (256, 256, 300), (512, 512, 64), (1024, 640, 40)])
def test_rank2_ozaki_long_runs_within_1e6(shaw, kv, ks, M):
    ((xv64, xs64), (sv64, ss64)), ((xvoz, xsoz), (svoz, ssoz)) = _fp64_vs_mixed(
        shaw, shaw.MIXED_OZAKI_BF16, kv, ks, M, 2000, 0.5, kv + M, freq=50, smax=0.2)
    errs = [relerr(a, b) for a, b in ((xvoz, xv64), (xsoz, xs64), (svoz, sv64), (ssoz, ss64))]
    assert max(errs) <= 1e-8, errs
    rows = np.random.default_rng(0).standard_normal((7, kv)) / np.sqrt(kv)
    assert relerr(np.einsum("rk,ktm->rtm", rows, svoz), np.einsum("rk,ktm->rtm", rows, sv64)) <= 1e-8


def test_rank2_ozaki_advance_in_pieces(shaw):
    av, as_, _ = stable_system(128, 9)
    b = np.random.default_rng(9).standard_normal((128, 40)) * 1e-3
    r = shaw.Rom(av * 0.2, as_ * 0.2, b, rank=2, precision=shaw.MIXED_OZAKI_BF16)
    r.set_signals("ricker", 40.0, 20.0)
    r.run(0.5, 100)
    whole = r.get_state()
    r.reset()
    r.advance(0.5, 30)
    r.advance(0.5, 70)
    r.synchronize()
    part = r.get_state()
    assert np.array_equal(whole[0], part[0]) and np.array_equal(whole[1], part[1])


@pytest.mark.parametrize("R,freq", [(5, 1), (181, 2)])
def test_rank2_ozaki_in_loop_seismogram(shaw, R, freq):
    """Receivers on the tensor-core path: the seismogram formed inside the persistent
    kernel (exact sliced product of the receiver rows with the velocity state) against
    the FP64 path's DGEMM seismogram; a run in pieces gives the same samples."""
    kv, ks, M, n, dt = 200, 160, 70, 400, 0.5
    av, as_, _ = stable_system(ks, 21)
    big_v = np.zeros((kv, ks))
    big_v[:ks, :ks] = av * 0.2
    big_s = np.zeros((ks, kv))
    big_s[:ks, :ks] = as_ * 0.2
    rng = np.random.default_rng(R)
    b = rng.standard_normal((kv, M)) * 1e-3
    rows = rng.standard_normal((R, kv)) / np.sqrt(kv)
    periods = rng.uniform(30, 90, M)
    out = {}
    for p in (shaw.FP64, shaw.MIXED_OZAKI_BF16):
        r = shaw.Rom(big_v, big_s, b, rank=2, precision=p)
        r.set_signals("gaussDer", periods, 40.0)
        r.set_receivers(rows, freq, n)
        r.run(dt, n)
        out[p] = r.seismogram()
        if p == shaw.MIXED_OZAKI_BF16:
            r.reset()
            r.advance(dt, 100)
            r.advance(dt, n - 100)
            r.synchronize()
            assert np.array_equal(r.seismogram(), out[p])
        r.close()
    assert out[shaw.FP64].shape == (R, n // freq, M)
    assert np.max(np.abs(out[shaw.FP64])) > 0
    assert relerr(out[shaw.MIXED_OZAKI_BF16], out[shaw.FP64]) <= 1e-8


def test_rank2_tf32x3_receivers_unsupported(shaw):
    av, as_, _ = stable_system(128, 3)
    r = shaw.Rom(av * 0.2, as_ * 0.2, np.ones((128, 4)) * 1e-3, rank=2, precision=shaw.MIXED_TF32X3)
    with pytest.raises(shaw.ShawError) as e:
        r.set_receivers(np.ones((3, 128)), 1, 10)
    assert e.value.code == shaw.ERR_UNSUPPORTED
    r.close()


# ---- SHAW_OZAKI_FP64: 9 six-bit slices, FP64 state: held to the FP64 bar -----------------

@pytest.mark.parametrize("M", [1, 5, 16])
def test_rank2_ozaki_fp64_matches_oracle(shaw, oracle, setup, M):
    """The FP64-grade tensor-core form against the oracle at the FP64 path's bar (1e-12):
    snapshots, final states and the in-loop seismogram."""
    rng = np.random.default_rng(M)
    specs = [(float(rng.uniform(200, 1500)), float(rng.uniform(0, 180))) for _ in range(M)]
    pv, av, as_, b = _rom_inputs(shaw, setup, 48, specs)
    periods = rng.uniform(30, 90, M)
    n, dt = 400, 1.0
    r = shaw.Rom(av, as_, b, rank=2, precision=shaw.OZAKI_FP64)
    r.set_signals("gaussDer", periods, 100.0)
    r.set_snapshots(4, 8, n)
    rcv = [setup[0].map_receiver(a) for a in (20, 80, 160)]
    r.set_receivers(pv[rcv, :], 2, n)
    r.run(dt, n)
    ref = oracle.rom_run(av, as_, b, n, dt, [2] * M, periods, [100.0] * M, 4, 8)
    svp, ssp = r.snapshots()
    assert relerr(svp, ref["snaps_vp"]) <= 1e-12 and relerr(ssp, ref["snaps_sp"]) <= 1e-12
    xv, xs = r.get_state()
    assert relerr(xv, ref["final_vp"]) <= 1e-12 and relerr(xs, ref["final_sp"]) <= 1e-12
    seis = r.seismogram()
    expect = np.einsum("rk,ktm->rtm", pv[rcv, :], ref["snaps_vp"])
    assert relerr(seis[:, 1::2, :], expect) <= 1e-12
    r.close()


@pytest.mark.parametrize("kv,ks,M", [(100, 72, 45), (256, 256, 300), (512, 512, 64), (1024, 640, 40)])
def test_rank2_ozaki_fp64_long_runs_within_1e12(shaw, kv, ks, M):
    """2000 steps against the FP64 (DGEMM) path: states and snapshots within 1e-12."""
    ((xv64, xs64), (sv64, ss64)), ((xvoz, xsoz), (svoz, ssoz)) = _fp64_vs_mixed(
        shaw, shaw.OZAKI_FP64, kv, ks, M, 2000, 0.5, kv + M + 1, freq=50, smax=0.2)
    errs = [relerr(a, b) for a, b in ((xvoz, xv64), (xsoz, xs64), (svoz, sv64), (ssoz, ss64))]
    assert max(errs) <= 1e-12, errs


def test_rank2_ozaki_fp64_advance_in_pieces(shaw):
    av, as_, _ = stable_system(256, 19)
    b = np.random.default_rng(19).standard_normal((256, 40)) * 1e-3
    r = shaw.Rom(av * 0.2, as_ * 0.2, b, rank=2, precision=shaw.OZAKI_FP64)
    r.set_signals("ricker", 40.0, 20.0)
    r.run(0.5, 100)
    whole = r.get_state()
    r.reset()
    r.advance(0.5, 31)
    r.advance(0.5, 69)
    r.synchronize()
    part = r.get_state()
    assert np.array_equal(whole[0], part[0]) and np.array_equal(whole[1], part[1])
    r.close()


def _bounded_pair(kv, ks, seed):
    """Av (kv x ks) with As = -Av^T (ks x kv): a symplectic, bounded rank-1 leapfrog at dt 0.5."""
    rng = np.random.default_rng(seed)
    av = rng.standard_normal((kv, ks)) * (0.5 / np.sqrt(max(kv, ks)))
    return av, -av.T.copy(), rng.standard_normal(kv) * 1e-3, rng.standard_normal((7, kv)) / np.sqrt(kv)


@pytest.mark.parametrize("kv,ks", [(32, 32), (256, 256), (200, 256), (513, 384)])
def test_rank1_bands_equal_cluster(shaw, kv, ks):
    """The row-band launch (the FP64 default) and the cluster launch run the same row
    arithmetic, so states, snapshots and seismograms agree bit for bit, also when the run
    is advanced in uneven pieces (each piece a launch with new exchange tags)."""
    av, as_, b, rows = _bounded_pair(kv, ks, kv + ks)
    n = 400
    out = {}
    for sched in (shaw.ROM_SCHEDULE_CLUSTER, shaw.ROM_SCHEDULE_BANDS):
        r = shaw.Rom(av, as_, b, rank=1)
        r.set_schedule(sched)
        r.set_signals("ricker", 40.0, 10.0)
        r.set_snapshots(4, 4, n)
        r.set_receivers(rows, 2, n)
        r.run(0.5, n)
        whole = (r.get_state(), tuple(x.copy() for x in r.snapshots()), r.seismogram().copy())
        r.reset()
        for m in (1, 150, 249):
            r.advance(0.5, m)
        r.synchronize()
        parts = (r.get_state(), tuple(x.copy() for x in r.snapshots()), r.seismogram().copy())
        r.close()
        for x, y in zip(whole[0] + whole[1] + (whole[2],), parts[0] + parts[1] + (parts[2],)):
            assert np.array_equal(x, y)
        out[sched] = whole
    a, c = out[shaw.ROM_SCHEDULE_BANDS], out[shaw.ROM_SCHEDULE_CLUSTER]
    for x, y in zip(a[0] + a[1] + (a[2],), c[0] + c[1] + (c[2],)):
        assert np.array_equal(x, y)
    assert np.max(np.abs(a[2])) > 0


def test_rank1_bands_1024_modes_match_oracle(shaw, oracle):
    """1024 modes per dof: the operators no longer fit a 16-CTA cluster; the row bands run
    them (one CTA per SM, seven rows each on 152 SMs) within 1e-12 of the oracle."""
    k, n, dt = 1024, 300, 0.5
    av, as_, b, rows = _bounded_pair(k, k, 99)
    r = shaw.Rom(av, as_, b, rank=1)
    r.set_signals("gaussDer", 30.0, 20.0)
    r.set_snapshots(10, 10, n)
    r.run(dt, n)
    ref = oracle.rom_run(av, as_, b.reshape(-1, 1), n, dt, [2], [30.0], [20.0], 10, 10)
    xv, xs = r.get_state()
    assert relerr(xv, ref["final_vp"]) <= 1e-12 and relerr(xs, ref["final_sp"]) <= 1e-12
    svp, ssp = r.snapshots()
    assert relerr(svp, ref["snaps_vp"]) <= 1e-12 and relerr(ssp, ref["snaps_sp"]) <= 1e-12
    with pytest.raises(shaw.ShawError) as e:
        r.set_schedule(shaw.ROM_SCHEDULE_CLUSTER)
    assert e.value.code == shaw.ERR_UNSUPPORTED
    r.close()


def test_rom_schedule_errors(shaw):
    av, as_, b, _ = _bounded_pair(64, 64, 3)
    r = shaw.Rom(av, as_, b, rank=1, precision=shaw.MIXED_FP32)
    r.set_schedule(shaw.ROM_SCHEDULE_AUTO)
    for sched in (shaw.ROM_SCHEDULE_CLUSTER, shaw.ROM_SCHEDULE_BANDS):
        with pytest.raises(shaw.ShawError) as e:
            r.set_schedule(sched)
        assert e.value.code == shaw.ERR_UNSUPPORTED
    r.close()
    r = shaw.Rom(av, as_, np.column_stack([b, b]), rank=2)
    with pytest.raises(shaw.ShawError) as e:
        r.set_schedule(shaw.ROM_SCHEDULE_BANDS)
    assert e.value.code == shaw.ERR_UNSUPPORTED
    with pytest.raises(shaw.ShawError) as e:
        r.set_schedule(7)
    assert e.value.code == shaw.ERR_INVALID_ARG
    r.close()


def test_rank1_bands_handles_of_different_sizes(shaw):
    """A 1024-mode band handle (its kernel's shared memory far above a 64-mode handle's)
    still launches after the smaller handle was planned, and equals a run of its own."""
    big = _bounded_pair(1024, 1024, 21)
    small = _bounded_pair(64, 64, 22)
    rb = shaw.Rom(big[0], big[1], big[2], rank=1)
    rs = shaw.Rom(small[0], small[1], small[2], rank=1)
    for r in (rb, rs):
        r.set_signals("ricker", 40.0, 10.0)
        r.run(0.5, 100)
    xb = rb.get_state()
    rb.close()
    rs.close()
    r = shaw.Rom(big[0], big[1], big[2], rank=1)
    r.set_signals("ricker", 40.0, 10.0)
    r.run(0.5, 100)
    x = r.get_state()
    assert np.array_equal(x[0], xb[0]) and np.array_equal(x[1], xb[1])
    r.close()
