"""Batched rank-2 ROM: many reduced systems of uneven size in one handle.

Each instance is runRomRankTwoForcing's system (src/kokkos/torevise/
run_rom_rank_two_forcing.hpp:149-188).  FP64 batches are held to 1e-12 of the oracle
per instance; the tensor-core (Ozaki) batch must equal the single-system tensor-core
path bit for bit (exact accumulation makes the result independent of the tiling) and
stay within 1e-9 of FP64.
"""
import ctypes

import numpy as np
import pytest

from test_rom_gpu import relerr, stable_system

pytestmark = pytest.mark.gpu

# (kv, ks, M): uneven modes (not multiples of 128 included) and forcing counts
SHAPES = [(100, 72, 5), (128, 128, 37), (40, 40, 1), (256, 200, 70), (64, 96, 16)]


def _instances(seed, shapes=SHAPES, smax=0.2):
    rng = np.random.default_rng(seed)
    out = []
    for kv, ks, M in shapes:
        kmin = min(kv, ks)
        av, as_, _ = stable_system(kmin, int(rng.integers(1 << 30)))
        big_v = np.zeros((kv, ks))
        big_v[:kmin, :kmin] = av * smax
        big_s = np.zeros((ks, kv))
        big_s[:kmin, :kmin] = as_ * smax
        out.append(dict(rom_jvp=big_v, rom_jsp=big_s, b=rng.standard_normal((kv, M)) * 1e-3,
                        kind=rng.integers(0, 3, M), period=rng.uniform(30, 90, M), delay=rng.uniform(0, 60, M)))
    return out


def test_batch_fp64_matches_oracle(shaw, oracle):
    insts = _instances(1)
    n, dt = 300, 0.5
    bt = shaw.RomBatch(insts, precision=shaw.FP64)
    for i in range(len(insts)):
        bt.set_snapshots(i, 3, 5, n)
    bt.run(dt, n)
    for i, d in enumerate(insts):
        ref = oracle.rom_run(d["rom_jvp"], d["rom_jsp"], d["b"], n, dt, d["kind"], d["period"], d["delay"], 3, 5)
        xv, xs = bt.get_state(i)
        assert relerr(xv, ref["final_vp"]) <= 1e-12 and relerr(xs, ref["final_sp"]) <= 1e-12
        svp, ssp = bt.snapshots(i)
        assert relerr(svp, ref["snaps_vp"]) <= 1e-12 and relerr(ssp, ref["snaps_sp"]) <= 1e-12


def test_batch_fp64_equals_single_system_path(shaw):
    insts = _instances(2)
    n, dt = 120, 0.5
    bt = shaw.RomBatch(insts, precision=shaw.FP64)
    bt.run(dt, n)
    for i, d in enumerate(insts):
        r = shaw.Rom(d["rom_jvp"], d["rom_jsp"], d["b"], rank=2)
        r.set_signals(d["kind"], d["period"], d["delay"])
        r.run(dt, n)
        a, b = bt.get_state(i), r.get_state()
        assert relerr(a[0], b[0]) <= 1e-14 and relerr(a[1], b[1]) <= 1e-14
        r.close()


def test_batch_ozaki_bitwise_equals_single_system(shaw):
    insts = _instances(3)
    n, dt = 150, 0.5
    bt = shaw.RomBatch(insts, precision=shaw.MIXED_OZAKI_BF16)
    bt.run(dt, n)
    single = []
    for d in insts:
        r = shaw.Rom(d["rom_jvp"], d["rom_jsp"], d["b"], rank=2, precision=shaw.MIXED_OZAKI_BF16)
        r.set_signals(d["kind"], d["period"], d["delay"])
        r.run(dt, n)
        single.append(r.get_state())
        r.close()
    for i in range(len(insts)):
        a = bt.get_state(i)
        assert np.array_equal(a[0], single[i][0]) and np.array_equal(a[1], single[i][1])
    # the autotuner changes tile widths and the schedule, never the numbers
    report = bt.tune(dt, 3)
    assert "chosen" in report
    bt.run(dt, n)
    for i in range(len(insts)):
        a = bt.get_state(i)
        assert np.array_equal(a[0], single[i][0]) and np.array_equal(a[1], single[i][1])


def test_batch_ozaki_within_1e9_of_fp64(shaw):
    insts = _instances(4)
    n, dt = 1000, 0.5
    res = {}
    for p in (shaw.FP64, shaw.MIXED_OZAKI_BF16):
        bt = shaw.RomBatch(insts, precision=p)
        for i in range(len(insts)):
            bt.set_snapshots(i, 100, 100, n)
        bt.run(dt, n)
        res[p] = [(bt.get_state(i), bt.snapshots(i)) for i in range(len(insts))]
        bt.close()
    for i in range(len(insts)):
        (x64, s64), (xoz, soz) = res[shaw.FP64][i], res[shaw.MIXED_OZAKI_BF16][i]
        errs = [relerr(xoz[0], x64[0]), relerr(xoz[1], x64[1]), relerr(soz[0], s64[0]), relerr(soz[1], s64[1])]
        assert max(errs) <= 1e-9, (i, errs)


def test_batch_ozaki_advance_in_pieces_and_tiles(shaw):
    insts = _instances(5, shapes=[(384, 256, 100), (128, 128, 3), (512, 512, 33)])
    bt = shaw.RomBatch(insts, precision=shaw.MIXED_OZAKI_BF16)
    bt.run(0.5, 90)
    whole = [bt.get_state(i) for i in range(3)]
    bt.reset()
    bt.advance(0.5, 10)
    bt.advance(0.5, 80)
    bt.synchronize()
    for i in range(3):
        part = bt.get_state(i)
        assert np.array_equal(whole[i][0], part[0]) and np.array_equal(whole[i][1], part[1])
    assert "tile width" in bt.describe()


def test_batch_errors(shaw):
    good = _instances(6, shapes=[(32, 32, 4)])
    with pytest.raises(shaw.ShawError) as e:
        shaw.RomBatch(good, precision=shaw.MIXED_TF32X3)
    assert e.value.code == shaw.ERR_UNSUPPORTED
    big = _instances(6, shapes=[(1100, 64, 2)])
    with pytest.raises(shaw.ShawError) as e:
        shaw.RomBatch(big, precision=shaw.MIXED_OZAKI_BF16)
    assert e.value.code == shaw.ERR_UNSUPPORTED
    bad = _instances(6, shapes=[(32, 32, 4)])
    bad[0]["period"] = np.array([30.0, -1.0, 30.0, 30.0])
    with pytest.raises(shaw.ShawError) as e:
        shaw.RomBatch(bad, precision=shaw.FP64)
    assert e.value.code == shaw.ERR_INVALID_ARG
    bt = shaw.RomBatch(good, precision=shaw.FP64)
    x = np.zeros(32 * 4)
    xp = x.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    assert shaw.lib().shaw_rom_batch_get_state(bt.h, 3, xp, xp) == shaw.ERR_INVALID_ARG  # no instance 3
    bt.set_snapshots(0, 2, 2, 10)
    with pytest.raises(shaw.ShawError):
        bt.advance(0.5, 11)


def test_batch_seismograms(shaw):
    """Per-instance receivers: the FP64 batch equals the single-system FP64 path, the
    tensor-core batch (seismogram formed inside the persistent kernel) is within 1e-8."""
    insts = _instances(7)
    n, dt = 200, 0.5
    rng = np.random.default_rng(8)
    rows = [rng.standard_normal((R, d["rom_jvp"].shape[0])) for R, d in zip((3, 130, 1, 7, 20), insts)]
    freqs = (1, 2, 4, 1, 5)
    seis = {}
    for p in (shaw.FP64, shaw.MIXED_OZAKI_BF16):
        bt = shaw.RomBatch(insts, precision=p)
        for i in range(len(insts)):
            bt.set_receivers(i, rows[i], freqs[i], n)
        bt.run(dt, n)
        seis[p] = [bt.seismogram(i) for i in range(len(insts))]
        bt.close()
    for i, d in enumerate(insts):
        r = shaw.Rom(d["rom_jvp"], d["rom_jsp"], d["b"], rank=2)
        r.set_signals(d["kind"], d["period"], d["delay"])
        r.set_receivers(rows[i], freqs[i], n)
        r.run(dt, n)
        single = r.seismogram()
        r.close()
        assert seis[shaw.FP64][i].shape == single.shape
        assert np.max(np.abs(single)) > 0
        assert relerr(seis[shaw.FP64][i], single) <= 1e-14
        assert relerr(seis[shaw.MIXED_OZAKI_BF16][i], single) <= 1e-8


@pytest.mark.parametrize("width", [16, 64])
def test_batch_ozaki_paired_tiles_bitwise(shaw, width):
    """Tiles split across CTA pairs (each CTA half of the 128-row blocks, shared slices,
    a step barrier, level gates on the peer's row blocks) give the same numbers as whole
    tiles: states, snapshots and seismograms bit for bit, also when advanced in pieces
    and with an odd number of row blocks (384 modes) or a part without receiver rows (3
    receivers).  Width 16: two accumulator sets; width 64: one set staged in TMEM."""
    insts = _instances(9, shapes=[(384, 256, 100), (512, 512, 33), (256, 384, 20)])
    n, dt = 60, 0.5
    rng = np.random.default_rng(10)
    rows = [rng.standard_normal((R, d["rom_jvp"].shape[0])) for R, d in zip((130, 3, 7), insts)]
    out = {}
    for paired in (False, True):
        bt = shaw.RomBatch(insts, precision=shaw.MIXED_OZAKI_BF16)
        bt.set_tiling(width, paired=paired)
        assert ("pair" in bt.describe()) == paired
        for i in range(len(insts)):
            bt.set_snapshots(i, 7, 5, n)
            bt.set_receivers(i, rows[i], 3, n)
        bt.advance(dt, 25)
        bt.advance(dt, n - 25)
        bt.synchronize()
        out[paired] = [(bt.get_state(i), bt.snapshots(i), bt.seismogram(i)) for i in range(len(insts))]
        bt.close()
    for i in range(len(insts)):
        (xa, sa, ga), (xb, sb, gb) = out[False][i], out[True][i]
        for u, v in zip(xa + sa + (ga,), xb + sb + (gb,)):
            assert np.array_equal(u, v), i
        assert np.max(np.abs(ga)) > 0


def test_bounded_waits_report_timeouts(shaw):
    """Failure detection without a fault: the persistent kernels' waits are bounded.
    A wait on an mbarrier phase that nothing completes, one on a counter that nothing
    increments and one on a tagged exchange word that nothing writes (the band kernels'
    row exchange) each give up after the poll limit and report it (bits 64, 128, 256), and
    the device stays usable: a tensor-core batch runs right after and matches the FP64
    batch."""
    st = ctypes.c_uint32(0)
    assert shaw.lib().shaw_selftest_bounded_waits(1 << 14, ctypes.byref(st)) == 0
    assert st.value == 64 | 128 | 256
    assert shaw.lib().shaw_selftest_bounded_waits(0, ctypes.byref(st)) == shaw.ERR_INVALID_ARG
    # beyond the kernels' own wait limit (2^24 polls): refused before any launch
    assert shaw.lib().shaw_selftest_bounded_waits((1 << 24) + 1, ctypes.byref(st)) == shaw.ERR_INVALID_ARG
    assert shaw.lib().shaw_selftest_bounded_waits(2 ** 64 - 1, ctypes.byref(st)) == shaw.ERR_INVALID_ARG
    insts = _instances(21, shapes=[(256, 256, 16)])
    res = {}
    for p in (shaw.FP64, shaw.OZAKI_FP64):
        bt = shaw.RomBatch(insts, precision=p)
        bt.run(0.5, 40)
        res[p] = bt.get_state(0)
        bt.close()
    assert relerr(res[shaw.OZAKI_FP64][0], res[shaw.FP64][0]) <= 1e-12
    assert relerr(res[shaw.OZAKI_FP64][1], res[shaw.FP64][1]) <= 1e-12


def test_batch_tiling_errors(shaw):
    small = _instances(11, shapes=[(128, 256, 40)])
    bt = shaw.RomBatch(small, precision=shaw.MIXED_OZAKI_BF16)
    with pytest.raises(shaw.ShawError) as e:
        bt.set_tiling(32, paired=True)  # one 128-row block per velocity phase: nothing to split
    assert e.value.code == shaw.ERR_UNSUPPORTED
    with pytest.raises(shaw.ShawError) as e:
        bt.set_tiling(48)
    assert e.value.code == shaw.ERR_INVALID_ARG
    bt.close()
    bt = shaw.RomBatch(small, precision=shaw.FP64)
    with pytest.raises(shaw.ShawError) as e:
        bt.set_tiling(32)
    assert e.value.code == shaw.ERR_UNSUPPORTED
    bt.close()


def test_batch_ozaki_fp64_form(shaw):
    """The FP64-grade tensor-core batch: every instance within 1e-12 of the FP64 batch,
    bit for bit the single-system kernel (exact accumulation: independent of the tiling,
    paired or not), seismograms within 1e-12; tiles are at most 32 columns wide."""
    insts = _instances(14)
    n, dt = 300, 0.5
    rng = np.random.default_rng(15)
    rows = [rng.standard_normal((R, d["rom_jvp"].shape[0])) for R, d in zip((3, 130, 1, 7, 20), insts)]
    res = {}
    for p in (shaw.FP64, shaw.OZAKI_FP64):
        bt = shaw.RomBatch(insts, precision=p)
        for i in range(len(insts)):
            bt.set_snapshots(i, 25, 30, n)
            bt.set_receivers(i, rows[i], 4, n)
        bt.run(dt, n)
        res[p] = [(bt.get_state(i), bt.snapshots(i), bt.seismogram(i)) for i in range(len(insts))]
        if p == shaw.OZAKI_FP64:
            with pytest.raises(shaw.ShawError) as e:
                bt.set_tiling(64)
            assert e.value.code == shaw.ERR_UNSUPPORTED
        bt.close()
    for i in range(len(insts)):
        (x64, s64, g64), (xoz, soz, goz) = res[shaw.FP64][i], res[shaw.OZAKI_FP64][i]
        errs = [relerr(xoz[0], x64[0]), relerr(xoz[1], x64[1]), relerr(soz[0], s64[0]), relerr(soz[1], s64[1]),
                relerr(goz, g64)]
        assert max(errs) <= 1e-12, (i, errs)
    for i, d in enumerate(insts):
        r = shaw.Rom(d["rom_jvp"], d["rom_jsp"], d["b"], rank=2, precision=shaw.OZAKI_FP64)
        r.set_signals(d["kind"], d["period"], d["delay"])
        r.run(dt, n)
        a = r.get_state()
        r.close()
        assert np.array_equal(a[0], res[shaw.OZAKI_FP64][i][0][0]) and np.array_equal(a[1], res[shaw.OZAKI_FP64][i][0][1])


@pytest.mark.parametrize("width", [16, 32])
def test_batch_ozaki_fp64_paired_bitwise(shaw, width):
    """Tiles of 16 columns (two accumulator sets) and 32 columns (one set staged in TMEM),
    whole or split across CTA pairs, advanced in pieces: the same numbers bit for bit."""
    insts = _instances(16, shapes=[(384, 256, 40), (512, 512, 20)])
    out = {}
    for paired in (False, True):
        bt = shaw.RomBatch(insts, precision=shaw.OZAKI_FP64)
        bt.set_tiling(width, paired=paired)
        bt.advance(0.5, 17)
        bt.advance(0.5, 43)
        bt.synchronize()
        out[paired] = [bt.get_state(i) for i in range(len(insts))]
        bt.close()
    for i in range(len(insts)):
        assert np.array_equal(out[False][i][0], out[True][i][0]) and np.array_equal(out[False][i][1], out[True][i][1])
