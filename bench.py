"""Benchmark of the FOM rank-2 FP64 velocity-stress leapfrog (DOF-updates/s).

Workload (one GPU): staggered axisymmetric grid of 1000 theta x 2000 r vertices,
theta in [0, 180] deg, r in [3480, 6371] km; radially layered material with
density 3.3->5.6 g/cm^3 and shear speed 4.4->7.3 km/s increasing with depth;
M = 256 forcings (Gaussian-derivative signals, depths U[200,700] km, periods
U[30,90] s, delay 180 s, seeded); dt from CFL 0.25; receivers every 1 degree at
the surface (seismogram every step).  A "step" is one leapfrog step (velocity
half-step + stress half-step) of all 256 columns: 5,997,000 x 256 DOF-updates.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the reference's CRS leapfrog
(oracle/, Kokkos-Kernels CRS row semantics, OpenMP over all host threads) on a
bounded sample of the same workload.  Under torchrun every rank runs its own
256 forcing columns (the columns are independent: weak scaling, no collective
in the time loop); rank 0 prints one JSON line.
"""
import argparse
import json
import os
import platform
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NTH, NR, M = 1000, 2000, 256
MATERIAL = [3300.0, 2300.0 / 2891000.0, 0.0, 4400.0, 2900.0 / 2891000.0, 0.0]
SEED = 20261203
METRIC = "FOM DOF-updates/s (rank-2 FP64 leapfrog)"
WORKLOAD = "FOM rank-2 FP64, 1000 theta x 2000 r grid, M=256 forcings"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    # smaller cases for profiling captures (the default is the benchmark workload)
    p.add_argument("--forcings", type=int, default=M)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extra", action="store_true", help="skip the other configurations' lines")
    p.add_argument("--profile-rom", default=None,
                   choices=["ozaki", "ozaki-fp64", "tf32x3", "fp64", "rank1-fp64", "rank1-mixed"],
                   help="only run the rank-2 ROM (k=512, M=4096) or the rank-1 ROM (k=256, 181 receivers) "
                        "for --steps steps, for profiler captures")
    p.add_argument("--profile-fom", default=None, choices=["fp64", "fp32", "rank1", "rank1-wide"],
                   help="only run the FOM on the 1000x2000 grid with --forcings columns for --steps steps")
    p.add_argument("--schedule", default="auto", choices=["auto", "two-pass", "sweep", "persistent"],
                   help="FOM schedule of --profile-fom")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def workload_inputs(np, mesh, rank=0, world=1):
    """This rank's M forcing columns of the job's world * M seeded draws."""
    from shaw_gb300.sharding import shard_range
    rng = np.random.default_rng(SEED)
    depths = rng.uniform(200.0, 700.0, M * world)
    periods = rng.uniform(30.0, 90.0, M * world)
    lo, hi = shard_range(M * world, rank, world)
    depths, periods = depths[lo:hi], periods[lo:hi]
    gids = [mesh.map_source(float(d), 0.0) for d in depths]
    rcv = [mesh.map_receiver(float(a)) for a in range(0, 181)]
    dt = 0.25 * min(mesh.info[5], mesh.info[4] * mesh.info[2]) / (2.0 ** 0.5 * 7300.0)
    return gids, periods, rcv, dt


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


# DRAM bytes (read + write) of one fom_stress_kernel launch per forcing column, from the
# ncu capture summarised in profiles/fom_kernels_rank2_1000x2000.md (M = 16, scaled by M).
TRAFFIC_STRESS_PER_FORCING = (831.617024e6 + 461.196032e6) / 16
# DRAM bytes (read + write) of one fom_sweep_kernel launch per forcing column (FP64 state), from
# the ncu capture summarised in profiles/ (M = 32, scaled by M); None until that capture exists.
TRAFFIC_SWEEP_PER_FORCING = None


def dgemm_tflops(torch):
    """FP64 peak proxy: cuBLAS DGEMM 8192^3, best of 3 (CUDA events)."""
    a = torch.randn(8192, 8192, dtype=torch.float64, device="cuda")
    b = torch.randn(8192, 8192, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    best = 1e30
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    torch.cuda.empty_cache()
    return 2.0 * 8192 ** 3 / (best / 1e3) / 1e12


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def host_cpu():
    """CPU model and core counts of this host, recorded beside every CPU timing."""
    model = None
    try:
        out = subprocess.run(["lscpu"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
                             timeout=20).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                model = ln.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if not model:
        try:
            with open("/proc/cpuinfo") as fh:
                for ln in fh:
                    if ln.lower().startswith(("model name", "cpu part")):
                        model = ln.split(":", 1)[1].strip()
                        break
        except OSError:
            pass
    return {"model": model or platform.processor() or platform.machine(), "nproc": os.cpu_count(),
            "machine": platform.machine()}


def omp_binding():
    """Thread placement of the reference's scaling runs (python_scripts_revise/utils.py:72-74);
    set before any OpenMP runtime starts in this process."""
    os.environ.setdefault("OMP_PROC_BIND", "spread")
    os.environ.setdefault("OMP_PLACES", "threads")
    return {k: os.environ[k] for k in ("OMP_PROC_BIND", "OMP_PLACES")}


def oracle_workload(np, world=1):
    """The benchmark workload built with the oracle alone (its own mesher, material,
    mappers): rank 0's M forcing columns of the job's world * M seeded draws."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    oracle_lib.build()
    with tempfile.TemporaryDirectory() as d:
        oracle_lib.write_full_mesh(NTH, NR, d)
        om = oracle_lib.OracleMesh(d)
    om.set_material("unilayer", [(MATERIAL[0:3], MATERIAL[3:6])])
    rng = np.random.default_rng(SEED)
    depths = rng.uniform(200.0, 700.0, M * world)[:M]
    periods = rng.uniform(30.0, 90.0, M * world)[:M]
    gids = [om.map_source(float(x), 0.0) for x in depths]
    rcv = [om.map_receiver(float(a)) for a in range(0, 181)]
    dt = 0.25 * min(om.info[5], om.info[4] * om.info[2]) / (2.0 ** 0.5 * 7300.0)
    return oracle_lib, om, gids, periods, rcv, dt


def oracle_steps(np, om, gids, periods, rcv, dt, warmup, steps=None, budget_s=None):
    """Time full leapfrog steps of all M columns on the host cores (the oracle's CRS
    SpMM leapfrog with the forcing and the 181-receiver gather of every step): `warmup`
    untimed steps, then `steps` timed ones (or as many as fit in budget_s)."""
    xv = np.zeros((om.nvp, M))
    xs = np.zeros((om.nsp, M))
    kinds = [2] * M
    om.fom_advance_forced(xv, xs, 0, warmup, dt, gids, kinds, periods, 180.0, rcv)
    done = warmup
    if steps is None:  # size the sample from one timed step
        t0 = time.perf_counter()
        om.fom_advance_forced(xv, xs, done, 1, dt, gids, kinds, periods, 180.0, rcv)
        done += 1
        steps = int(max(2, min(200, budget_s / max(time.perf_counter() - t0, 1e-3))))
    t0 = time.perf_counter()
    om.fom_advance_forced(xv, xs, done, steps, dt, gids, kinds, periods, 180.0, rcv)
    el = time.perf_counter() - t0
    return steps, el


def cpu_baseline(np, budget_s=12.0):
    """The oracle's leapfrog on the same workload (all 256 columns), all host threads, a
    bounded number of steps."""
    orc, om, gids, periods, rcv, dt = oracle_workload(np)
    threads = orc.lib().orc_num_threads(0)
    steps, el = oracle_steps(np, om, gids, periods, rcv, dt, 2, budget_s=budget_s)
    units = (om.nvp + om.nsp) * M * steps
    return dict(value=units / el, unit="DOF-updates/s", cores=threads, kind="port",
                sample="%d leapfrog steps of all %d forcing columns on the 1000x2000 grid, forcing and "
                       "181-receiver gather every step (%.1f s)" % (steps, M, el),
                cpu=host_cpu(), omp=omp_binding())


def _timed(torch, stream_ptr, fn):
    s = torch.cuda.ExternalStream(stream_ptr)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    fn()
    e1.record(s)
    e1.synchronize()
    return e0.elapsed_time(e1) / 1e3


def _relerr(np, a, b):
    """max |a - b| / max |b|; the absolute difference where b is all zero (e.g. surface
    receivers that the wave has not reached yet)."""
    scale = float(np.max(np.abs(b)))
    diff = float(np.max(np.abs(a - b)))
    return diff / scale if scale > 0 else diff


def stable_rom(np, k, seed, smin, smax):
    """Seeded reduced pair with As = -Av^T and singular values in [smin, smax]: a
    bounded (symplectic) leapfrog standing in for a POD-projected SHAW ROM."""
    rng = np.random.default_rng(seed)
    q1 = np.linalg.qr(rng.standard_normal((k, k)))[0]
    q2 = np.linalg.qr(rng.standard_normal((k, k)))[0]
    av = q1 @ np.diag(np.linspace(smin, smax, k)) @ q2.T
    return av, -av.T.copy()


def oracle_mesh(nth, nr):
    """The oracle's own copy of a generated grid (mesher, material and operators of the
    oracle), for the error legs."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    oracle_lib.build()
    with tempfile.TemporaryDirectory() as d:
        oracle_lib.write_full_mesh(nth, nr, d)
        om = oracle_lib.OracleMesh(d)
    om.set_material("unilayer", [(MATERIAL[0:3], MATERIAL[3:6])])
    return oracle_lib, om


def fom_rank1_config1(np, torch, shaw, nth, nr, n=2000):
    """Config 1: FOM rank 1, one gaussDer source at 640 km on the axis (period 60 s, delay
    180 s), 181 surface receivers, 2000 steps; then the same run against the oracle."""
    mesh = shaw.Mesh.generate(nth, nr)
    mesh.set_material("unilayer", MATERIAL)
    dt = 0.25 * min(mesh.info[5], mesh.info[4] * mesh.info[2]) / (2.0 ** 0.5 * 7300.0)
    src = mesh.map_source(640.0, 0.0)
    rcv = [mesh.map_receiver(float(a)) for a in range(181)]
    f = shaw.Fom(mesh, 1, 1)
    f.set_sources([src], "gaussDer", 60.0, 180.0)
    f.set_receivers(rcv, 1, n)
    f.run(dt, n)  # warm-up
    f.reset()
    l0 = f.kernel_launches
    t = _timed(torch, f.stream, lambda: f.advance(dt, n))
    f.synchronize()
    launches = f.kernel_launches - l0
    seis = f.seismogram()
    vp, sp = f.get_state()
    # the same run on the two half-step kernels (CUDA-graph chunks), for comparison
    f.set_schedule(shaw.SCHEDULE_TWO_PASS)
    f.run(dt, n)
    f.reset()
    t2 = _timed(torch, f.stream, lambda: f.advance(dt, n))
    f.synchronize()
    f.close()
    _, om = oracle_mesh(nth, nr)
    ref = om.fom_run(1, n, dt, [src], [2], [60.0], [180.0], rcv, 1, 0, 0)
    return {"metric": "FOM DOF-updates/s", "value": (mesh.nvp + mesh.nsp) * n / t, "steps": n,
            "us_per_step": t / n * 1e6, "launches": launches,
            "schedule": "persistent (one cooperative launch of row or column bands; the default for rank-1 FP64)",
            "two_pass_us_per_step": t2 / n * 1e6,
            "max_rel_err_vs_oracle": {"seismogram": _relerr(np, seis, ref["seis"]),
                                      "state_vp": _relerr(np, vp, ref["final_vp"]),
                                      "state_sp": _relerr(np, sp, ref["final_sp"]),
                                      "compared": "the timed 2000-step run, 181 receivers every step"}}


def extra_workloads(np, torch, shaw):
    """The other configurations, each timed with CUDA events on its handle's stream, each
    FP64 result with its error against the oracle, each mixed result with its error
    against an FP64-grade form over the configured number of steps."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    oracle_lib.build()
    out = {}
    # config 1 as worded (101 theta x 201 r) and on the reference fixture's orientation
    out["fom_rank1_101x201"] = fom_rank1_config1(np, torch, shaw, 101, 201)
    out["fom_rank1_fixture_201x101"] = fom_rank1_config1(np, torch, shaw, 201, 101)
    mesh = shaw.Mesh.generate(101, 201)
    mesh.set_material("unilayer", MATERIAL)
    dt = 0.25 * min(mesh.info[5], mesh.info[4] * mesh.info[2]) / (2.0 ** 0.5 * 7300.0)
    basis = pod_basis(np, shaw, mesh, dt)
    rcv = [mesh.map_receiver(float(a)) for a in range(181)]
    rho_inv = mesh.arrays()["rho_inv_vp"]

    def forcing_vectors(k, gids):
        g = np.asarray(gids)
        return np.asfortranarray(basis["phi_v"][g, :k].T * rho_inv[g][None, :])

    # config 3: ROM rank-1, kv = ks = 256 modes, one new forcing (depth U[200,700] km,
    # period U[30,90] s), 20000 steps, FP64 vs mixed (FP32 hi + lo, compensated)
    k, n = 256, 20000
    rng = np.random.default_rng(SEED + 3)
    depth, period = float(rng.uniform(200.0, 700.0)), float(rng.uniform(30.0, 90.0))
    av, as_ = basis["av"][:k, :k], basis["as"][:k, :k]
    b = forcing_vectors(k, [mesh.map_source(depth, 0.0)])[:, 0]
    rows = np.ascontiguousarray(basis["phi_v"][rcv, :k])
    res = {}
    # FP64 on its default launch (row bands over the SMs), FP64 on the 16-CTA cluster, mixed
    for key, prec, sched in (("fp64", shaw.FP64, shaw.ROM_SCHEDULE_AUTO),
                             ("fp64_cluster", shaw.FP64, shaw.ROM_SCHEDULE_CLUSTER),
                             ("mixed", shaw.MIXED_FP32, shaw.ROM_SCHEDULE_AUTO)):
        r = shaw.Rom(av, as_, b, rank=1, precision=prec)
        r.set_schedule(sched)
        r.set_signals("gaussDer", period, 180.0)
        r.set_receivers(rows, 1, n)
        r.reset()
        t = _timed(torch, r.stream, lambda: r.advance(dt, n))
        r.synchronize()
        res[key] = (t, r.seismogram().copy(), r.get_state())
        r.close()
    assert np.array_equal(res["fp64"][1], res["fp64_cluster"][1])  # the same row arithmetic
    res[shaw.FP64], res[shaw.MIXED_FP32] = res["fp64"], res["mixed"]
    ref = oracle_lib.rom_run(av, as_, b.reshape(k, 1), n, dt, [2], [period], [180.0], freq_vp=1)
    ref_seis = np.einsum("rk,kt->rt", rows, ref["snaps_vp"][:, :, 0])[:, :, None]
    out["rom_rank1_k256"] = {"metric": "ROM forcing-steps/s", "steps": n,
                             "fp64": n / res[shaw.FP64][0], "mixed_fp32": n / res[shaw.MIXED_FP32][0],
                             "fp64_launch": "row bands over the SMs, new rows gathered through L2 (the default)",
                             "fp64_cluster": n / res["fp64_cluster"][0],
                             "speedup": res[shaw.FP64][0] / res[shaw.MIXED_FP32][0],
                             "seismogram_rel_err": _relerr(np, res[shaw.MIXED_FP32][1], res[shaw.FP64][1]),
                             "seismogram_max_abs": float(np.max(np.abs(res[shaw.FP64][1]))),
                             "fp64_max_rel_err_vs_oracle": {
                                 "seismogram": _relerr(np, res[shaw.FP64][1], ref_seis),
                                 "state_vp": _relerr(np, res[shaw.FP64][2][0][:, 0], ref["final_vp"][:, 0]),
                                 "state_sp": _relerr(np, res[shaw.FP64][2][1][:, 0], ref["final_sp"][:, 0]),
                                 "compared": "the timed 20000-step run (oracle: the reference's GEMV loop)"},
                             "forcing": {"depth_km": depth, "period_s": period, "delay_s": 180.0},
                             "cpu_oracle": rom_cpu_oracle(np, av, as_, b, 2000, dt, period),
                             "basis": basis["info"]}
    out["rom_rank2_k512_M4096"] = rom_rank2_config4(np, torch, shaw, oracle_lib, mesh, dt, basis, forcing_vectors,
                                                    rcv)
    out["rom_batch_64_uneven"] = batched_workload(np, torch, shaw, mesh, dt, basis, forcing_vectors, rcv)
    out["fom_rank2_2000x4000_M64"] = fom_fp64_vs_fp32(np, torch, shaw)
    return out


def rom_rank2_config4(np, torch, shaw, oracle_lib, mesh, dt, basis, forcing_vectors, rcv, k=512, M=4096, n=100,
                      n_long=20000, n_cross=2000, n_oracle_cols=256):
    """Config 4: k = 512, M = 4096 forcings.  Throughput of each form over n steps; FP64
    forms against the oracle (first n_oracle_cols columns, n steps); the mixed form over the
    configured n_long steps against the FP64-grade Ozaki form, which is itself checked
    against the DGEMM path over n_cross steps (seismograms every 100 steps)."""
    rng = np.random.default_rng(SEED + 4)
    depths, periods = rng.uniform(200.0, 700.0, M), rng.uniform(30.0, 90.0, M)
    av, as_ = basis["av"][:k, :k], basis["as"][:k, :k]
    b = forcing_vectors(k, [mesh.map_source(float(d), 0.0) for d in depths])
    rows = np.ascontiguousarray(basis["phi_v"][rcv, :k])
    res = {}
    for prec in (shaw.FP64, shaw.MIXED_OZAKI_BF16, shaw.OZAKI_FP64, shaw.MIXED_TF32X3):
        r = shaw.Rom(av, as_, b, rank=2, precision=prec)
        r.set_signals("gaussDer", periods, 180.0)
        r.reset()
        r.advance(dt, 2 if prec == shaw.FP64 else n)  # warm-up
        r.synchronize()
        r.reset()
        t = _timed(torch, r.stream, lambda: r.advance(dt, n))
        r.synchronize()
        res[prec] = (t, r.get_state())
        r.close()
    ref = oracle_lib.rom_run(av, as_, b[:, :n_oracle_cols], n, dt, [2] * n_oracle_cols, periods[:n_oracle_cols],
                             [180.0] * n_oracle_cols)

    def vs_oracle(state):
        return {"state_vp": _relerr(np, state[0][:, :n_oracle_cols], ref["final_vp"]),
                "state_sp": _relerr(np, state[1][:, :n_oracle_cols], ref["final_sp"])}

    def long_seis(prec, nsteps, freq=100):
        r = shaw.Rom(av, as_, b, rank=2, precision=prec)
        r.set_signals("gaussDer", periods, 180.0)
        r.set_receivers(rows, freq, nsteps)
        r.run(dt, nsteps)
        s = r.seismogram()
        r.close()
        return s

    s_oz_long, s_f64_long = long_seis(shaw.MIXED_OZAKI_BF16, n_long), long_seis(shaw.OZAKI_FP64, n_long)
    s_f64_cross, s_dgemm_cross = long_seis(shaw.OZAKI_FP64, n_cross), long_seis(shaw.FP64, n_cross)
    t64 = res[shaw.FP64][0]
    return {
        "metric": "ROM forcing-steps/s", "steps": n, "fp64": M * n / t64,
        "ozaki_bf16": M * n / res[shaw.MIXED_OZAKI_BF16][0], "ozaki_fp64": M * n / res[shaw.OZAKI_FP64][0],
        "tf32x3_experimental": M * n / res[shaw.MIXED_TF32X3][0],
        "speedup_ozaki": t64 / res[shaw.MIXED_OZAKI_BF16][0], "speedup_ozaki_fp64": t64 / res[shaw.OZAKI_FP64][0],
        "algorithmic_tflops_ozaki": 4.0 * k * k * M * n / res[shaw.MIXED_OZAKI_BF16][0] / 1e12,
        "algorithmic_tflops_ozaki_fp64": 4.0 * k * k * M * n / res[shaw.OZAKI_FP64][0] / 1e12,
        "fp64_max_rel_err_vs_oracle": dict(vs_oracle(res[shaw.FP64][1]), compared=
                                           "final states after the timed %d steps, first %d of %d columns"
                                           % (n, n_oracle_cols, M)),
        "ozaki_fp64_max_rel_err_vs_oracle": dict(vs_oracle(res[shaw.OZAKI_FP64][1]), compared=
                                                 "final states after the timed %d steps, first %d of %d columns"
                                                 % (n, n_oracle_cols, M)),
        "ozaki_fp64_seismogram_rel_err_vs_dgemm": {"value": _relerr(np, s_f64_cross, s_dgemm_cross),
                                                   "steps": n_cross, "samples_every": 100},
        "ozaki_bf16_seismogram_rel_err_vs_ozaki_fp64": {"value": _relerr(np, s_oz_long, s_f64_long),
                                                        "steps": n_long, "samples_every": 100},
        "tf32x3_state_rel_err_vs_fp64": _relerr(np, res[shaw.MIXED_TF32X3][1][0], res[shaw.FP64][1][0]),
        "cpu_oracle": rom_cpu_oracle(np, av, as_, b[:, :64], 60, dt, periods[:64]),
        "basis": "leading 512 modes of the POD basis of config 3"}


def rom_cpu_oracle(np, av, as_, b, nsteps, dt, periods):
    """The oracle's ROM leapfrog (the reference's GEMV / GEMM loop restated, FP64, all host
    threads) on a bounded sample: forcing-steps/s on the host cores."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    oracle_lib.build()
    b = np.asfortranarray(np.asarray(b, np.float64).reshape(av.shape[0], -1, order="F"))
    M = b.shape[1]
    periods = np.broadcast_to(np.asarray(periods, np.float64), (M,))
    t0 = time.perf_counter()
    oracle_lib.rom_run(av, as_, b, nsteps, dt, [2] * M, periods, [180.0] * M)
    el = time.perf_counter() - t0
    return {"value": M * nsteps / el, "unit": "forcing-steps/s", "cores": oracle_lib.lib().orc_num_threads(0),
            "kind": "port", "sample": "%d steps of %d forcing column(s) (%.2f s)" % (nsteps, M, el)}


def fom_fp64_vs_fp32(np, torch, shaw, nth=2000, nr=4000, M=64, n_time=20, n_err=1000):
    """Config 5's FOM job: 2000 theta x 4000 r grid, M = 64 forcings (depth U[200,700] km,
    period U[30,90] s, seeded), FP64 vs FP32 state.  Error probe: velocity traces over
    n_err steps at the 64 source points and 10 grid rows (7 km) above each (the surface
    receivers see nothing before t = delay + travel time, ~13000 steps at this dt)."""
    mesh = shaw.Mesh.generate(nth, nr)
    mesh.set_material("unilayer", MATERIAL)
    dt = 0.25 * min(mesh.info[5], mesh.info[4] * mesh.info[2]) / (2.0 ** 0.5 * 7300.0)
    rng = np.random.default_rng(SEED + 5)
    gids = [mesh.map_source(float(d), 0.0) for d in rng.uniform(200.0, 700.0, M)]
    periods = rng.uniform(30.0, 90.0, M)
    probe = list(gids) + [g + 10 * nth for g in gids]
    dofs = (mesh.nvp + mesh.nsp) * M
    res = {}
    for prec in (shaw.FP64, shaw.MIXED_FP32):
        f = shaw.Fom(mesh, 2, M, precision=prec)
        f.set_sources(gids, "gaussDer", periods, 180.0)
        f.set_receivers(probe, 1, n_err)
        f.reset()
        f.advance(dt, 3)  # warm-up
        f.synchronize()
        f.reset()
        t = _timed(torch, f.stream, lambda: f.advance(dt, n_time))
        f.synchronize()
        timed_state = f.get_state() if prec == shaw.FP64 else None
        f.run(dt, n_err)
        res[prec] = (t, f.seismogram(), timed_state)
        f.close()
    _, om = oracle_mesh(nth, nr)
    ref = om.fom_run(2, n_time, dt, gids, [2] * M, periods, [180.0] * M, [], 0, 0, 0)
    vp, sp = res[shaw.FP64][2]
    err64 = {"state_vp": _relerr(np, vp, ref["final_vp"]), "state_sp": _relerr(np, sp, ref["final_sp"]),
             "compared": "final state of the timed %d-step FP64 run from rest, all %d columns" % (n_time, M)}
    del ref, vp, sp, om
    v64, v32 = dofs * n_time / res[shaw.FP64][0], dofs * n_time / res[shaw.MIXED_FP32][0]
    return {"metric": "FOM DOF-updates/s", "grid": [nth, nr], "forcings": M, "fp64": v64, "mixed_fp32": v32,
            "fp64_max_rel_err_vs_oracle": err64,
            "speedup": v32 / v64, "timed_steps": n_time,
            "trace_rel_err_fp32": _relerr(np, res[shaw.MIXED_FP32][1], res[shaw.FP64][1]),
            "error_probe": "velocity at the 64 source points and 7 km above them, every step",
            "error_after_steps": n_err,
            "mixed_fp32_schedule": "single sweep (one kernel per step)",
            "mixed_fp32_hbm_frac": v32 * 8 / 1e9 / measured_peaks()[0],
            "fp64_hbm_frac": v64 * 16 / 1e9 / measured_peaks()[0],
            "mixed_fp32_bytes_per_dof_update": 8, "fp64_bytes_per_dof_update": 16}


def pod_basis(np, shaw, mesh, dt, kmax=1024, n_train=8):
    """FOM -> POD -> Galerkin projection, all on the GPU, on the 101 x 201 grid of config 1.

    Training: the config-1 source (640 km on the axis, period 60 s) plus 7 seeded sources
    (depth U[200,700] km, angle U[0,180] deg, period U[30,90] s), 2000 steps, snapshots
    every 5 steps: 400 snapshots per forcing, 3200 per dof.  (The 400 snapshots of the
    config-1 source alone have numerical rank 175 < 256; their 256-mode Galerkin system
    has an eigenvalue of dt^2 As Av with positive real part and the leapfrog diverges.)"""
    rng = np.random.default_rng(5)
    specs = [(640.0, 0.0, 60.0)] + [(float(rng.uniform(200, 700)), float(rng.uniform(0, 180)),
                                     float(rng.uniform(30, 90))) for _ in range(n_train - 1)]
    t0 = time.perf_counter()
    f = shaw.Fom(mesh, 2, n_train)
    f.set_sources([mesh.map_source(d, a) for d, a, _ in specs], "gaussDer", [p for _, _, p in specs], 180.0)
    f.set_snapshots(5, 5, 2000)
    f.run(dt, 2000)
    svp, ssp = f.snapshots()
    t_fom = time.perf_counter() - t0
    phi_v, sv_v = shaw.pod(svp.reshape(svp.shape[0], -1, order="F"), method=2)
    phi_s, sv_s = shaw.pod(ssp.reshape(ssp.shape[0], -1, order="F"), method=2)
    t_pod = time.perf_counter() - t0 - t_fom
    phi_v, phi_s = np.asfortranarray(phi_v[:, :kmax]), np.asfortranarray(phi_s[:, :kmax])
    av, as_ = shaw.rom_project(f, phi_v, phi_s)
    t_all = time.perf_counter() - t0
    f.close()
    info = ("POD of 3200 FOM snapshots per dof (8 training forcings x 400, config-1 grid): FOM %.2f s, "
            "thin SVDs %.2f s, projection to %d modes %.2f s (GPU); sigma_k/sigma_1 (vp) k=256 %.1e, "
            "512 %.1e, 1024 %.1e" % (t_fom, t_pod, kmax, t_all - t_fom - t_pod, sv_v[255] / sv_v[0],
                                     sv_v[511] / sv_v[0], sv_v[kmax - 1] / sv_v[0]))
    return {"phi_v": phi_v, "phi_s": phi_s, "av": av, "as": as_, "info": info}


def batched_workload(np, torch, shaw, mesh, dt, basis, forcing_vectors, rcv, n_inst=64, seed=20261205,
                     n_long=20000, n_cross=100, seis_freq=500):
    """64 reduced systems, k ~ U{64, 128, ..., 1024}, M ~ U[16, 2048] (seeded), each the
    leading k modes of the POD basis with its own M axis sources (depth U[200,700] km,
    period U[30,90] s), advanced together: FP64 (cuBLAS DGEMM per instance) vs the Ozaki
    tensor-core batch (one persistent launch, autotuned tile widths and schedule).
    Errors: the mixed form against the FP64-grade form over the configured n_long steps,
    and the FP64-grade form against the DGEMM batch over n_cross steps (seismograms of 37
    receivers, every 5 degrees, every seis_freq / 100 steps)."""
    rng = np.random.default_rng(seed)
    ks = rng.integers(1, 17, n_inst) * 64
    Ms = rng.integers(16, 2049, n_inst)
    insts = []
    for k, M in zip(ks, Ms):
        k = int(k)
        gids = [mesh.map_source(float(d), 0.0) for d in rng.uniform(200.0, 700.0, M)]
        insts.append(dict(rom_jvp=basis["av"][:k, :k], rom_jsp=basis["as"][:k, :k], b=forcing_vectors(k, gids),
                          kind="gaussDer", period=rng.uniform(30.0, 90.0, M), delay=180.0))
    flops = float(sum(4.0 * k * k * M for k, M in zip(ks, Ms)))
    cols = int(Ms.sum())
    n64, n_oz = 6, 120
    rows = {i: np.ascontiguousarray(basis["phi_v"][rcv[::5], :int(ks[i])]) for i in range(n_inst)}
    res = {}
    for prec in (shaw.FP64, shaw.MIXED_OZAKI_BF16, shaw.OZAKI_FP64):
        bt = shaw.RomBatch(insts, precision=prec)
        report = bt.tune(dt, 4) if prec != shaw.FP64 else ""
        bt.reset()
        bt.advance(dt, 2)  # warm-up
        bt.synchronize()
        bt.reset()
        n = n64 if prec == shaw.FP64 else n_oz
        l0 = bt.kernel_launches
        t = _timed(torch, bt.stream, lambda: bt.advance(dt, n))
        bt.synchronize()
        launches = bt.kernel_launches - l0
        res[prec] = dict(t=t, n=n, describe=bt.describe(), report=report, launches=launches)
        bt.close()

    def seismograms(prec, nsteps, freq):
        bt = shaw.RomBatch(insts, precision=prec)
        for i in range(n_inst):
            bt.set_receivers(i, rows[i], freq, nsteps)
        bt.run(dt, nsteps)
        out = [bt.seismogram(i) for i in range(n_inst)]
        bt.close()
        return out

    t0 = time.perf_counter()
    s_oz, s_f64 = seismograms(shaw.MIXED_OZAKI_BF16, n_long, seis_freq), seismograms(shaw.OZAKI_FP64, n_long, seis_freq)
    err_long = max(_relerr(np, a, b) for a, b in zip(s_oz, s_f64))
    del s_oz, s_f64
    c_f64, c_dgemm = seismograms(shaw.OZAKI_FP64, n_cross, 1), seismograms(shaw.FP64, n_cross, 1)
    err_cross = max(_relerr(np, a, b) for a, b in zip(c_f64, c_dgemm))
    t_err = time.perf_counter() - t0
    r64, roz, rof = res[shaw.FP64], res[shaw.MIXED_OZAKI_BF16], res[shaw.OZAKI_FP64]
    v64, voz, vof = cols * r64["n"] / r64["t"], cols * roz["n"] / roz["t"], cols * rof["n"] / rof["t"]
    return {"metric": "ROM forcing-steps/s", "instances": n_inst, "total_forcings": cols,
            "k_range": [int(ks.min()), int(ks.max())], "M_range": [int(Ms.min()), int(Ms.max())],
            "fp64": v64, "ozaki_bf16": voz, "speedup_ozaki": voz / v64,
            "ozaki_fp64": vof, "speedup_ozaki_fp64": vof / v64,
            "algorithmic_tflops_ozaki_fp64": flops * rof["n"] / rof["t"] / 1e12, "tiling_ozaki_fp64": rof["describe"],
            "fp64_steps": r64["n"], "ozaki_steps": roz["n"], "ozaki_launches": roz["launches"],
            "algorithmic_tflops_fp64": flops * r64["n"] / r64["t"] / 1e12,
            "algorithmic_tflops_ozaki": flops * roz["n"] / roz["t"] / 1e12,
            "ozaki_bf16_seismogram_rel_err_vs_ozaki_fp64": {"value": err_long, "steps": n_long,
                                                            "samples_every": seis_freq, "receivers": len(rcv[::5]),
                                                            "instances": n_inst},
            "ozaki_fp64_seismogram_rel_err_vs_dgemm": {"value": err_cross, "steps": n_cross, "samples_every": 1,
                                                       "receivers": len(rcv[::5]), "instances": n_inst},
            "error_legs_seconds": t_err,
            "tiling": roz["describe"], "autotuner": roz["report"].strip().split("\n")}


def run_reference(args):
    """The reference arm: the oracle's restatement of the reference's CRS leapfrog (the
    reference's Kokkos build cannot be made here) on the host cores, on the same workload
    as our arm (mesh, material, sources, receivers built by the oracle; the product library
    is never loaded).  Rank 0 alone runs it."""
    import numpy as np
    rank, world, _ = dist_env()
    if rank != 0:
        return
    omp = omp_binding()
    orc, om, gids, periods, rcv, dt = oracle_workload(np, world)
    threads = orc.lib().orc_num_threads(0)
    steps, el = oracle_steps(np, om, gids, periods, rcv, dt, args.warmup, steps=args.steps)
    dofs = (om.nvp + om.nsp) * M
    value = dofs * steps / el
    sample = ("%d full leapfrog steps of all %d forcing columns on the 1000x2000 grid after %d warm-up steps, "
              "forcing and 181-receiver gather every step" % (steps, M, args.warmup))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "DOF-updates/s", "n_gpus": world,
            "steps": steps, "warmup": args.warmup, "ms_per_step": el / steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "nth": NTH, "nr": NR, "forcings": M, "dt": dt,
                       "receivers": len(rcv), "seismogram_freq": 1,
                       "l2": "inputs larger than L2 (state 12 GB)"},
            "same_config": True,
            "cpu_baseline": {"value": value, "unit": "DOF-updates/s", "cores": threads, "kind": "port",
                             "sample": sample, "cpu": host_cpu(), "omp": omp,
                             "build": "g++ -O3 -fopenmp -ffp-contract=off (portable flags: the same objects "
                                      "build and give the same results on x86_64 and aarch64)"},
            "e2e": {"value": value, "unit": "DOF-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "host": platform.machine(), "cpu_threads": threads}
    print(json.dumps(line), flush=True)


def run_ours(args):
    rank, world, local = dist_env()
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    import numpy as np
    import torch
    import shaw_gb300 as shaw
    shaw.build()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(0)

    mesh = shaw.Mesh.generate(NTH, NR)
    mesh.set_material("unilayer", MATERIAL)
    gids, periods, rcv, dt = workload_inputs(np, mesh, rank, world)
    dofs = (mesh.nvp + mesh.nsp) * M
    total_steps = args.warmup + args.steps

    def barrier():
        if dist:
            dist.barrier()

    # ---- device-resident throughput -------------------------------------------------
    f = shaw.Fom(mesh, 2, M)
    f.set_sources(gids, "gaussDer", periods, 180.0)
    f.set_receivers(rcv, 1, total_steps)
    f.reset()
    stream = torch.cuda.ExternalStream(f.stream)
    f.advance(dt, args.warmup)
    f.synchronize()
    barrier()
    torch.cuda.synchronize()
    launches0 = f.kernel_launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        f.advance(dt, args.steps)
        e1.record(stream)
        e1.synchronize()
    f.synchronize()
    torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    launches = f.kernel_launches - launches0
    # the timed run's result, for the comparison with the oracle after every GPU leg
    timed_seis = f.seismogram()
    timed_vp, timed_sp = f.get_state()
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * dofs * args.steps / (ms / 1e3)

    # ---- single launches of each schedule (CUDA events on the launching stream) ---------
    def timed_ms(fn, reps=6):
        ts = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b))
        ts = sorted(ts)[1:-1]
        return sum(ts) / len(ts) / 1e3

    # the timed run used the default schedule: for FP64 handles the two half-step kernels
    # (on GB300 both schedules are bound by the FP64 pipe; the sweep is timed beside them)
    sweep = False
    f.set_receivers([], 0, 0)
    sched = {}
    if M % 32 == 0:
        f.set_schedule(shaw.SCHEDULE_SWEEP)
        sched["sweep"] = timed_ms(lambda: f.advance(dt, 1))  # one fom_sweep_kernel launch
    f.set_schedule(shaw.SCHEDULE_TWO_PASS)
    t_v = timed_ms(lambda: f.update_velocity(dt, total_steps))
    t_s = timed_ms(lambda: f.update_stress(dt))
    sched["two_pass_velocity"], sched["two_pass_stress"] = t_v, t_s
    f.close()

    # ---- end to end through the C ABI from host buffers -------------------------------
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    g = shaw.Fom(mesh, 2, M)                      # operators H2D from the host mesh arrays
    g.set_sources(gids, "gaussDer", periods, 180.0)
    g.set_receivers(rcv, 1, args.steps)
    g.run(dt, args.steps)
    seis = g.seismogram()                         # D2H of the result
    e2e_s = time.perf_counter() - t0
    g.close()
    barrier()
    if dist:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = world * dofs * args.steps / e2e_s
    h2d = (mesh.nvp * (5 * 8 + 2 * 8 + 8 + 4 * 8 + 8) + mesh.nsp * (3 * 8 + 4 + 2 * 8 + 8 + 8)  # desc arrays
           + M * (8 + 4 + 8 + 8) + len(rcv) * 8)
    d2h = seis.nbytes
    gathered = M
    if dist:  # host gather of every rank's seismogram columns onto rank 0 (after the timed regions)
        from shaw_gb300.sharding import gather_columns
        full = gather_columns(seis, M * world, dist, group=dist.new_group(backend="gloo"))
        gathered = full.shape[-1] if full is not None else 0

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    hbm, peak_kind = measured_peaks()
    fp64_peak = dgemm_tflops(torch)
    # Algorithmic bytes: 16 B per DOF-update (one read and one write of every FP64 state
    # value per leapfrog step).  Per launch of the two-pass schedule: nsp*M*16 for the
    # stress half-step, nvp*M*16 for the velocity half-step; the schedule itself moves
    # (3*nvp + 3*nsp)*M*8 = 24 B per DOF-update.
    canon_step = (mesh.nvp + mesh.nsp) * M * 16
    canon_s = mesh.nsp * M * 16
    two_pass_step = 3 * (mesh.nvp + mesh.nsp) * M * 8
    ms_step = ms / args.steps
    ach_step = canon_step / (ms_step / 1e3) / 1e9
    dofs_step = (mesh.nvp + mesh.nsp) * M
    if sweep:
        # one launch per step: the dominant (only) kernel
        kern, launch_s, canon_launch = "fom_sweep_kernel", sched["sweep"], canon_step
        fp64_instr = (4 * (mesh.nvp - 2 * mesh.nr) + 2 * mesh.nsp) * M
        sched_bytes = canon_step
    else:
        kern, launch_s, canon_launch = "fom_stress_kernel (dominant: nsp = 2 nvp)", t_s, canon_s
        fp64_instr = (4 * (mesh.nvp - 2 * mesh.nr) + 2 * mesh.nsp) * M
        sched_bytes = two_pass_step
    ach = canon_launch / launch_s / 1e9
    # FP64 pipe: instructions per second against the DGEMM's FMA rate (peak flop/s / 2)
    fp64_pipe_frac = fp64_instr / (ms_step / 1e3) / (fp64_peak * 1e12 / 2)
    bound = "fp64" if fp64_pipe_frac > ach_step / hbm else "hbm"
    line = {
        "metric": METRIC, "value": value, "unit": "DOF-updates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "nth": NTH, "nr": NR, "forcings_per_gpu": M, "dt": dt,
                   "receivers": len(rcv), "seismogram_freq": 1,
                   "l2": "inputs larger than L2 (state 12.3 GB per GPU), no flush needed",
                   "parallelism": "forcing columns sharded across GPUs" if world > 1 else "single GPU",
                   "seismogram_columns_gathered": gathered},
        "roofline": {"bound": bound, "kernel": kern, "achieved": ach, "peak": hbm, "peak_kind": peak_kind,
                     "unit": "GB/s", "frac": ach / hbm,
                     "traffic": ((TRAFFIC_SWEEP_PER_FORCING * M if TRAFFIC_SWEEP_PER_FORCING else None)
                                 if sweep else TRAFFIC_STRESS_PER_FORCING * M),
                     "algorithmic_bytes_per_launch": canon_launch, "launch_ms": launch_s * 1e3,
                     "bytes_per_dof_update": 16,
                     "per_step": {"algorithmic_bytes": canon_step, "ms": ms_step, "achieved": ach_step,
                                  "frac": ach_step / hbm},
                     "schedule_bytes_vs_algorithmic": sched_bytes / canon_step,
                     "fp64_pipe": {"instructions_per_step": fp64_instr, "frac": fp64_pipe_frac,
                                   "peak_tflops": fp64_peak, "peak_kind": "measured (cuBLAS DGEMM 8192^3)"},
                     "schedules_ms_per_launch": {k: v * 1e3 for k, v in sched.items()}},
        "e2e": {"value": e2e_value, "unit": "DOF-updates/s", "h2d_bytes_per_step": h2d / args.steps,
                "d2h_bytes_per_step": d2h / args.steps, "seconds": e2e_s},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    # the timed run against the oracle (host cores, after every GPU timing)
    orc, om, ogids, operiods, orcv, odt = oracle_workload(np, world)
    assert list(ogids) == list(gids) and list(orcv) == list(rcv) and odt == dt
    ref = om.fom_run(2, total_steps, dt, gids, [2] * M, periods, [180.0] * M, rcv, 1, 0, 0)
    line["max_rel_err_vs_oracle"] = {
        "seismogram": _relerr(np, timed_seis, ref["seis"]), "state_vp": _relerr(np, timed_vp, ref["final_vp"]),
        "state_sp": _relerr(np, timed_sp, ref["final_sp"]),
        "compared": "the timed run (%d warm-up + %d timed steps from rest, all %d columns): final state and "
                    "181-receiver seismogram" % (args.warmup, args.steps, M)}
    del ref, timed_vp, timed_sp, om
    if world == 1 and not args.no_extra:  # the other configurations: single-GPU runs only
        line["other_configs"] = extra_workloads(np, torch, shaw)
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = {k: v for k, v in cpu_baseline(np).items() if k in
                                ("value", "unit", "cores", "kind", "sample")}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    global M, WORKLOAD
    args = parse()
    omp_binding()  # before any OpenMP runtime of this process starts
    if args.forcings != M:
        M = args.forcings
        WORKLOAD = "FOM rank-2 FP64, 1000 theta x 2000 r grid, M=%d forcings" % M
    if args.profile_rom:
        import numpy as np
        import shaw_gb300 as shaw
        shaw.build()
        if args.profile_rom.startswith("rank1"):
            av, as_ = stable_rom(np, 256, 3, 0.004, 0.2)
            rng = np.random.default_rng(4)
            prec = shaw.FP64 if args.profile_rom == "rank1-fp64" else shaw.MIXED_FP32
            r = shaw.Rom(av, as_, rng.standard_normal(256) * 1e-3, rank=1, precision=prec)
            r.set_signals("gaussDer", 60.0, 180.0)
            r.set_receivers(rng.standard_normal((181, 256)) / 16.0, 1, args.steps)
        else:
            prec = {"ozaki": shaw.MIXED_OZAKI_BF16, "ozaki-fp64": shaw.OZAKI_FP64, "tf32x3": shaw.MIXED_TF32X3,
                    "fp64": shaw.FP64}[args.profile_rom]
            av, as_ = stable_rom(np, 512, 7, 0.004, 0.2)
            rng = np.random.default_rng(8)
            r = shaw.Rom(av, as_, rng.standard_normal((512, 4096)) * 1e-3, rank=2, precision=prec)
            r.set_signals("gaussDer", rng.uniform(30.0, 90.0, 4096), 180.0)
        r.run(0.5, args.steps)
        print(json.dumps({"profile_rom": args.profile_rom, "steps": args.steps, "launches": r.kernel_launches}))
        r.close()
    elif args.profile_fom in ("rank1", "rank1-wide"):
        import shaw_gb300 as shaw
        shaw.build()
        # config 1: rank 1, 181 surface receivers, on 101 theta x 201 r or the fixture's 201 x 101
        mesh = shaw.Mesh.generate(*((101, 201) if args.profile_fom == "rank1" else (201, 101)))
        mesh.set_material("unilayer", MATERIAL)
        dt = 0.25 * min(mesh.info[5], mesh.info[4] * mesh.info[2]) / (2.0 ** 0.5 * 7300.0)
        f = shaw.Fom(mesh, 1, 1)
        f.set_schedule({"auto": shaw.SCHEDULE_AUTO, "two-pass": shaw.SCHEDULE_TWO_PASS, "sweep": shaw.SCHEDULE_SWEEP,
                        "persistent": shaw.SCHEDULE_PERSISTENT}[args.schedule])
        f.set_sources([mesh.map_source(640.0, 0.0)], "gaussDer", 60.0, 180.0)
        f.set_receivers([mesh.map_receiver(float(a)) for a in range(181)], 1, args.steps)
        f.run(dt, args.steps)
        print(json.dumps({"profile_fom": args.profile_fom, "steps": args.steps, "launches": f.kernel_launches}))
    elif args.profile_fom:
        import numpy as np
        import shaw_gb300 as shaw
        shaw.build()
        mesh = shaw.Mesh.generate(NTH, NR)
        mesh.set_material("unilayer", MATERIAL)
        gids, periods, rcv, dt = workload_inputs(np, mesh)
        m = args.forcings
        f = shaw.Fom(mesh, 2, m, precision=shaw.FP64 if args.profile_fom == "fp64" else shaw.MIXED_FP32)
        f.set_schedule({"auto": shaw.SCHEDULE_AUTO, "two-pass": shaw.SCHEDULE_TWO_PASS,
                        "sweep": shaw.SCHEDULE_SWEEP}[args.schedule])
        f.set_sources(gids[:m], "gaussDer", periods[:m], 180.0)
        f.reset()
        f.advance(dt, args.steps)
        f.synchronize()
        print(json.dumps({"profile_fom": args.profile_fom, "forcings": m, "steps": args.steps,
                          "launches": f.kernel_launches}))
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
