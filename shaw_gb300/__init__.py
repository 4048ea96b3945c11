"""shaw_gb300 -- Python view of the C ABI in include/shaw_gpu.h.

The compute path is libshaw_gpu.so (hand-written sm_103a CUDA kernels + C ABI),
built in-tree by shaw_gb300.build.  This module only binds it with ctypes: it
has no compute fallback, and importing it fails loudly when the library has not
been built.

The classes mirror the reference's objects for the hot path:
  Mesh  -- MeshInfo + mesh readers + material model + grid mappers + checkers
  Fom   -- ShWavePP operators + runFom (rank-1 / rank-2 leapfrog on the GPU)
  Rom   -- reduced operators + runRomRankOneForcing / runRomRankTwoForcing
"""
import ctypes
import os

import numpy as np

from . import build as _build_mod

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libshaw_gpu.so")
EXE_PATH = os.path.join(_HERE, "_build", "shaw_exe")
POD_EXE_PATH = os.path.join(_HERE, "_build", "computeThinSVD")

OK = 0
ERR_INVALID_ARG = 1
ERR_CUDA = 2
ERR_MESH = 3
ERR_FREQ_DIVISOR = 4
ERR_CFL = 5
ERR_DISPERSION = 6
ERR_FORCING_SETS = 7
ERR_NONFINITE = 8
ERR_IO = 9
ERR_PARSE = 10
ERR_UNSUPPORTED = 11
ERR_OUT_OF_MEMORY = 12
ERR_STATE = 13

SIGNAL = {"ricker": 0, "sinusoid": 1, "gaussDer": 2}
MATERIAL = {"unilayer": 0, "bilayer": 1, "prem": 2}
# MIXED_TF32X3 is experimental: it does not meet the 1e-6 mixed-precision bar (see the C header).
FP64, MIXED_TF32X3, MIXED_FP32, MIXED_OZAKI_BF16, OZAKI_FP64 = 0, 1, 3, 4, 5
SCHEDULE_AUTO, SCHEDULE_TWO_PASS, SCHEDULE_SWEEP, SCHEDULE_PERSISTENT = 0, 1, 2, 3
ROM_SCHEDULE_AUTO, ROM_SCHEDULE_CLUSTER, ROM_SCHEDULE_BANDS = 0, 1, 2


class ShawError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("shaw error %d: %s" % (code, msg))
        self.code = code


def build():
    """Compile libshaw_gpu.so, shaw_exe and computeThinSVD for sm_103a (idempotent)."""
    return _build_mod.build()


_u64p = ctypes.POINTER(ctypes.c_uint64)
_i64p = ctypes.POINTER(ctypes.c_int64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p


class OperatorDesc(ctypes.Structure):
    _fields_ = [("nth", ctypes.c_uint64), ("nr", ctypes.c_uint64), ("nvp", ctypes.c_uint64),
                ("nsp", ctypes.c_uint64), ("dth_inv", ctypes.c_double), ("drr_inv", ctypes.c_double),
                ("graph_vp", _i64p), ("graph_sp", _i64p), ("labels_sp", _i32p),
                ("coords_vp", _dp), ("coords_sp", _dp), ("cot_vp", _dp), ("cot_sp", _dp),
                ("coeff_vp", _dp), ("rho_inv_vp", _dp), ("shear_mod_sp", _dp)]


# (name, restype, argtypes) of every exported entry point declared in include/shaw_gpu.h
SIGNATURES = [
    ("shaw_last_error", ctypes.c_char_p, []),
    ("shaw_version", ctypes.c_char_p, []),
    ("shaw_fom_create", ctypes.c_int, [ctypes.POINTER(OperatorDesc), ctypes.c_int, ctypes.c_uint32, ctypes.c_int,
                                       ctypes.POINTER(_vp)]),
    ("shaw_fom_destroy", None, [_vp]),
    ("shaw_fom_set_sources", ctypes.c_int, [_vp, _u64p, _i32p, _dp, _dp]),
    ("shaw_fom_set_receivers", ctypes.c_int, [_vp, _u64p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64]),
    ("shaw_fom_set_snapshots", ctypes.c_int, [_vp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, _dp, _dp]),
    ("shaw_fom_run", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_uint64]),
    ("shaw_fom_reset", ctypes.c_int, [_vp]),
    ("shaw_fom_advance", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_uint64]),
    ("shaw_fom_update_velocity", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_uint64]),
    ("shaw_fom_update_stress", ctypes.c_int, [_vp, ctypes.c_double]),
    ("shaw_fom_synchronize", ctypes.c_int, [_vp]),
    ("shaw_fom_get_seismogram", ctypes.c_int, [_vp, _dp]),
    ("shaw_fom_get_state", ctypes.c_int, [_vp, _dp, _dp]),
    ("shaw_fom_set_state", ctypes.c_int, [_vp, _dp, _dp]),
    ("shaw_fom_stream", _vp, [_vp]),
    ("shaw_fom_set_schedule", ctypes.c_int, [_vp, ctypes.c_int]),
    ("shaw_fom_kernel_launches", ctypes.c_uint64, [_vp]),
    ("shaw_rom_project", ctypes.c_int, [_vp, _dp, ctypes.c_uint64, _dp, ctypes.c_uint64, _dp, _dp]),
    ("shaw_rom_project_noalloc", ctypes.c_int, [_vp, _vp, ctypes.c_uint64, _vp, ctypes.c_uint64, _vp, _vp, _vp]),
    ("shaw_rom_batch_create", ctypes.c_int, [ctypes.c_uint32, _vp, ctypes.c_int, ctypes.POINTER(_vp)]),
    ("shaw_rom_batch_destroy", None, [_vp]),
    ("shaw_rom_batch_tune", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_uint64, ctypes.c_char_p, ctypes.c_size_t]),
    ("shaw_rom_batch_set_tiling", ctypes.c_int, [_vp, ctypes.c_uint32, ctypes.c_int]),
    ("shaw_selftest_bounded_waits", ctypes.c_int, [ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint32)]),
    ("shaw_rom_batch_set_snapshots", ctypes.c_int, [_vp, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64,
                                                    ctypes.c_uint64, _dp, _dp]),
    ("shaw_rom_batch_set_receivers", ctypes.c_int, [_vp, ctypes.c_uint32, _dp, ctypes.c_uint32, ctypes.c_uint64,
                                                    ctypes.c_uint64]),
    ("shaw_rom_batch_get_seismogram", ctypes.c_int, [_vp, ctypes.c_uint32, _dp]),
    ("shaw_rom_batch_reset", ctypes.c_int, [_vp]),
    ("shaw_rom_batch_advance", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_uint64]),
    ("shaw_rom_batch_run", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_uint64]),
    ("shaw_rom_batch_synchronize", ctypes.c_int, [_vp]),
    ("shaw_rom_batch_get_state", ctypes.c_int, [_vp, ctypes.c_uint32, _dp, _dp]),
    ("shaw_rom_batch_describe", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_size_t]),
    ("shaw_rom_batch_stream", _vp, [_vp]),
    ("shaw_rom_batch_kernel_launches", ctypes.c_uint64, [_vp]),
    ("shaw_rom_batch_step", ctypes.c_uint64, [_vp]),
    ("shaw_pod", ctypes.c_int, [_dp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, _dp, _dp]),
    ("shaw_pod_tool", ctypes.c_int, [ctypes.POINTER(ctypes.c_char_p), ctypes.c_uint32, ctypes.c_char_p,
                                     ctypes.c_char_p, ctypes.c_int]),
    ("shaw_rom_create", ctypes.c_int, [ctypes.c_uint64, ctypes.c_uint64, _dp, _dp, ctypes.c_int, ctypes.c_uint32,
                                       _dp, ctypes.c_int, ctypes.POINTER(_vp)]),
    ("shaw_rom_destroy", None, [_vp]),
    ("shaw_rom_set_signals", ctypes.c_int, [_vp, _i32p, _dp, _dp]),
    ("shaw_rom_set_snapshots", ctypes.c_int, [_vp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, _dp, _dp]),
    ("shaw_rom_set_receivers", ctypes.c_int, [_vp, _dp, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64]),
    ("shaw_rom_run", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_uint64]),
    ("shaw_rom_reset", ctypes.c_int, [_vp]),
    ("shaw_rom_set_schedule", ctypes.c_int, [_vp, ctypes.c_int]),
    ("shaw_rom_advance", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_uint64]),
    ("shaw_rom_synchronize", ctypes.c_int, [_vp]),
    ("shaw_rom_get_state", ctypes.c_int, [_vp, _dp, _dp]),
    ("shaw_rom_get_seismogram", ctypes.c_int, [_vp, _dp]),
    ("shaw_rom_stream", _vp, [_vp]),
    ("shaw_rom_kernel_launches", ctypes.c_uint64, [_vp]),
    ("shaw_mesh_load", ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_vp)]),
    ("shaw_mesh_generate", ctypes.c_int, [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_double, ctypes.POINTER(_vp)]),
    ("shaw_mesh_write", ctypes.c_int, [_vp, ctypes.c_char_p]),
    ("shaw_mesh_info", ctypes.c_int, [_vp, _dp]),
    ("shaw_mesh_set_material", ctypes.c_int, [_vp, ctypes.c_int, _dp, ctypes.c_uint32]),
    ("shaw_mesh_set_material_arrays", ctypes.c_int, [_vp, _dp, _dp]),
    ("shaw_mesh_min_max_vs", ctypes.c_int, [_vp, _dp]),
    ("shaw_mesh_operator_desc", ctypes.c_int, [_vp, ctypes.POINTER(OperatorDesc)]),
    ("shaw_mesh_map_source", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double, _u64p]),
    ("shaw_mesh_map_receiver", ctypes.c_int, [_vp, ctypes.c_double, _u64p]),
    ("shaw_mesh_check_cfl", ctypes.c_int, [_vp, ctypes.c_double, _dp]),
    ("shaw_mesh_check_dispersion", ctypes.c_int, [_vp, ctypes.c_double]),
    ("shaw_mesh_destroy", None, [_vp]),
    ("shaw_run_input_file", ctypes.c_int, [ctypes.c_char_p]),
    ("shaw_parse_input", ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t]),
]

_lib = None


def lib():
    """The loaded libshaw_gpu.so; raises when it was not built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libshaw_gpu.so is missing (%s): run shaw_gb300.build() first" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name, None)
            if f is None:
                continue
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(rc):
    if rc != OK:
        raise ShawError(rc, lib().shaw_last_error().decode())


def _p(a, t):
    return ctypes.cast(None, t) if a is None else a.ctypes.data_as(t)


class Mesh:
    """MeshInfo + graph/coeff readers (or the full-mesh generator) + material."""

    def __init__(self, handle):
        self.h = handle
        info = np.zeros(14)
        _check(lib().shaw_mesh_info(self.h, _p(info, _dp)))
        self.info = info
        self.nvp, self.nsp, self.nth, self.nr = (int(x) for x in info[8:12])
        self._desc = None

    @classmethod
    def load(cls, mesh_dir):
        h = _vp()
        _check(lib().shaw_mesh_load(os.fsencode(mesh_dir), ctypes.byref(h)))
        return cls(h)

    @classmethod
    def generate(cls, nth, nr, th_left=0.0, th_right=180.0, r_cmb=3480.0, r_surf=6371.0):
        h = _vp()
        _check(lib().shaw_mesh_generate(nth, nr, th_left, th_right, r_cmb, r_surf, ctypes.byref(h)))
        return cls(h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().shaw_mesh_destroy(self.h)
            self.h = None

    def write(self, mesh_dir):
        _check(lib().shaw_mesh_write(self.h, os.fsencode(mesh_dir)))

    def set_material(self, kind, params=()):
        p = np.zeros(13)
        p[:len(params)] = params
        _check(lib().shaw_mesh_set_material(self.h, MATERIAL[kind], _p(p, _dp), len(p)))

    def set_material_arrays(self, rho_inv_vp, shear_mod_sp):
        a = np.ascontiguousarray(rho_inv_vp, np.float64)
        b = np.ascontiguousarray(shear_mod_sp, np.float64)
        _check(lib().shaw_mesh_set_material_arrays(self.h, _p(a, _dp), _p(b, _dp)))

    def min_max_vs(self):
        mm = np.zeros(2)
        _check(lib().shaw_mesh_min_max_vs(self.h, _p(mm, _dp)))
        return mm

    def operator_desc(self):
        d = OperatorDesc()
        _check(lib().shaw_mesh_operator_desc(self.h, ctypes.byref(d)))
        self._desc = d
        return d

    def arrays(self):
        """Copies of the descriptor arrays (gid-indexed), for inspection in tests."""
        d = self.operator_desc()

        def get(ptr, n, dt, shape):
            return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dt).reshape(shape).copy()
        nvp, nsp = self.nvp, self.nsp
        return dict(graph_vp=get(d.graph_vp, nvp * 5, np.int64, (nvp, 5)),
                    graph_sp=get(d.graph_sp, nsp * 3, np.int64, (nsp, 3)),
                    labels=get(d.labels_sp, nsp, np.int32, (nsp,)),
                    coords_vp=get(d.coords_vp, nvp * 2, np.float64, (nvp, 2)),
                    coords_sp=get(d.coords_sp, nsp * 2, np.float64, (nsp, 2)),
                    cot_vp=get(d.cot_vp, nvp, np.float64, (nvp,)),
                    cot_sp=get(d.cot_sp, nsp, np.float64, (nsp,)),
                    coeff_vp=get(d.coeff_vp, nvp * 4, np.float64, (nvp, 4)),
                    rho_inv_vp=get(d.rho_inv_vp, nvp, np.float64, (nvp,)),
                    shear_mod_sp=get(d.shear_mod_sp, nsp, np.float64, (nsp,)))

    def map_source(self, depth_km, angle_deg):
        g = ctypes.c_uint64()
        _check(lib().shaw_mesh_map_source(self.h, depth_km, angle_deg, ctypes.byref(g)))
        return g.value

    def map_receiver(self, angle_deg):
        g = ctypes.c_uint64()
        _check(lib().shaw_mesh_map_receiver(self.h, angle_deg, ctypes.byref(g)))
        return g.value

    def check_cfl(self, dt):
        v = ctypes.c_double()
        rc = lib().shaw_mesh_check_cfl(self.h, dt, ctypes.byref(v))
        return rc, v.value

    def check_dispersion(self, max_freq):
        return lib().shaw_mesh_check_dispersion(self.h, max_freq)


class Fom:
    """Device-resident FOM (rank 1 or 2) driven through the C ABI."""

    def __init__(self, mesh, rank=1, num_forcings=1, precision=FP64):
        self.mesh = mesh
        self.M = num_forcings
        self.nvp, self.nsp = mesh.nvp, mesh.nsp
        d = mesh.operator_desc()
        h = _vp()
        _check(lib().shaw_fom_create(ctypes.byref(d), rank, num_forcings, precision, ctypes.byref(h)))
        self.h = h
        self._snaps = None
        self.R = 0
        self.T = 0

    def close(self):
        if getattr(self, "h", None):
            lib().shaw_fom_destroy(self.h)
            self.h = None

    __del__ = close

    def set_sources(self, gids, kinds, periods, delays):
        M = self.M
        g = np.ascontiguousarray(np.broadcast_to(np.asarray(gids, np.uint64), (M,)))
        k = np.ascontiguousarray(np.broadcast_to(np.asarray([SIGNAL.get(x, x) for x in np.atleast_1d(kinds)],
                                                            np.int32), (M,)))
        p = np.ascontiguousarray(np.broadcast_to(np.asarray(periods, np.float64), (M,)))
        d = np.ascontiguousarray(np.broadcast_to(np.asarray(delays, np.float64), (M,)))
        _check(lib().shaw_fom_set_sources(self.h, _p(g, _u64p), _p(k, _i32p), _p(p, _dp), _p(d, _dp)))

    def set_receivers(self, gids, freq, nsteps):
        g = np.ascontiguousarray(gids, np.uint64)
        _check(lib().shaw_fom_set_receivers(self.h, _p(g, _u64p), len(g), freq, nsteps))
        self.R = len(g)
        self.T = nsteps // freq if freq else 0

    def set_snapshots(self, freq_vp, freq_sp, nsteps):
        if freq_vp == 0:
            _check(lib().shaw_fom_set_snapshots(self.h, 0, 0, 0, None, None))
            self._snaps = None
            return
        svp = np.zeros((self.nvp, nsteps // freq_vp, self.M), order="F")
        ssp = np.zeros((self.nsp, nsteps // freq_sp, self.M), order="F")
        _check(lib().shaw_fom_set_snapshots(self.h, freq_vp, freq_sp, nsteps, _p(svp, _dp), _p(ssp, _dp)))
        self._snaps = (svp, ssp)

    def snapshots(self):
        return self._snaps

    def run(self, dt, nsteps):
        _check(lib().shaw_fom_run(self.h, dt, nsteps))

    def reset(self):
        _check(lib().shaw_fom_reset(self.h))

    def advance(self, dt, nsteps):
        _check(lib().shaw_fom_advance(self.h, dt, nsteps))

    def update_velocity(self, dt, step):
        _check(lib().shaw_fom_update_velocity(self.h, dt, step))

    def update_stress(self, dt):
        _check(lib().shaw_fom_update_stress(self.h, dt))

    def synchronize(self):
        _check(lib().shaw_fom_synchronize(self.h))

    def seismogram(self):
        out = np.zeros((self.R, self.T, self.M), order="F")
        _check(lib().shaw_fom_get_seismogram(self.h, _p(out, _dp)))
        return out

    def get_state(self):
        vp = np.zeros((self.nvp, self.M), order="F")
        sp = np.zeros((self.nsp, self.M), order="F")
        _check(lib().shaw_fom_get_state(self.h, _p(vp, _dp), _p(sp, _dp)))
        return vp, sp

    def set_state(self, vp, sp):
        vp = np.asfortranarray(vp, np.float64).reshape((self.nvp, self.M), order="F")
        sp = np.asfortranarray(sp, np.float64).reshape((self.nsp, self.M), order="F")
        _check(lib().shaw_fom_set_state(self.h, _p(vp, _dp), _p(sp, _dp)))

    def set_schedule(self, schedule):
        """SCHEDULE_AUTO, SCHEDULE_TWO_PASS, SCHEDULE_SWEEP or SCHEDULE_PERSISTENT (see shaw_fom_set_schedule)."""
        _check(lib().shaw_fom_set_schedule(self.h, schedule))

    @property
    def stream(self):
        return lib().shaw_fom_stream(self.h)

    @property
    def kernel_launches(self):
        return lib().shaw_fom_kernel_launches(self.h)


def rom_project(fom, phi_vp, phi_sp):
    """(romJvp, romJsp) = (PhiVp^T Jvp PhiSp, PhiSp^T Jsp PhiVp), FP64 on the GPU."""
    pv = np.asfortranarray(phi_vp, np.float64)
    ps = np.asfortranarray(phi_sp, np.float64)
    kv, ks = pv.shape[1], ps.shape[1]
    av = np.zeros((kv, ks))
    as_ = np.zeros((ks, kv))
    _check(lib().shaw_rom_project(fom.h, _p(pv, _dp), kv, _p(ps, _dp), ks, _p(av, _dp), _p(as_, _dp)))
    return av, as_


class RomInstanceDesc(ctypes.Structure):
    _fields_ = [("kv", ctypes.c_uint64), ("ks", ctypes.c_uint64), ("num_forcings", ctypes.c_uint32),
                ("rom_jvp", _dp), ("rom_jsp", _dp), ("b", _dp), ("kind", _i32p), ("period", _dp), ("delay", _dp)]


class RomBatch:
    """Many rank-2 reduced systems of uneven size advanced together on the GPU.

    instances: sequence of dicts with keys rom_jvp (kv x ks), rom_jsp (ks x kv), b
    (kv x M) and the per-column signals kind, period, delay (scalars broadcast)."""

    def __init__(self, instances, precision=FP64):
        self._keep = []
        descs = (RomInstanceDesc * len(instances))()
        self.shapes = []
        for d, inst in zip(descs, instances):
            av = np.ascontiguousarray(inst["rom_jvp"], np.float64)
            as_ = np.ascontiguousarray(inst["rom_jsp"], np.float64)
            kv, ks = av.shape
            b = np.asfortranarray(np.asarray(inst["b"], np.float64).reshape(kv, -1, order="F"))
            M = b.shape[1]
            k = np.ascontiguousarray(np.broadcast_to(
                np.asarray([SIGNAL.get(x, x) for x in np.atleast_1d(inst.get("kind", "gaussDer"))], np.int32), (M,)))
            p = np.ascontiguousarray(np.broadcast_to(np.asarray(inst["period"], np.float64), (M,)))
            dl = np.ascontiguousarray(np.broadcast_to(np.asarray(inst.get("delay", 0.0), np.float64), (M,)))
            self._keep += [av, as_, b, k, p, dl]
            d.kv, d.ks, d.num_forcings = kv, ks, M
            d.rom_jvp, d.rom_jsp, d.b = _p(av, _dp), _p(as_, _dp), _p(b, _dp)
            d.kind, d.period, d.delay = _p(k, _i32p), _p(p, _dp), _p(dl, _dp)
            self.shapes.append((kv, ks, M))
        h = _vp()
        _check(lib().shaw_rom_batch_create(len(instances), ctypes.cast(descs, _vp), precision, ctypes.byref(h)))
        self.h = h
        self._keep = []
        self._snaps = {}
        self._seis = {}

    def close(self):
        if getattr(self, "h", None):
            lib().shaw_rom_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def tune(self, dt, trial_steps=4):
        buf = ctypes.create_string_buffer(4096)
        _check(lib().shaw_rom_batch_tune(self.h, dt, trial_steps, buf, len(buf)))
        return buf.value.decode()

    def set_tiling(self, width, paired=False):
        """Fixed tensor-core tiling: `width` forcing columns per tile (16, 32, 64), each
        tile optionally split across two co-resident CTAs."""
        _check(lib().shaw_rom_batch_set_tiling(self.h, width, int(bool(paired))))

    def describe(self):
        buf = ctypes.create_string_buffer(512)
        _check(lib().shaw_rom_batch_describe(self.h, buf, len(buf)))
        return buf.value.decode()

    def set_snapshots(self, i, freq_vp, freq_sp, nsteps):
        kv, ks, M = self.shapes[i]
        svp = np.zeros((kv, nsteps // freq_vp, M), order="F")
        ssp = np.zeros((ks, nsteps // freq_sp, M), order="F")
        _check(lib().shaw_rom_batch_set_snapshots(self.h, i, freq_vp, freq_sp, nsteps, _p(svp, _dp), _p(ssp, _dp)))
        self._snaps[i] = (svp, ssp)

    def snapshots(self, i):
        return self._snaps[i]

    def set_receivers(self, i, phi_rows, freq, nsteps):
        pr = np.ascontiguousarray(phi_rows, np.float64)
        _check(lib().shaw_rom_batch_set_receivers(self.h, i, _p(pr, _dp), pr.shape[0], freq, nsteps))
        self._seis[i] = (pr.shape[0], nsteps // freq)

    def seismogram(self, i):
        R, T = self._seis[i]
        out = np.zeros((R, T, self.shapes[i][2]), order="F")
        _check(lib().shaw_rom_batch_get_seismogram(self.h, i, _p(out, _dp)))
        return out

    def reset(self):
        _check(lib().shaw_rom_batch_reset(self.h))

    def advance(self, dt, nsteps):
        _check(lib().shaw_rom_batch_advance(self.h, dt, nsteps))

    def run(self, dt, nsteps):
        _check(lib().shaw_rom_batch_run(self.h, dt, nsteps))

    def synchronize(self):
        _check(lib().shaw_rom_batch_synchronize(self.h))

    def get_state(self, i):
        kv, ks, M = self.shapes[i]
        xv = np.zeros((kv, M), order="F")
        xs = np.zeros((ks, M), order="F")
        _check(lib().shaw_rom_batch_get_state(self.h, i, _p(xv, _dp), _p(xs, _dp)))
        return xv, xs

    @property
    def stream(self):
        return lib().shaw_rom_batch_stream(self.h)

    @property
    def kernel_launches(self):
        return lib().shaw_rom_batch_kernel_launches(self.h)


def pod(snaps, method=2):
    """Thin SVD of the n x t snapshot matrix on the GPU (computeThinSVD,
    src/tools/main_eigen_svd.cc:113-197): returns (U n x min(n,t), singular values).
    Each column of U is determined up to its sign."""
    a = np.asfortranarray(snaps, np.float64)
    n, t = a.shape
    k = min(n, t)
    u = np.zeros((n, k), order="F")
    sv = np.zeros(k)
    _check(lib().shaw_pod(_p(a, _dp), n, t, method, _p(u, _dp), _p(sv, _dp)))
    return u, sv


def pod_tool(dirs, informat="binary", outformat="binary", method=2):
    """computeThinSVD --dirs ... --informat ... --outformat ... --method ...: writes
    sva_vp, lsv_vp, sva_sp, lsv_sp into the current directory."""
    arr = (ctypes.c_char_p * len(dirs))(*[os.fsencode(d) for d in dirs])
    _check(lib().shaw_pod_tool(arr, len(dirs), informat.encode(), outformat.encode(), method))


class Rom:
    """Reduced-order leapfrog on the GPU (rank 1 or 2)."""

    def __init__(self, rom_jvp, rom_jsp, b, rank=1, precision=FP64):
        av = np.ascontiguousarray(rom_jvp, np.float64)
        as_ = np.ascontiguousarray(rom_jsp, np.float64)
        b = np.asfortranarray(np.asarray(b, np.float64).reshape(av.shape[0], -1, order="F"))
        self.kv, self.ks = av.shape
        self.M = b.shape[1]
        h = _vp()
        _check(lib().shaw_rom_create(self.kv, self.ks, _p(av, _dp), _p(as_, _dp), rank, self.M, _p(b, _dp),
                                     precision, ctypes.byref(h)))
        self.h = h
        self._snaps = None
        self.R = self.T = 0

    def close(self):
        if getattr(self, "h", None):
            lib().shaw_rom_destroy(self.h)
            self.h = None

    __del__ = close

    def set_signals(self, kinds, periods, delays):
        M = self.M
        k = np.ascontiguousarray(np.broadcast_to(np.asarray([SIGNAL.get(x, x) for x in np.atleast_1d(kinds)],
                                                            np.int32), (M,)))
        p = np.ascontiguousarray(np.broadcast_to(np.asarray(periods, np.float64), (M,)))
        d = np.ascontiguousarray(np.broadcast_to(np.asarray(delays, np.float64), (M,)))
        _check(lib().shaw_rom_set_signals(self.h, _p(k, _i32p), _p(p, _dp), _p(d, _dp)))

    def set_snapshots(self, freq_vp, freq_sp, nsteps):
        if freq_vp == 0:
            _check(lib().shaw_rom_set_snapshots(self.h, 0, 0, 0, None, None))
            self._snaps = None
            return
        svp = np.zeros((self.kv, nsteps // freq_vp, self.M), order="F")
        ssp = np.zeros((self.ks, nsteps // freq_sp, self.M), order="F")
        _check(lib().shaw_rom_set_snapshots(self.h, freq_vp, freq_sp, nsteps, _p(svp, _dp), _p(ssp, _dp)))
        self._snaps = (svp, ssp)

    def snapshots(self):
        return self._snaps

    def set_receivers(self, phi_rows, freq, nsteps):
        pr = np.ascontiguousarray(phi_rows, np.float64)
        _check(lib().shaw_rom_set_receivers(self.h, _p(pr, _dp), pr.shape[0], freq, nsteps))
        self.R, self.T = pr.shape[0], nsteps // freq

    def run(self, dt, nsteps):
        _check(lib().shaw_rom_run(self.h, dt, nsteps))

    def reset(self):
        _check(lib().shaw_rom_reset(self.h))

    def set_schedule(self, schedule):
        """ROM_SCHEDULE_AUTO, ROM_SCHEDULE_CLUSTER or ROM_SCHEDULE_BANDS (see shaw_rom_set_schedule)."""
        _check(lib().shaw_rom_set_schedule(self.h, schedule))

    def advance(self, dt, nsteps):
        _check(lib().shaw_rom_advance(self.h, dt, nsteps))

    def synchronize(self):
        _check(lib().shaw_rom_synchronize(self.h))

    def get_state(self):
        xv = np.zeros((self.kv, self.M), order="F")
        xs = np.zeros((self.ks, self.M), order="F")
        _check(lib().shaw_rom_get_state(self.h, _p(xv, _dp), _p(xs, _dp)))
        return xv, xs

    def seismogram(self):
        out = np.zeros((self.R, self.T, self.M), order="F")
        _check(lib().shaw_rom_get_seismogram(self.h, _p(out, _dp)))
        return out

    @property
    def stream(self):
        return lib().shaw_rom_stream(self.h)

    @property
    def kernel_launches(self):
        return lib().shaw_rom_kernel_launches(self.h)


def parse_input(path):
    """The parsed input file as a dict of the reference's getter names -> text values."""
    buf = ctypes.create_string_buffer(1 << 16)
    _check(lib().shaw_parse_input(os.fsencode(path), buf, len(buf)))
    out = {}
    for ln in buf.value.decode().splitlines():
        k, _, v = ln.partition("=")
        out[k] = v
    return out


def run_input_file(path):
    """shawExe <input.yaml>: outputs land in the current directory."""
    _check(lib().shaw_run_input_file(os.fsencode(path)))
