"""ctypes wrapper around the CPU oracle (oracle/shaw_oracle.cpp).

Test infrastructure only: the oracle is the checker the GPU path is compared
against, never part of the product.
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "_build", "libshaw_oracle.so")

SIGNAL_KINDS = {"ricker": 0, "sinusoid": 1, "gaussDer": 2}
MATERIAL_KINDS = {"unilayer": 0, "bilayer": 1, "prem": 2}

_u64p = ctypes.POINTER(ctypes.c_uint64)
_i64p = ctypes.POINTER(ctypes.c_int64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_dp = ctypes.POINTER(ctypes.c_double)

_lib = None


def reference_root():
    """Root of the reference source tree: $SHAW_REFERENCE_ROOT, else the recipes' default
    location.  Only fixture scripts, the pinning tests and the oracle recipe read it; the
    GPU tests, smoke() and the benchmark never do."""
    return os.environ.get("SHAW_REFERENCE_ROOT", "/root/reference")


def _ptr(a, t):
    if a is None:
        return ctypes.cast(None, t)
    return a.ctypes.data_as(t)


def build():
    subprocess.check_call(["make", "-s", "-C", ORACLE_DIR])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        L = ctypes.CDLL(ORACLE_SO)
        L.orc_error.restype = ctypes.c_char_p
        L.orc_mesh_load.restype = ctypes.c_void_p
        L.orc_mesh_load.argtypes = [ctypes.c_char_p]
        L.orc_mesh_free.argtypes = [ctypes.c_void_p]
        L.orc_mesh_info.argtypes = [ctypes.c_void_p, _dp]
        L.orc_mesh_graph.argtypes = [ctypes.c_void_p, _i64p, _i64p, _i32p, _dp, _dp, _dp]
        L.orc_set_material.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp]
        L.orc_material_get.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.orc_crs_sizes.argtypes = [ctypes.c_void_p, ctypes.c_int, _u64p]
        L.orc_crs_get.argtypes = [ctypes.c_void_p, ctypes.c_int, _u64p, _u64p, _dp]
        L.orc_map_source.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, _u64p]
        L.orc_map_receiver.argtypes = [ctypes.c_void_p, ctypes.c_double, _u64p]
        L.orc_signal.restype = ctypes.c_double
        L.orc_signal.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.orc_check_cfl.argtypes = [ctypes.c_void_p, ctypes.c_double, _dp]
        L.orc_check_dispersion.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.orc_fom_run.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.c_double,
                                  _u64p, _i32p, _dp, _dp,
                                  ctypes.c_int, _u64p, ctypes.c_uint64, _dp,
                                  ctypes.c_uint64, ctypes.c_uint64, _dp, _dp, _dp, _dp, ctypes.c_int]
        L.orc_fom_advance.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_double,
                                      _dp, _dp, ctypes.c_int]
        L.orc_num_threads.argtypes = [ctypes.c_int]
        L.orc_rom_operators.argtypes = [ctypes.c_void_p, _dp, ctypes.c_uint64, _dp, ctypes.c_uint64,
                                        _dp, _dp, ctypes.c_int]
        L.orc_rom_forcing_vector.argtypes = [ctypes.c_void_p, _dp, ctypes.c_uint64, ctypes.c_uint64, _dp]
        L.orc_rom_run.argtypes = [ctypes.c_uint64, ctypes.c_uint64, _dp, _dp, ctypes.c_int, _dp,
                                  ctypes.c_uint64, ctypes.c_double, _i32p, _dp, _dp,
                                  ctypes.c_uint64, ctypes.c_uint64, _dp, _dp, _dp, _dp, ctypes.c_int]
        L.orc_rom_seismogram.argtypes = [_dp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, _u64p,
                                         _dp, ctypes.c_uint64, _dp]
        L.orc_fom_advance_forced.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64,
                                             ctypes.c_double, _u64p, _i32p, _dp, _dp, ctypes.c_int, _u64p, _dp,
                                             _dp, _dp, ctypes.c_int]
        L.orc_write_full_mesh.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_double, ctypes.c_char_p]
        _lib = L
    return _lib


def material_params(kind, layers):
    """Flatten material coefficients: unilayer (rho[3], vs[3]); bilayer adds disc_km, rho2[3], vs2[3]."""
    p = np.zeros(13)
    if kind in ("unilayer", "bilayer"):
        rho, vs = layers[0]
        p[0:len(rho)] = rho
        p[3:3 + len(vs)] = vs
    if kind == "bilayer":
        rho, vs, disc = layers[1]
        p[6] = disc
        p[7:7 + len(rho)] = rho
        p[10:10 + len(vs)] = vs
    return p


def write_full_mesh(nth, nr, directory, th_left=0.0, th_right=180.0, r_cmb=3480.0, r_surf=6371.0):
    """The reference mesher's full mesh (two variable groups) written into `directory`."""
    if lib().orc_write_full_mesh(nth, nr, th_left, th_right, r_cmb, r_surf, directory.encode()) != 0:
        raise RuntimeError(lib().orc_error().decode())


class OracleMesh:
    def __init__(self, mesh_dir):
        L = lib()
        self.h = L.orc_mesh_load(mesh_dir.encode())
        if not self.h:
            raise RuntimeError(L.orc_error().decode())
        info = np.zeros(14)
        L.orc_mesh_info(self.h, _ptr(info, _dp))
        self.info = info
        self.nvp, self.nsp, self.nth, self.nr = (int(x) for x in info[8:12])

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_mesh_free(self.h)
            self.h = None

    def graph(self):
        gvp = np.zeros((self.nvp, 5), np.int64)
        gsp = np.zeros((self.nsp, 3), np.int64)
        lab = np.zeros(self.nsp, np.int32)
        cvp = np.zeros((self.nvp, 2))
        csp = np.zeros((self.nsp, 2))
        coeff = np.zeros((self.nvp, 4))
        lib().orc_mesh_graph(self.h, _ptr(gvp, _i64p), _ptr(gsp, _i64p), _ptr(lab, _i32p),
                             _ptr(cvp, _dp), _ptr(csp, _dp), _ptr(coeff, _dp))
        return dict(gvp=gvp, gsp=gsp, labels=lab, coords_vp=cvp, coords_sp=csp, coeff_vp=coeff)

    def set_material(self, kind, layers=None):
        p = material_params(kind, layers or [])
        if lib().orc_set_material(self.h, MATERIAL_KINDS[kind], _ptr(p, _dp)) != 0:
            raise RuntimeError(lib().orc_error().decode())

    def material(self):
        rv = np.zeros(self.nvp)
        gs = np.zeros(self.nsp)
        mm = np.zeros(2)
        lib().orc_material_get(self.h, _ptr(rv, _dp), _ptr(gs, _dp), _ptr(mm, _dp))
        return rv, gs, mm

    def crs(self, which):
        s = np.zeros(3, np.uint64)
        lib().orc_crs_sizes(self.h, which, _ptr(s, _u64p))
        nrows, _, nnz = (int(x) for x in s)
        ptr = np.zeros(nrows + 1, np.uint64)
        ind = np.zeros(nnz, np.uint64)
        val = np.zeros(nnz)
        lib().orc_crs_get(self.h, which, _ptr(ptr, _u64p), _ptr(ind, _u64p), _ptr(val, _dp))
        return ptr, ind, val

    def map_source(self, depth_km, angle_deg):
        g = ctypes.c_uint64(0)
        if lib().orc_map_source(self.h, depth_km, angle_deg, ctypes.byref(g)) != 0:
            raise RuntimeError(lib().orc_error().decode())
        return g.value

    def map_receiver(self, angle_deg):
        g = ctypes.c_uint64(0)
        if lib().orc_map_receiver(self.h, angle_deg, ctypes.byref(g)) != 0:
            raise RuntimeError(lib().orc_error().decode())
        return g.value

    def check_cfl(self, dt):
        v = ctypes.c_double(0)
        rc = lib().orc_check_cfl(self.h, dt, ctypes.byref(v))
        return rc, v.value

    def check_dispersion(self, maxfreq):
        return lib().orc_check_dispersion(self.h, maxfreq)

    def fom_run(self, rank, nsteps, dt, src_gids, kinds, periods, delays,
                rcv_gids=(), seis_freq=0, freq_vp=0, freq_sp=0, nthreads=0, want_final=True):
        M = len(src_gids)
        src = np.asarray(src_gids, np.uint64)
        kd = np.asarray(kinds, np.int32)
        pe = np.asarray(periods, np.float64)
        de = np.asarray(delays, np.float64)
        rc = np.asarray(rcv_gids, np.uint64)
        R = len(rc)
        out = {}
        seis = np.zeros((R, nsteps // seis_freq, M), order="F") if seis_freq else None
        svp = np.zeros((self.nvp, nsteps // freq_vp, M), order="F") if freq_vp else None
        ssp = np.zeros((self.nsp, nsteps // freq_sp, M), order="F") if freq_sp else None
        fvp = np.zeros((self.nvp, M), order="F") if want_final else None
        fsp = np.zeros((self.nsp, M), order="F") if want_final else None
        r = lib().orc_fom_run(self.h, rank, M, nsteps, dt, _ptr(src, _u64p), _ptr(kd, _i32p),
                              _ptr(pe, _dp), _ptr(de, _dp), R, _ptr(rc if R else None, _u64p),
                              seis_freq, _ptr(seis, _dp), freq_vp, freq_sp, _ptr(svp, _dp), _ptr(ssp, _dp),
                              _ptr(fvp, _dp), _ptr(fsp, _dp), nthreads)
        if r != 0:
            raise RuntimeError(lib().orc_error().decode())
        out.update(seis=seis, snaps_vp=svp, snaps_sp=ssp, final_vp=fvp, final_sp=fsp)
        return out

    def fom_advance(self, xv, xs, nsteps, dt, nthreads=0):
        """Advance row-major states (nvp x M, nsp x M) in place with no forcing."""
        M = xv.shape[1]
        r = lib().orc_fom_advance(self.h, M, nsteps, dt, _ptr(xv, _dp), _ptr(xs, _dp), nthreads)
        if r != 0:
            raise RuntimeError(lib().orc_error().decode())

    def fom_advance_forced(self, xv, xs, step0, nsteps, dt, src_gids, kinds, periods, delays, rcv_gids=None,
                           nthreads=0):
        """The rank-2 leapfrog continued in place from step0 completed steps (row-major
        states nvp x M, nsp x M) with the forcing of every column and, when rcv_gids is
        given, the receiver gather of every step.  Returns the last step's receiver row."""
        M = xv.shape[1]
        src = np.ascontiguousarray(src_gids, np.uint64)
        kinds = np.ascontiguousarray(kinds, np.int32)
        periods = np.ascontiguousarray(np.broadcast_to(periods, (M,)), np.float64)
        delays = np.ascontiguousarray(np.broadcast_to(delays, (M,)), np.float64)
        rcv = None if rcv_gids is None else np.ascontiguousarray(rcv_gids, np.uint64)
        R = 0 if rcv is None else len(rcv)
        row = np.zeros((R, M), order="F") if R else None
        r = lib().orc_fom_advance_forced(self.h, M, step0, nsteps, dt, _ptr(src, _u64p), _ptr(kinds, _i32p),
                                         _ptr(periods, _dp), _ptr(delays, _dp), R, _ptr(rcv, _u64p),
                                         _ptr(row, _dp), _ptr(xv, _dp), _ptr(xs, _dp), nthreads)
        if r != 0:
            raise RuntimeError(lib().orc_error().decode())
        return row

    def rom_operators(self, phi_vp, phi_sp, nthreads=0):
        phi_vp = np.asfortranarray(phi_vp, dtype=np.float64)
        phi_sp = np.asfortranarray(phi_sp, dtype=np.float64)
        kv, ks = phi_vp.shape[1], phi_sp.shape[1]
        av = np.zeros((kv, ks))
        as_ = np.zeros((ks, kv))
        r = lib().orc_rom_operators(self.h, _ptr(phi_vp, _dp), kv, _ptr(phi_sp, _dp), ks,
                                    _ptr(av, _dp), _ptr(as_, _dp), nthreads)
        if r != 0:
            raise RuntimeError(lib().orc_error().decode())
        return av, as_

    def rom_forcing_vector(self, phi_vp, src_gid):
        phi_vp = np.asfortranarray(phi_vp, dtype=np.float64)
        b = np.zeros(phi_vp.shape[1])
        lib().orc_rom_forcing_vector(self.h, _ptr(phi_vp, _dp), phi_vp.shape[1], src_gid, _ptr(b, _dp))
        return b


def signal(kind, delay, period, t):
    return lib().orc_signal(SIGNAL_KINDS.get(kind, kind), delay, period, t)


def rom_run(av, as_, b, nsteps, dt, kinds, periods, delays, freq_vp=0, freq_sp=0, nthreads=0):
    av = np.ascontiguousarray(av, np.float64)
    as_ = np.ascontiguousarray(as_, np.float64)
    b = np.asfortranarray(b, np.float64)
    kv, ks = av.shape
    M = b.shape[1]
    kd = np.asarray(kinds, np.int32)
    pe = np.asarray(periods, np.float64)
    de = np.asarray(delays, np.float64)
    svp = np.zeros((kv, nsteps // freq_vp, M), order="F") if freq_vp else None
    ssp = np.zeros((ks, nsteps // freq_sp, M), order="F") if freq_sp else None
    fvp = np.zeros((kv, M), order="F")
    fsp = np.zeros((ks, M), order="F")
    r = lib().orc_rom_run(kv, ks, _ptr(av, _dp), _ptr(as_, _dp), M, _ptr(b, _dp), nsteps, dt,
                          _ptr(kd, _i32p), _ptr(pe, _dp), _ptr(de, _dp), freq_vp, freq_sp,
                          _ptr(svp, _dp), _ptr(ssp, _dp), _ptr(fvp, _dp), _ptr(fsp, _dp), nthreads)
    if r != 0:
        raise RuntimeError(lib().orc_error().decode())
    return dict(snaps_vp=svp, snaps_sp=ssp, final_vp=fvp, final_sp=fsp)
