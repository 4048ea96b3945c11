"""The allocation-free projection entry point, shaw_rom_project_noalloc.

It serves callers that cannot allocate device memory while they run (a fixed
memory budget handed over up front, a code path where an allocation would
synchronise the device, a runtime that owns all device allocations).  This test
calls it through the C ABI with caller-owned device buffers and checks it
against shaw_rom_project, the allocating entry point, to the 1e-12 relative
tolerance of the other FP64 parity tests -- on two calls in a row, since every
call reuses the same fixed scratch array.  It lives in its own file so that it
runs after every other test; it passes alone in a fresh process as well.
"""
import ctypes

import numpy as np
import pytest

from conftest import mesh_dir

pytestmark = pytest.mark.gpu


def relerr(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def test_noalloc_projection_matches_allocating_projection(shaw):
    torch = pytest.importorskip("torch")
    m = shaw.Mesh.load(mesh_dir("fullMesh21x51"))
    m.set_material("unilayer", [2000.0, 0.0, 0.0, 5000.0, 0.0, 0.0])
    fom = shaw.Fom(m, 1, 1)
    rng = np.random.default_rng(42)
    kv, ks = 40, 56
    pv = np.asfortranarray(np.linalg.qr(rng.standard_normal((m.nvp, kv)))[0])
    ps = np.asfortranarray(np.linalg.qr(rng.standard_normal((m.nsp, ks)))[0])
    ref_v, ref_s = shaw.rom_project(fom, pv, ps)

    dev = torch.device("cuda:0")
    d_pv = torch.from_numpy(pv.ravel(order="F").copy()).to(dev)
    d_ps = torch.from_numpy(ps.ravel(order="F").copy()).to(dev)
    stream = torch.cuda.current_stream(dev)
    for call in range(2):
        d_av = torch.full((kv * ks,), float("nan"), dtype=torch.float64, device=dev)
        d_as = torch.full((ks * kv,), float("nan"), dtype=torch.float64, device=dev)
        rc = shaw.lib().shaw_rom_project_noalloc(fom.h, ctypes.c_void_p(d_pv.data_ptr()), kv,
                                                 ctypes.c_void_p(d_ps.data_ptr()), ks,
                                                 ctypes.c_void_p(d_av.data_ptr()), ctypes.c_void_p(d_as.data_ptr()),
                                                 ctypes.c_void_p(stream.cuda_stream))
        assert rc == shaw.OK, shaw.lib().shaw_last_error().decode()
        torch.cuda.synchronize()
        av = d_av.cpu().numpy().reshape(kv, ks)
        as_ = d_as.cpu().numpy().reshape(ks, kv)
        assert np.all(np.isfinite(av)) and np.all(np.isfinite(as_)), call
        assert relerr(av, ref_v) <= 1e-12 and relerr(as_, ref_s) <= 1e-12, call
    fom.close()


def test_noalloc_projection_on_a_mesh_larger_than_its_scratch(shaw):
    """nsp = 4,198,900 rows: J*Phi passes through the 16 MiB array in 129 row blocks
    (32768 rows x 64 modes each); two calls in a row against the allocating path."""
    torch = pytest.importorskip("torch")
    m = shaw.Mesh.generate(1000, 2100)
    m.set_material("unilayer", [3300.0, 0.0, 0.0, 4400.0, 0.0, 0.0])
    fom = shaw.Fom(m, 1, 1)
    rng = np.random.default_rng(7)
    kv, ks = 64, 48
    pv = np.asfortranarray(rng.standard_normal((m.nvp, kv)) / np.sqrt(m.nvp))
    ps = np.asfortranarray(rng.standard_normal((m.nsp, ks)) / np.sqrt(m.nsp))
    ref_v, ref_s = shaw.rom_project(fom, pv, ps)
    dev = torch.device("cuda:0")
    d_pv = torch.from_numpy(pv.ravel(order="F").copy()).to(dev)
    d_ps = torch.from_numpy(ps.ravel(order="F").copy()).to(dev)
    stream = torch.cuda.current_stream(dev)
    for call in range(2):
        d_av = torch.full((kv * ks,), float("nan"), dtype=torch.float64, device=dev)
        d_as = torch.full((ks * kv,), float("nan"), dtype=torch.float64, device=dev)
        rc = shaw.lib().shaw_rom_project_noalloc(fom.h, ctypes.c_void_p(d_pv.data_ptr()), kv,
                                                 ctypes.c_void_p(d_ps.data_ptr()), ks,
                                                 ctypes.c_void_p(d_av.data_ptr()), ctypes.c_void_p(d_as.data_ptr()),
                                                 ctypes.c_void_p(stream.cuda_stream))
        assert rc == shaw.OK, shaw.lib().shaw_last_error().decode()
        torch.cuda.synchronize()
        av = d_av.cpu().numpy().reshape(kv, ks)
        as_ = d_as.cpu().numpy().reshape(ks, kv)
        assert relerr(av, ref_v) <= 1e-12 and relerr(as_, ref_s) <= 1e-12, call
    fom.close()


def test_noalloc_projection_rejects_mode_counts_beyond_its_scratch(shaw):
    torch = pytest.importorskip("torch")
    m = shaw.Mesh.load(mesh_dir("fullMesh21x51"))
    m.set_material("unilayer", [2000.0, 0.0, 0.0, 5000.0, 0.0, 0.0])
    fom = shaw.Fom(m, 1, 1)
    d = torch.zeros(8, dtype=torch.float64, device="cuda:0")
    p = ctypes.c_void_p(d.data_ptr())
    rc = shaw.lib().shaw_rom_project_noalloc(fom.h, p, 65536, p, 1, p, p, None)
    assert rc == shaw.ERR_INVALID_ARG
    assert "65535" in shaw.lib().shaw_last_error().decode()
    fom.close()
