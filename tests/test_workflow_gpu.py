"""The reference's FOM -> POD -> ROM workflow through the drop-in executables.

  shaw_exe fom.yaml          (snapshots snaps_vp_0 / snaps_sp_0, binary)
  computeThinSVD --dirs ...  (lsv_vp / lsv_sp, sva_vp / sva_sp)
  shaw_exe rom.yaml          (rom section: numModes + modesFile = lsv_*; reduced snapshots)

The reduced snapshots must equal the oracle's ROM (oracle projection of the same basis,
oracle leapfrog) to 1e-12; the POD basis must reproduce numpy's thin SVD of the FOM
snapshots (up to signs).
"""
import os
import struct
import subprocess

import numpy as np
import pytest

from conftest import mesh_dir

pytestmark = pytest.mark.gpu

MAT = "material:\n  kind: unilayer\n  layer: {density: [2000., 0.], velocity: [5000., 0.]}\n"


def _general(final):
    return ("general:\n  meshDir: %s\n  dt: 1.\n  finalTime: %s\n  checkNumericalDispersion: false\n"
            "  checkCfl: false\n" % (mesh_dir("fullMesh21x51"), final))


def _snaps(freq):
    return ("io:\n snapshotMatrix:\n   binary: true\n   velocity: {freq: %d, fileName: snaps_vp}\n"
            "   stress:   {freq: %d, fileName: snaps_sp}\n" % (freq, freq))


def _read(path):
    with open(path, "rb") as f:
        r, c = struct.unpack("<QQ", f.read(16))
        return np.frombuffer(f.read(), "<f8").reshape((r, c), order="F")


def _run(cmd, cwd):
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout[-2000:]
    return r.stdout


def test_fom_pod_rom_workflow(shaw, oracle, tmp_path):
    fom_dir, pod_dir = tmp_path / "fom", tmp_path / "pod"
    fom_dir.mkdir()
    pod_dir.mkdir()
    (fom_dir / "fom.yaml").write_text(
        _general(600.) + _snaps(2) +
        "source:\n  signal: {kind: ricker, depth: 900.0, angle: 60., period: 45., delay: 10.0}\n" + MAT)
    _run([shaw.EXE_PATH, "fom.yaml"], fom_dir)
    snaps_v = _read(fom_dir / "snaps_vp_0")
    snaps_s = _read(fom_dir / "snaps_sp_0")
    assert snaps_v.shape[1] == 300

    out = _run([shaw.POD_EXE_PATH, "--dirs", str(fom_dir), "--informat", "binary", "--outformat", "binary",
                "--method", "2"], pod_dir)
    assert "Done with SVD" in out
    phi_v, phi_s = _read(pod_dir / "lsv_vp"), _read(pod_dir / "lsv_sp")
    sv_v = np.array([float(x) for x in (pod_dir / "sva_vp").read_text().split()])
    u, s, _ = np.linalg.svd(snaps_v, full_matrices=False)
    np.testing.assert_allclose(sv_v, s, rtol=0, atol=1e-13 * s[0])
    # well-determined leading modes (above the snapshots' numerical rank the vectors are
    # arbitrary): sigma_i > 1e-6 sigma_1 and separated from both neighbours
    gap = np.minimum(np.abs(np.diff(s, prepend=np.inf)), np.abs(np.diff(s, append=0.0))) / s[0]
    good = (s > 1e-6 * s[0]) & (gap > 1e-4)
    assert good[:10].all()
    dots = np.abs(np.sum(phi_v * u, axis=0))
    assert np.max(np.abs(dots[good] - 1)) < 1e-8
    k = 20  # within the numerical rank of 300 single-source snapshots

    (pod_dir / "rom.yaml").write_text(
        _general(600.) + _snaps(5) +
        "source:\n  signal: {kind: ricker, depth: 1300.0, angle: 100., period: 50., delay: 10.0}\n" + MAT +
        "rom:\n  velocity: {numModes: %d, modesFile: lsv_vp, binary: true}\n"
        "  stress: {numModes: %d, modesFile: lsv_sp, binary: true}\n" % (k, k))
    _run([shaw.EXE_PATH, "rom.yaml"], pod_dir)
    red_v, red_s = _read(pod_dir / "snaps_vp_0"), _read(pod_dir / "snaps_sp_0")
    assert red_v.shape == (k, 120) and red_s.shape == (k, 120)

    om = oracle.OracleMesh(mesh_dir("fullMesh21x51"))
    om.set_material("unilayer", [([2000.0, 0.0, 0.0], [5000.0, 0.0, 0.0])])
    pv, ps = np.asfortranarray(phi_v[:, :k]), np.asfortranarray(phi_s[:, :k])
    av, as_ = om.rom_operators(pv, ps)
    b = om.rom_forcing_vector(pv, om.map_source(1300.0, 100.0))
    ref = oracle.rom_run(av, as_, b.reshape(-1, 1), 600, 1.0, [0], [50.0], [10.0], 5, 5)
    scale = np.max(np.abs(ref["snaps_vp"]))
    assert scale > 0
    assert np.max(np.abs(red_v - ref["snaps_vp"][:, :, 0])) <= 1e-12 * scale
    assert np.max(np.abs(red_s - ref["snaps_sp"][:, :, 0])) <= 1e-12 * np.max(np.abs(ref["snaps_sp"]))
