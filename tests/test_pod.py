"""POD (computeThinSVD, src/tools/main_eigen_svd.cc) parity.

The golden outputs under tests/golden/pod/ were written by the reference's own tool,
compiled from the reference sources (tests/golden/make_pod_golden.py).  CPU tests pin
them against numpy's LAPACK SVD; GPU tests compare shaw_pod and the computeThinSVD
drop-in executable with them.  Singular vectors are compared up to their sign.
"""
import os
import struct
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

POD = os.path.join(GOLDEN, "pod")
# FP64 SVD of matrices with condition number 1e5: singular values agree to a few ulp of
# sigma_max; singular vectors u_i to ~eps * sigma_max / gap_i.
SV_TOL = 1e-13
VEC_TOL = 1e-9


def read_binary(path):
    with open(path, "rb") as f:
        rows, cols = struct.unpack("<QQ", f.read(16))
        a = np.frombuffer(f.read(), dtype="<f8")
    assert a.size == rows * cols
    return a.reshape((rows, cols), order="F")


def read_sva(path):
    with open(path) as f:
        txt = f.read()
    return txt, np.array([float(x) for x in txt.split()])


def snapshots(case, dof):
    runs = sorted(d for d in os.listdir(os.path.join(POD, case)) if d.startswith("run"))
    return np.hstack([read_binary(os.path.join(POD, case, r, "snaps_%s_0" % dof)) for r in runs])


def golden(case, method, dof):
    d = os.path.join(POD, case, "method%d" % method)
    return read_binary(os.path.join(d, "lsv_" + dof)), read_sva(os.path.join(d, "sva_" + dof))[1]


def assert_same_basis(u, s, u_ref, s_ref):
    assert u.shape == u_ref.shape
    np.testing.assert_allclose(s, s_ref, rtol=0, atol=SV_TOL * s_ref[0])
    dots = np.abs(np.sum(u * u_ref, axis=0))
    assert np.max(np.abs(dots - 1.0)) < VEC_TOL, dots
    k = u.shape[1]
    assert np.max(np.abs(u.T @ u - np.eye(k))) < 1e-13


GOLD_CASES = [("tall", 1), ("tall", 2), ("wide", 1)]


@pytest.mark.parametrize("case,method", GOLD_CASES)
@pytest.mark.parametrize("dof", ["vp", "sp"])
def test_golden_matches_numpy_svd(case, method, dof):
    """Pin: the reference tool's output is the thin SVD (numpy/LAPACK) of the concatenated snapshots."""
    a = snapshots(case, dof)
    u_ref, s_ref = golden(case, method, dof)
    u, s, _ = np.linalg.svd(a, full_matrices=False)
    assert_same_basis(u, s, u_ref, s_ref)


def test_golden_sva_text_layout():
    """Eigen prints the singular values one per line, right-aligned to the widest, 17 digits."""
    txt, vals = read_sva(os.path.join(POD, "wide", "method1", "sva_vp"))
    lines = txt.split("\n")
    assert lines[-1] == "" and len(lines) == vals.size + 1
    assert len(set(len(x) for x in lines[:-1])) == 1


# ---- GPU --------------------------------------------------------------------


@pytest.mark.gpu
@pytest.mark.parametrize("case,method", GOLD_CASES)
@pytest.mark.parametrize("dof", ["vp", "sp"])
def test_pod_vs_reference_tool(shaw, case, method, dof):
    a = snapshots(case, dof)
    u_ref, s_ref = golden(case, method, dof)
    u, s = shaw.pod(a, method=method)
    assert_same_basis(u, s, u_ref, s_ref)


def _tool():
    import shaw_gb300
    return shaw_gb300.POD_EXE_PATH


@pytest.mark.gpu
@pytest.mark.parametrize("case,method", GOLD_CASES)
def test_pod_executable_drop_in(shaw, tmp_path, case, method):
    """computeThinSVD --dirs run0 run1 --informat binary --outformat binary --method m."""
    runs = sorted(os.path.join(POD, case, d) for d in os.listdir(os.path.join(POD, case)) if d.startswith("run"))
    r = subprocess.run([_tool(), "--dirs", *runs, "--informat", "binary", "--outformat", "binary",
                        "--method", str(method)], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "Final snapshot matrix size" in r.stdout
    for dof in ("vp", "sp"):
        u_ref, s_ref = golden(case, method, dof)
        txt, s = read_sva(os.path.join(tmp_path, "sva_" + dof))
        lines = txt.split("\n")
        assert lines[-1] == "" and len(lines) == s.size + 1
        assert len(set(len(x) for x in lines[:-1])) == 1
        u = read_binary(os.path.join(tmp_path, "lsv_" + dof))
        assert_same_basis(u, s, u_ref, s_ref)


@pytest.mark.gpu
def test_pod_executable_errors(shaw, tmp_path):
    runs = [os.path.join(POD, "tall", d) for d in ("run0", "run1")]
    exe = _tool()
    # missing --method: "Invalid method" (main_eigen_svd.cc:298-300)
    r = subprocess.run([exe, "--dirs", *runs, "--informat", "binary", "--outformat", "binary"],
                       cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode != 0 and "Invalid method" in r.stderr
    # the reader receives --outformat (main_eigen_svd.cc:302): non-binary -> empty matrix -> error
    r = subprocess.run([exe, "--dirs", *runs, "--informat", "binary", "--outformat", "ascii", "--method", "2"],
                       cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode != 0 and "empty snapshot matrix" in r.stderr
    # and --informat is not consulted
    r = subprocess.run([exe, "--dirs", *runs, "--informat", "ascii", "--outformat", "binary", "--method", "2"],
                       cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # mismatching rows across directories
    r = subprocess.run([exe, "--dirs", runs[0], os.path.join(POD, "wide", "run0"), "--informat", "binary",
                        "--outformat", "binary", "--method", "1"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode != 0 and "Mismatching # rows" in r.stderr


@pytest.mark.gpu
def test_pod_api_errors(shaw):
    a = np.ones((4, 6))
    with pytest.raises(shaw.ShawError):
        shaw.pod(a, method=2)  # QR route needs n >= t
    with pytest.raises(shaw.ShawError):
        shaw.pod(np.ones((6, 4)), method=3)
    with pytest.raises(shaw.ShawError):
        shaw.pod(np.ones((0, 4)), method=1)


@pytest.mark.gpu
@pytest.mark.parametrize("n,t,method", [(1, 1, 1), (7, 1, 2), (1, 5, 1), (33, 33, 2), (300, 37, 1)])
def test_pod_ragged_shapes(shaw, n, t, method):
    rng = np.random.default_rng(n * 1000 + t)
    a = rng.standard_normal((n, t))
    u, s = shaw.pod(a, method=method)
    u_np, s_np, _ = np.linalg.svd(a, full_matrices=False)
    np.testing.assert_allclose(s, s_np, rtol=0, atol=1e-13 * s_np[0])
    k = min(n, t)
    assert u.shape == (n, k)
    assert np.max(np.abs(u.T @ u - np.eye(k))) < 1e-12
    # reconstruction through the computed basis: A = U U^T A
    assert np.max(np.abs(u @ (u.T @ a) - a)) < 1e-12 * s_np[0]


@pytest.mark.gpu
def test_pod_fom_snapshots_large(shaw):
    """Snapshot matrix at POD scale (20,301 vp rows x 400 snapshots): orthonormal basis,
    singular values equal to numpy's, snapshots reproduced by the basis."""
    rng = np.random.default_rng(7)
    n, t = 20301, 400
    a = rng.standard_normal((n, 24)) @ (rng.standard_normal((24, t)) * 10.0 ** -np.arange(24)[:, None] / 4)
    a += 1e-9 * rng.standard_normal((n, t))
    u, s = shaw.pod(a, method=2)
    s_np = np.linalg.svd(a, compute_uv=False)
    np.testing.assert_allclose(s, s_np, rtol=0, atol=1e-13 * s_np[0])
    assert np.max(np.abs(u.T @ u - np.eye(t))) < 1e-12
    assert np.max(np.abs(u[:, :24] @ (u[:, :24].T @ a) - a)) < 1e-7 * s_np[0]
