"""Pin the CPU oracle to the reference's own golden values (CPU only).

Golds come from the reference's test tree (tests/golden/make_fixtures.py): the
CRS Jacobians, graphs, coordinates, labels, mapped gids of its unit tests, and
the snapshot/seismogram files of its regression tests (atol 1e-13 for vp, 1e-10
for sp in the reference's compare.py; the oracle is held to 1e-12 relative).
"""
import json
import os

import numpy as np
import pytest

from cases import CASES, as_text_layout, parse_case, run_case
from conftest import GOLDEN, mesh_dir
from oracle_lib import reference_root

UNIT = json.load(open(os.path.join(GOLDEN, "unit_golds.json")))
REF_TESTS = os.path.join(reference_root(), "tests")


def _mesh(oracle, name, rho=1.0, vs=1.0):
    m = oracle.OracleMesh(mesh_dir(name))
    m.set_material("unilayer", [([rho, 0.0], [vs, 0.0])])
    return m


def test_jacobian_vp_gold(oracle):
    m = _mesh(oracle, "fullMesh4x5")
    ptr, ind, val = m.crs(0)
    g = UNIT["jacobian_vp"]
    assert np.array_equal(np.diff(ptr), g["nnz_per_row"])
    for r in range(m.nvp):
        cols = ind[ptr[r]:ptr[r + 1]]
        vals = val[ptr[r]:ptr[r + 1]]
        assert list(cols) == g["col_ind"][r]
        assert np.max(np.abs(vals - np.array(g["values"][r]))) <= 1e-13


def test_jacobian_sp_gold(oracle):
    m = _mesh(oracle, "fullMesh4x5")
    ptr, ind, val = m.crs(1)
    g = UNIT["jacobian_sp"]
    assert np.all(np.diff(ptr) == 2)
    assert ind.reshape(-1, 2).tolist() == g["col_ind"]
    assert np.max(np.abs(val.reshape(-1, 2) - np.array(g["values"]))) <= 1e-13


def test_graphs_coords_labels_gold(oracle):
    g = _mesh(oracle, "fullMesh4x5").graph()
    assert g["gvp"][:, 1:].tolist() == UNIT["graphs"]["vp"]
    assert np.array_equal(g["gvp"][:, 0], np.arange(len(g["gvp"])))
    assert g["gsp"][:, 1:].tolist() == UNIT["graphs"]["sp"]
    assert g["labels"].tolist() == UNIT["stress_labels"]
    c = _mesh(oracle, "nonPhysicalFullMesh5x5").graph()
    for dof, key in (("coords_vp", "vp"), ("coords_sp", "sp")):
        gold = np.array(UNIT["coords"][key])
        assert np.max(np.abs(c[dof][:, 0] - gold[:, 0])) <= 1e-13
        assert np.max(np.abs(c[dof][:, 1] - 1.0 / (gold[:, 1] * 1000.0))) <= 1e-13


def test_mesh_info_gold(oracle):
    m = _mesh(oracle, "fullMesh21x51", 2000.0, 5000.0)
    i = m.info
    vals = {"meshInfo.getAngularSpacing()": i[4], "meshInfo.getRadialSpacing()": i[5],
            "meshInfo.getAngularSpacingInverse()": i[6], "meshInfo.getRadialSpacingInverse()": i[7],
            "meshInfo.getMinRadius()": i[2], "meshInfo.getMinRadiusKm()": i[2] / 1000.0,
            "meshInfo.getMaxRadius()": i[3], "meshInfo.getMaxRadiusKm()": i[3] / 1000.0,
            "meshInfo.getMinArc()": i[12], "meshInfo.getMaxArc()": i[13],
            "db[0]": i[0], "db[1]": i[1], "db[2]": i[2], "db[3]": i[3]}
    for expr, gold in UNIT["meshInfo"]["checks"]:
        assert abs(vals[expr] - float(gold)) <= 1e-10, expr
    counts = {"getNumPtsAlongR": m.nr, "getNumPtsAlongTheta": m.nth, "getNumVpPts": m.nvp, "getNumSpPts": m.nsp}
    for k, v in UNIT["meshInfo"]["counts"]:
        assert counts[k] == int(v)


def test_mapped_gids_gold(oracle):
    m = _mesh(oracle, "fullMesh21x51", 2000.0, 5000.0)
    # tests/seismogram/input.yaml: receivers [25, 50, 120, 160]
    assert [m.map_receiver(a) for a in (25, 50, 120, 160)] == UNIT["seismogram_gids"]
    # tests/forcing_rank1/input.yaml: depth 1111 km, angle 88 deg, period 25 s
    assert m.map_source(1111.0, 88.0) == UNIT["forcing_rank1"]["gid"]
    assert 1.0 / 25.0 == UNIT["forcing_rank1"]["max_freq"]


GOLDS = np.load(os.path.join(GOLDEN, "regression_golds.npz"))
PRINTS = json.load(open(os.path.join(GOLDEN, "regression_fingerprints.json")))


def _compare_gold(key, mine):
    """Our (rows x T) array against a stored gold: all values, or the fingerprint."""
    hdr = PRINTS["_headers"][key]
    if key in GOLDS.files:
        gold = GOLDS[key]
        assert gold.shape == mine.shape
        scale = np.abs(gold).max()
        assert np.max(np.abs(mine - gold)) <= 1e-12 * scale + 1e-300
        tol = 1e-10 if "snaps_sp" in key else 1e-13
        assert np.allclose(mine, gold, atol=tol, rtol=0)
        return hdr
    fp = PRINTS[key]
    scale = max(np.max(fp["colmax"]), 1e-300)
    assert np.allclose(mine.sum(axis=0), fp["colsum"], rtol=0, atol=1e-11 * scale * mine.shape[0])
    assert np.allclose((mine * mine).sum(axis=0), fp["colsq"], rtol=1e-10, atol=1e-24)
    assert np.allclose(np.abs(mine).max(axis=0), fp["colmax"], rtol=1e-12, atol=1e-300)
    assert np.allclose(mine.ravel()[::97], fp["sample"], rtol=0, atol=1e-12 * scale)
    return hdr


@pytest.mark.parametrize("case", CASES)
def test_regression_case_gold(oracle, case):
    c = parse_case(case)
    m = oracle.OracleMesh(mesh_dir(c["mesh"]))
    m.set_material("unilayer", [([2000.0, 0.0], [5000.0, 0.0])])
    runs = run_case(m, c)
    rank = 1 if c["forcing_size"] is None else 2
    checked = 0
    for rid, out in runs.items():
        for name, arr in (("snaps_vp", out["snaps_vp"]), ("snaps_sp", out["snaps_sp"]), ("seismogram", out["seis"])):
            key = "%s/%s_%d_gold" % (case, name, rid)
            if key not in PRINTS["_headers"]:
                continue
            mine = as_text_layout(arr, rank)
            if name == "seismogram":
                gold = GOLDS[key]
                # the reference's compare.py drops the first line of files without a header
                assert np.allclose(mine[1:], gold[1:] if gold.shape[0] == mine.shape[0] else gold, atol=1e-13,
                                   rtol=0) or np.allclose(mine, gold, atol=1e-13, rtol=0)
                assert np.max(np.abs(mine - gold)) <= 1e-12 * np.abs(gold).max()
            else:
                hdr = _compare_gold(key, mine)
                assert hdr == list(arr.shape[:2]) + ([arr.shape[2]] if rank == 2 else [])
            checked += 1
    if case in ("fomNearCmb", "fomSymmetryAxisThetaPi", "fomSymmetryAxisThetaZero"):
        assert checked == 0  # their golds are missing blobs in the reference tree
    else:
        assert checked > 0


@pytest.mark.skipif(not os.path.isdir(REF_TESTS), reason="reference tree not present")
def test_every_reference_gold_file(oracle):
    """Where the reference tree exists, compare against every raw gold file in full."""
    from cases import read_output
    n = 0
    for case in CASES:
        c = parse_case(case)
        m = oracle.OracleMesh(mesh_dir(c["mesh"]))
        m.set_material("unilayer", [([2000.0, 0.0], [5000.0, 0.0])])
        runs = run_case(m, c)
        rank = 1 if c["forcing_size"] is None else 2
        for rid, out in runs.items():
            for name, arr in (("snaps_vp", out["snaps_vp"]), ("snaps_sp", out["snaps_sp"]),
                              ("seismogram", out["seis"])):
                f = os.path.join(REF_TESTS, case, "%s_%d_gold" % (name, rid))
                if not os.path.exists(f):
                    continue
                _, gold = read_output(f, name != "seismogram")
                mine = as_text_layout(arr, rank)
                assert np.max(np.abs(mine - gold)) <= 1e-12 * np.abs(gold).max(), f
                n += 1
    assert n >= 60


def test_oracle_mesher_writes_reference_mesh_files_byte_for_byte(oracle):
    """The oracle's own restatement of the mesher (used where the product library must not
    be loaded, e.g. the benchmark's reference arm) against the reference mesher's files."""
    import hashlib
    import tempfile
    digests = json.load(open(os.path.join(GOLDEN, "mesh_sha256.json")))
    for name, info in digests.items():
        with tempfile.TemporaryDirectory() as d:
            oracle.write_full_mesh(info["nth"], info["nr"], d, info["thL"], info["thR"], info["rCmb"], info["rSurf"])
            for f in ("mesh_info.dat", "graph_vp.dat", "graph_sp.dat", "coeff_vp.dat"):
                h = hashlib.sha256(open(os.path.join(d, f), "rb").read()).hexdigest()
                assert h == info[f], (name, f)
