"""Regenerate the golden fixtures under tests/golden/ from the reference tree.

Reads the reference project's own test data as text (mesh fixtures, input files,
gold snapshot/seismogram files, and the gold values spelled out in its unit-test
sources) and writes compact copies here, so the tests run where the reference
tree is absent.  Usage:

    python tests/golden/make_fixtures.py [REFERENCE_ROOT]

REFERENCE_ROOT defaults to $SHAW_REFERENCE_ROOT (tests/oracle_lib.py:reference_root).
"""
import hashlib
import json
import os
import re
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

COPY_MESHES = ["fullMesh4x5", "nonPhysicalFullMesh5x5", "fullMesh21x51"]
HASH_MESHES = ["fullMesh50x200", "fullMesh101x201", "fullMesh21x51", "fullMesh4x5", "nonPhysicalFullMesh5x5"]
MESH_FILES = ["mesh_info.dat", "graph_vp.dat", "graph_sp.dat", "coeff_vp.dat"]
CASES = ["fomInnerDomain", "fomNearEarthSurface", "fomNearCmb", "fomSymmetryAxisThetaPi",
         "fomSymmetryAxisThetaZero", "multiDepthsForcingRank1", "multiPeriodsForcingRank1",
         "multiDepthsAndPeriodsForcingRank1", "multiDepthsForcingRank2", "multiPeriodsForcingRank2",
         "multiDepthsAndPeriodsForcingRank2"]
# gold files stored with every value (the rest are stored as fingerprints)
FULL = {("fomInnerDomain", "snaps_vp_0_gold"),
        ("multiDepthsAndPeriodsForcingRank2", "snaps_vp_0_gold"),
        ("multiDepthsAndPeriodsForcingRank2", "snaps_sp_0_gold")}
UNIT_INPUTS = {"jacobian_vp": "input.yaml", "jacobian_sp": "input.yaml", "seismogram": "input.yaml",
               "forcing_rank1": "input.yaml", "meshInfo": "input.yaml"}


def load_gold(path):
    """A gold text file: optional size header line + rows of numbers."""
    with open(path) as f:
        lines = [ln for ln in f.read().split("\n") if ln.strip()]
    return lines


def fingerprint(a):
    """Per-column (time sample) sums that pin a snapshot matrix without all its values."""
    a = np.asarray(a, np.float64)
    return dict(colsum=a.sum(axis=0).tolist(), colsq=(a * a).sum(axis=0).tolist(),
                colmax=np.abs(a).max(axis=0).tolist(), sample=a.ravel()[::97].tolist())


def cxx_numbers(text):
    return [float(x) for x in re.findall(r"[-+]?\d+\.?\d*(?:[eE][-+]?\d+)?", text)]


def block(src, name):
    """The brace initializer following `name =` in a C++ source."""
    i = src.index(name)
    j = src.index("{", i)
    depth = 0
    for k in range(j, len(src)):
        if src[k] == "{":
            depth += 1
        elif src[k] == "}":
            depth -= 1
            if depth == 0:
                return src[j:k + 1]
    raise ValueError(name)


def rows_of(init):
    """Split a nested initializer {{..},{..}} into rows of numbers."""
    inner = init.strip()[1:-1]
    return [cxx_numbers(r) for r in re.findall(r"\{([^{}]*)\}", inner)]


def main(ref):
    tests = os.path.join(ref, "tests")
    meshes = os.path.join(HERE, "meshes")
    os.makedirs(meshes, exist_ok=True)
    for m in COPY_MESHES:
        dst = os.path.join(meshes, m)
        os.makedirs(dst, exist_ok=True)
        for f in MESH_FILES:
            shutil.copyfile(os.path.join(tests, m, f), os.path.join(dst, f))
    digests = {}
    for m in HASH_MESHES:
        info = {}
        for f in MESH_FILES:
            with open(os.path.join(tests, m, f), "rb") as fh:
                info[f] = hashlib.sha256(fh.read()).hexdigest()
        with open(os.path.join(tests, m, "mesh_info.dat")) as fh:
            kv = dict(ln.split()[:2] for ln in fh if ln.strip())
        info["nth"], info["nr"] = int(kv["nth"]), int(kv["nr"])
        info["thL"], info["thR"] = float(kv["thL"]), float(kv["thR"])
        info["rCmb"], info["rSurf"] = float(kv["rCmb"]), float(kv["rSurf"])
        digests[m] = info
    with open(os.path.join(HERE, "mesh_sha256.json"), "w") as fh:
        json.dump(digests, fh, indent=1, sort_keys=True)

    # regression cases: inputs + golds
    cases_dir = os.path.join(HERE, "cases")
    os.makedirs(cases_dir, exist_ok=True)
    arrays = {}
    prints = {}
    for c in CASES:
        d = os.path.join(cases_dir, c)
        os.makedirs(d, exist_ok=True)
        shutil.copyfile(os.path.join(tests, c, "input.yaml"), os.path.join(d, "input.yaml"))
        for f in sorted(os.listdir(os.path.join(tests, c))):
            if not f.endswith("_gold"):
                continue
            lines = load_gold(os.path.join(tests, c, f))
            has_header = not f.startswith("seismogram")
            header = [int(x) for x in lines[0].split()] if has_header else []
            body = np.array([[float(x) for x in ln.split()] for ln in lines[1 if has_header else 0:]])
            key = c + "/" + f
            if f.startswith("seismogram") or (c, f) in FULL:
                arrays[key] = body
            else:
                prints[key] = fingerprint(body)
            prints.setdefault("_headers", {})[key] = header
    np.savez_compressed(os.path.join(HERE, "regression_golds.npz"), **arrays)
    with open(os.path.join(HERE, "regression_fingerprints.json"), "w") as fh:
        json.dump(prints, fh)

    # unit-test golds spelled out in the reference's test sources
    unit = {}
    src = open(os.path.join(tests, "jacobian_vp", "main.cc")).read()
    host = src[src.index("HostSpace>::value\n  >::type\nrunTest"):]
    unit["jacobian_vp"] = dict(
        nnz_per_row=[int(x) for x in cxx_numbers(block(host, "goldNNZPerRow"))],
        col_ind=[[int(x) for x in r] for r in rows_of(block(host, "goldColIndPerRow"))],
        values=rows_of(block(host, "goldValPerRow")))
    src = open(os.path.join(tests, "jacobian_sp", "main.cc")).read()
    host = src[src.index("HostSpace>::value\n  >::type\nrunTest"):]
    unit["jacobian_sp"] = dict(
        col_ind=[[int(x) for x in r] for r in rows_of(block(host, "goldColIndPerRow"))],
        values=rows_of(block(host, "goldValPerRow")))
    src = open(os.path.join(tests, "graphs", "main.cc")).read()
    unit["graphs"] = dict(vp=[[int(x) for x in r] for r in rows_of(block(src, "goldGVp"))],
                          sp=[[int(x) for x in r] for r in rows_of(block(src, "goldGSp"))])
    src = open(os.path.join(tests, "coords", "main.cc")).read()
    unit["coords"] = dict(vp=rows_of(block(src, "goldVp")), sp=rows_of(block(src, "goldSp")))
    src = open(os.path.join(tests, "stress_labels", "main.cc")).read()
    unit["stress_labels"] = [int(x) for x in cxx_numbers(block(src, "goldLabels"))]
    src = open(os.path.join(tests, "seismogram", "main.cc")).read()
    unit["seismogram_gids"] = [int(x) for x in re.findall(r"gids\(\d\) != (\d+)", src)]
    src = open(os.path.join(tests, "forcing_rank1", "main.cc")).read()
    unit["forcing_rank1"] = dict(max_freq=float(re.search(r"getMaxFreq\(\) != ([\d.]+)", src).group(1)),
                                 gid=int(re.search(r"getVpGid\(\) != (\d+)", src).group(1)))
    src = open(os.path.join(tests, "meshInfo", "main.cc")).read()
    unit["meshInfo"] = dict(
        checks=re.findall(r"std::abs\(([\w.]*\(\))\s*-\s*([\d.]+)\)", src)
        + re.findall(r"std::abs\((db\[\d\])\s*-\s*([\d.]+)\)", src),
        counts=re.findall(r"meshInfo\.(\w+)\(\) != (\d+)", src))
    # the mesh dirs these unit tests read
    for t in ["graphs", "coords", "stress_labels", "jacobian_vp", "jacobian_sp", "seismogram", "forcing_rank1",
              "meshInfo"]:
        y = open(os.path.join(tests, t, "input.yaml")).read()
        unit.setdefault("inputs", {})[t] = y
    # parser tests: (expression, expected) pairs
    unit["parser"] = {}
    for i in range(1, 7):
        src = open(os.path.join(tests, "parser", "main%d.cc" % i)).read()
        pairs = re.findall(r"vb\.push_back\((.*?)\s*==\s*(.*?)\s*\);", src)
        gold_angles = re.search(r"goldAngles = \{([^}]*)\}", src)
        unit["parser"]["input%d" % i] = dict(
            yaml=open(os.path.join(tests, "parser", "input%d.yaml" % i)).read(),
            checks=pairs, gold_angles=cxx_numbers(gold_angles.group(1)) if gold_angles else None)
    with open(os.path.join(HERE, "unit_golds.json"), "w") as fh:
        json.dump(unit, fh, indent=1)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(HERE))
    from oracle_lib import reference_root
    main(sys.argv[1] if len(sys.argv) > 1 else reference_root())
