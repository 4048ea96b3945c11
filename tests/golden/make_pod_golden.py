"""Regenerates tests/golden/pod/: snapshot directories and the reference POD tool's outputs.

The snapshot matrices are synthetic, seeded, with prescribed well-separated singular
values (so every singular vector is well conditioned and can be compared up to sign):

  tall : vp 48 rows, sp 80 rows; run0 holds 7 snapshots, run1 holds 5 (t = 12)
  wide : vp 10 rows, sp 9 rows; run0 holds 8 snapshots, run1 holds 6 (t = 14, n < t)

Outputs come from the reference's computeThinSVD (src/tools/main_eigen_svd.cc) compiled
from the reference sources by `make -C oracle ref`:

  tall/method1, tall/method2, wide/method1 : sva_vp, lsv_vp, sva_sp, lsv_sp

Run from the repository root:  python tests/golden/make_pod_golden.py
"""
import os
import shutil
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "pod")
SEED = 20261203

CASES = {
    "tall": {"vp": 48, "sp": 80, "runs": (7, 5)},
    "wide": {"vp": 10, "sp": 9, "runs": (8, 6)},
}


def write_binary(path, a):
    """size_t rows, size_t cols, then the doubles column by column."""
    a = np.asfortranarray(a, np.float64)
    with open(path, "wb") as f:
        f.write(struct.pack("<QQ", *a.shape))
        f.write(a.tobytes(order="F"))


def synthetic(rng, n, t):
    k = min(n, t)
    q1, _ = np.linalg.qr(rng.standard_normal((n, k)))
    q2, _ = np.linalg.qr(rng.standard_normal((t, k)))
    s = 10.0 ** np.linspace(1.0, -4.0, k)
    return (q1 * s) @ q2.T


def main():
    tool = os.path.join(ROOT, "oracle", "_ref", "computeThinSVD")
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    rng = np.random.default_rng(SEED)
    if os.path.isdir(OUT):
        shutil.rmtree(OUT)
    for case, spec in CASES.items():
        base = os.path.join(OUT, case)
        runs = [os.path.join(base, "run%d" % i) for i in range(len(spec["runs"]))]
        for dof in ("vp", "sp"):
            full = synthetic(rng, spec[dof], sum(spec["runs"]))
            c0 = 0
            for d, t in zip(runs, spec["runs"]):
                os.makedirs(d, exist_ok=True)
                write_binary(os.path.join(d, "snaps_%s_0" % dof), full[:, c0:c0 + t])
                c0 += t
        methods = (1, 2) if case == "tall" else (1,)
        for m in methods:
            od = os.path.join(base, "method%d" % m)
            os.makedirs(od)
            rel = [os.path.relpath(d, od) for d in runs]
            subprocess.run([tool, "--dirs", *rel, "--informat", "binary", "--outformat", "binary",
                            "--method", str(m)], cwd=od, check=True, stdout=subprocess.DEVNULL)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
