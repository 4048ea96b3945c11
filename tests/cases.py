"""The reference's regression cases (tests/golden/cases/*/input.yaml) as oracle runs.

parse_case() reads the few input fields the oracle needs with a tiny, test-only
reader (the product parses the same files with its own C++ parser); run_case()
runs the oracle for every realization set the reference would run.
"""
import os
import re

import numpy as np

from conftest import GOLDEN

CASES = ["fomInnerDomain", "fomNearEarthSurface", "fomNearCmb", "fomSymmetryAxisThetaPi",
         "fomSymmetryAxisThetaZero", "multiDepthsForcingRank1", "multiPeriodsForcingRank1",
         "multiDepthsAndPeriodsForcingRank1", "multiDepthsForcingRank2", "multiPeriodsForcingRank2",
         "multiDepthsAndPeriodsForcingRank2"]


def case_yaml(name):
    return os.path.join(GOLDEN, "cases", name, "input.yaml")


def parse_case(name):
    t = open(case_yaml(name)).read()
    t = "\n".join(ln.split("#")[0] for ln in t.splitlines())

    def grab(key):
        m = re.search(r"\b" + key + r"\s*:\s*(\[[^\]]*\]|[^,}\n]+)", t)
        v = m.group(1).strip()
        if v.startswith("["):
            return [float(x) for x in v.strip("[]").split(",") if x.strip()]
        try:
            return [float(v)]
        except ValueError:
            return v
    freqs = [int(x) for x in re.findall(r"freq\s*:\s*(\d+)", t)]
    fs = re.search(r"forcingSize\s*:\s*(\d+)", t)
    c = dict(dt=grab("dt")[0], final=grab("finalTime")[0], kind=grab("kind").strip(),
             depths=grab("depth"), periods=grab("period"), delays=grab("delay"),
             angles=grab("angle") if re.search(r"\bangle\s*:", t) else [0.0],
             receivers=grab("receivers"), freq_vp=freqs[0], freq_sp=freqs[1], freq_seis=freqs[2],
             forcing_size=int(fs.group(1)) if fs else None, mesh=grab("meshDir").strip())
    c["nsteps"] = int(c["final"] / c["dt"])
    c["realizations"] = [(d, p, a, de) for d in c["depths"] for p in c["periods"] for a in c["angles"]
                         for de in c["delays"]]
    return c


def run_case(omesh, c):
    """Oracle outputs per run id: dict(run_id -> dict(snaps_vp, snaps_sp, seis))."""
    import oracle_lib as O
    rcv = [omesh.map_receiver(a) for a in c["receivers"]]
    kind = O.SIGNAL_KINDS[c["kind"]]
    out = {}
    if c["forcing_size"] is None:
        reals = c["realizations"] if len(c["realizations"]) > 1 else c["realizations"][:1]
        for i, (d, p, a, de) in enumerate(reals):
            src = omesh.map_source(d, a)
            out[i] = omesh.fom_run(1, c["nsteps"], c["dt"], [src], [kind], [p], [de], rcv, c["freq_seis"],
                                   c["freq_vp"], c["freq_sp"])
    else:
        M = c["forcing_size"]
        reals = c["realizations"]
        for i in range(len(reals) // M):
            s = reals[i * M:(i + 1) * M]
            src = [omesh.map_source(d, a) for (d, p, a, de) in s]
            out[i] = omesh.fom_run(2, c["nsteps"], c["dt"], src, [kind] * M, [p for (_, p, _, _) in s],
                                   [de for (_, _, _, de) in s], rcv, c["freq_seis"], c["freq_vp"], c["freq_sp"])
    return out


def as_text_layout(a3, rank):
    """The 2-D array a reference ASCII file holds: rank-1 -> (N, T); rank-2 -> stacked (M*N, T)."""
    if rank == 1:
        return a3[:, :, 0]
    return np.concatenate([a3[:, :, k] for k in range(a3.shape[2])], axis=0)


def read_output(path, has_header):
    with open(path) as f:
        lines = [ln for ln in f.read().split("\n") if ln.strip()]
    header = [int(x) for x in lines[0].split()] if has_header else []
    body = np.array([[float(x) for x in ln.split()] for ln in lines[1 if has_header else 0:]])
    return header, body
