"""Generate the golden fixtures under tests/golden/ from the real reference.

Run in the build container (the reference tree is not on the GPU host):
    bash oracle/build_ref.sh && python tests/golden/make_golden.py

Two kinds of fixture are written:
  * run1_log.npz      - the eigenvalue lines of the reference's own golden log
                        Runs/run1/output_NRG_test.txt (6 significant digits),
                        with the quantum numbers and Nkept per iteration;
  * <case>.npz        - full-precision outputs of the unmodified reference
                        routines driven by oracle/ref_harness.cpp.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(REPO, "oracle", "_ref", "ref_harness")
# the reference tree: REF_DIR, else the directory "reference" beside the repository
REF = os.environ.get("REF_DIR", os.path.join(os.path.dirname(REPO), "reference"))

# name: (model, nsites, ncutoff, Lambda, U, ed, Gamma1, Gamma2|B[, Delta_SC])
CASES = {
    # Runs/run1 inputs with Gamma rescaled by A_Lambda (the log predates the
    # sqrt(A_Lambda) factor of NRG_main.cpp:205-207).
    "run1_1chQS": ("1chQS", 4, 1000, 2.5, 0.5, -0.25, 0.026444289241359498, 0.0),
    # One-channel Anderson at the headline parameters, full 40-iteration sweep.
    "cfg0_1chQS_n40_k500": ("1chQS", 40, 500, 2.5, 0.5, -0.25, 0.02, 0.0),
    # One-channel Anderson in the (Q,Sz) basis with a magnetic field.
    "qsz_1chQSz_n14_k300": ("1chQSz", 14, 300, 2.5, 0.5, -0.25, 0.02, 1.0e-3),
    # Two-channel Anderson at the headline parameters, reduced kept count.
    "cfg1_2chQS_n8_k300": ("2chQS", 8, 300, 2.5, 0.3, -0.15, 0.01, 0.01),
    "small_2chQS_n5_k60": ("2chQS", 5, 60, 2.5, 0.3, -0.15, 0.01, 0.01),
    # One-channel Anderson in the charge-only |Q> basis (SymNo 3).
    "q_1chQ_n12_k200": ("1chQ", 12, 200, 2.5, 0.5, -0.25, 0.02, 0.0),
    # One-channel Anderson with superconducting leads (Delta_SC = 0.01, the
    # ninth entry) in the |S> basis (SymNo 7) and, with a field, |Sz> (SymNo 8).
    "s_1chS_n12_k200": ("1chS", 12, 200, 2.5, 0.5, -0.25, 0.02, 0.0, 0.01),
    "sz_1chSz_n12_k200": ("1chSz", 12, 200, 2.5, 0.5, -0.25, 0.02, 1.0e-3, 0.01),
}
# The headline two-channel workload at its full kept count, first iterations
# only (iteration 3 is the first at 3000 kept; each takes the reference
# about ten minutes on one core).  Generated only when named on the command
# line: python tests/golden/make_golden.py cfg1_2chQS_n5_k3000
SLOW_CASES = {
    "cfg1_2chQS_n5_k3000": ("2chQS", 5, 3000, 2.5, 0.3, -0.15, 0.01, 0.01),
}


def parse(text: str) -> dict:
    it = []
    opm1 = None
    cur = None
    for line in text.splitlines():
        t = line.split()
        if not t:
            continue
        if t[0] == "OPAVG" and t[1] == "-1":
            opm1 = [float(x) for x in t[3::2]]
            names = t[2::2]
        elif t[0] == "ITER":
            cur = {"params": [float(x) for x in t[2:]], "thermo": []}
            it.append(cur)
        elif t[0] == "BLK":
            nb, nq = int(t[1]), int(t[2])
            v = t[3:]
            q = np.array([[float(v[b * (nq + 1) + k]) for k in range(nq)] for b in range(nb)])
            s = np.array([int(v[b * (nq + 1) + nq]) for b in range(nb)])
            cur["qn"], cur["bsize"] = q, s
        elif t[0] == "EN":
            cur["en"] = np.array([float(x) for x in t[2:]])
        elif t[0] == "CUT":
            cur["ecut"], cur["nkept"] = float(t[1]), int(t[2])
        elif t[0] == "THERMO":
            cur["thermo"].append([float(x) for x in t[2:6]])
        elif t[0] == "OPAVG":
            cur["opavg"] = [float(x) for x in t[3::2]]
        elif t[0] == "KEPTBLK":
            cur["kept_bsize"] = [int(x) for x in t[2:]]
        elif t[0] == "TIME":
            cur["seconds"] = float(t[2])
    out = {"opnames": np.array(names), "opavg_m1": np.array(opm1), "niters": len(it)}
    for n, c in enumerate(it):
        out[f"params_{n}"] = np.array(c["params"])
        out[f"qn_{n}"] = c["qn"]
        out[f"bsize_{n}"] = c["bsize"]
        out[f"en_{n}"] = c["en"]
        out[f"ecut_{n}"] = np.array(c["ecut"])
        out[f"nkept_{n}"] = np.array(c["nkept"])
        out[f"thermo_{n}"] = np.array(c["thermo"])
        out[f"opavg_{n}"] = np.array(c["opavg"])
        out[f"kept_bsize_{n}"] = np.array(c["kept_bsize"])
        if "seconds" in c:  # wall time of the iteration, reference routines on one thread
            out[f"seconds_{n}"] = np.array(c["seconds"])
    return out


def run1_log() -> dict:
    path = os.path.join(REF, "Runs", "run1", "output_NRG_test.txt")
    en, q, s, shell = [], [], [], []
    nk = []
    for line in open(path):
        m = re.match(r"En = (\S+) ---\| (\S+)\s+(\S+)\s+(?:\(K\))?>_N= (\S+)", line)
        if m:
            en.append(float(m.group(1))); q.append(float(m.group(2))); s.append(float(m.group(3)))
            shell.append(int(m.group(4)))
        m = re.match(r"SetKept: Nkept = (\d+)", line)
        if m:
            nk.append(int(m.group(1)))
    return {"en": np.array(en), "q": np.array(q), "s": np.array(s), "shell": np.array(shell),
            "nkept": np.array(nk)}


def main() -> None:
    if not os.path.exists(HARNESS):
        sys.exit("build the reference first: bash oracle/build_ref.sh")
    np.savez_compressed(os.path.join(HERE, "run1_log.npz"), **run1_log())
    only = sys.argv[1:]
    for name, case in {**CASES, **SLOW_CASES}.items():
        if (only and name not in only) or (not only and name in SLOW_CASES):
            continue
        model, ns, nc, lam, U, ed, g1, x = case[:8]
        args = [HARNESS, model, str(ns), str(nc), repr(lam), repr(U), repr(ed), repr(g1), repr(x)]
        args += [repr(v) for v in case[8:]]
        env = dict(os.environ, OPENBLAS_NUM_THREADS="1")
        txt = subprocess.run(args, check=True, capture_output=True, text=True, env=env).stdout
        d = parse(txt)
        d["config"] = np.array(list(case), dtype=object).astype(str)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(name, d["niters"], "iterations")


if __name__ == "__main__":
    main()
