"""Generate the thermodynamics golden fixtures under tests/golden/ from the real reference.

Run in the build container (the reference tree is not on the GPU host):
    bash oracle/build_ref.sh && python tests/golden/make_thermo_golden.py

For each case the unmodified reference NRG_main runs twice in one directory,
as its documentation prescribes for the impurity susceptibility and entropy:
first with calc_density = 3 (the free Wilson chain; NRG_main switches to
ModelNo 3 and writes SuscepChain*.dat / EntropyChain*.dat), then with
calc_density = 2 (the impurity sweep, which reads the chain files back and
writes Suscep*.dat / Entropy*.dat with the chain subtracted).  The fixture
keeps the four columns of every file at full precision.  The two-channel
Anderson impurity is not among NRG_main's models (the two-channel files come
from its Kondo model), so the two-channel case keeps the chain files only.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
NRG_MAIN = os.path.join(REPO, "oracle", "_ref", "NRG_main")

# name: (NRG_main -m option, nsites, ncutoff, U, Gamma, ed, Lambda, extra line or None,
#        chain file stem, impurity file stem or None)
CASES = {
    "thermo_1chQS_n14_k150": ("Anderson", 14, 150, 0.5, 0.02, -0.25, 2.5, None,
                              "Chain1Ch_QS_zEQ1", "Imp1ChQS_Anderson_zEQ1"),
    "thermo_1chQSz_n12_k200": ("1chQSz_Anderson", 12, 200, 0.4, 0.015, -0.2, 2.5, 1.0e-4,
                               "Chain1Ch_QSz_zEQ1", "Imp1ChQSz_zEQ1"),
    "thermo_2chQS_chain_n8_k300": ("2chQS_Kondo", 8, 300, 0.3, 0.01, -0.15, 2.5, None,
                                   "Chain2Ch_QS_zEQ1", None),
    # |Q> symmetry: entropy only, files without the z-string
    "thermo_1chQ_n10_k150": ("1chQ_Anderson", 10, 150, 0.5, 0.02, -0.25, 2.5, None,
                             "Chain1Ch_Q", "Imp1Ch_Anderson_Q"),
}


def _input(d, ns, nc, U, G, ed, lam, extra, calcdens):
    with open(os.path.join(d, "input_nrg.dat"), "w") as f:
        # Nsitesmax, Ncutoff, U, Gamma, ed, Lambda, ChemPot, (unused), UpdateBefCut,
        # calc_density, separator, model parameters beyond the first three
        f.write(f"{ns}\n{nc}\n{U!r}\n{G!r}\n{ed!r}\n{lam!r}\n0\n0\n0\n{calcdens}\n9999999\n")
        if extra is not None:
            f.write(f"{extra!r}\n")


def run_case(opt, ns, nc, U, G, ed, lam, extra, chain, imp) -> dict:
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1")
    out = {"config": np.array([ns, nc, U, G, ed, lam, 0.0 if extra is None else extra], dtype=np.float64)}
    with tempfile.TemporaryDirectory() as d:
        _input(d, ns, nc, U, G, ed, lam, extra, 3)
        subprocess.run([NRG_MAIN, "-m", opt], cwd=d, check=True, capture_output=True, env=env)
        for kind in ("Suscep", "Entropy"):
            p = os.path.join(d, f"{kind}{chain}.dat")
            if os.path.exists(p):
                out[f"chain_{kind.lower()}"] = np.loadtxt(p)
        if imp is not None:
            _input(d, ns, nc, U, G, ed, lam, extra, 2)
            subprocess.run([NRG_MAIN, "-m", opt], cwd=d, check=True, capture_output=True, env=env)
            for kind in ("Suscep", "Entropy"):
                p = os.path.join(d, f"{kind}{imp}.dat")
                if os.path.exists(p):
                    out[f"imp_{kind.lower()}"] = np.loadtxt(p)
    return out


def main() -> None:
    if not os.path.exists(NRG_MAIN):
        sys.exit("build the reference first: bash oracle/build_ref.sh")
    only = sys.argv[1:]
    for name, case in CASES.items():
        if only and name not in only:
            continue
        d = run_case(*case)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(name, {k: v.shape for k, v in d.items()})


if __name__ == "__main__":
    main()
