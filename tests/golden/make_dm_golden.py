"""Generate the DM-NRG golden fixtures under tests/golden/ from the real reference.

Run in the build container (the reference tree is not on the GPU host):
    bash oracle/build_ref.sh && python tests/golden/make_dm_golden.py

For each case the unmodified reference NRG_main runs the one-channel |Q S>
Anderson model with the spectral density switched on (input_nrg.dat:
UpdateBefCut = 1, calc_density = 1), which saves Abasis/Acut/c_d per shell,
and the unmodified reference DM_NRG then computes the FDM spectral function of
c_d (-F) on its own frequency grid (-n per shell).  The fixture keeps the
inputs and rho_0_0_OmegaRhow.dat's (omega, A) columns at full precision.
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
DM_NRG = os.path.join(REPO, "oracle", "_ref", "DM_NRG")

# name: (nsites, ncutoff, U, Gamma, ed, Lambda, bbroad, nw, Mtemp or -1)
CASES = {
    "dm_1chQS_n10_k60_T0": (10, 60, 0.5, 0.02, -0.25, 2.5, 0.6, 4, -1),
    "dm_1chQS_n10_k60_M6": (10, 60, 0.5, 0.02, -0.25, 2.5, 0.6, 4, 6),
    "dm_1chQS_n16_k150_M12": (16, 150, 0.4, 0.015, -0.2, 2.5, 0.6, 6, 12),
}


def run_case(ns, nc, U, G, ed, lam, b, nw, mtemp) -> dict:
    with tempfile.TemporaryDirectory() as d:
        with open(os.path.join(d, "input_nrg.dat"), "w") as f:
            # Nsitesmax, Ncutoff, U, Gamma, ed, Lambda, Dband, tela,
            # UpdateBefCut, calc_density, separator
            f.write(f"{ns}\n{nc}\n{U!r}\n{G!r}\n{ed!r}\n{lam!r}\n0\n0\n1\n1\n9999999\n")
        env = dict(os.environ, OPENBLAS_NUM_THREADS="1")
        subprocess.run([NRG_MAIN, "-m", "Anderson"], cwd=d, check=True, capture_output=True, env=env)
        args = [DM_NRG, "-F", "-e", repr(b), "-n", str(nw)]
        if mtemp >= 0:
            args += ["-M", str(mtemp)]
        subprocess.run(args, cwd=d, check=True, capture_output=True, env=env)
        data = np.loadtxt(os.path.join(d, "rho_0_0_OmegaRhow.dat"))
    return {"omega": data[:, 0], "A": data[:, 1],
            "config": np.array([ns, nc, U, G, ed, lam, b, nw, mtemp], dtype=np.float64)}


def main() -> None:
    if not (os.path.exists(NRG_MAIN) and os.path.exists(DM_NRG)):
        sys.exit("build the reference first: bash oracle/build_ref.sh")
    only = sys.argv[1:]
    for name, case in CASES.items():
        if only and name not in only:
            continue
        d = run_case(*case)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(name, len(d["omega"]), "frequencies")


if __name__ == "__main__":
    main()
