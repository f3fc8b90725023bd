"""Generate the non-flat-band fixtures under tests/golden/ from the real reference.

Run in the build container (the reference tree is not on the GPU host):
    bash oracle/build_ref.sh && python tests/golden/make_chain_golden.py

chain_lanczos.npz: Wilson chains of several bands computed by the unmodified
reference CNRGchain::SetChainLanczos (oracle/ref_harness.cpp, "lanczos" mode;
the GSL quadrature it calls is the accurate stand-in of
oracle/ref_shim/gsl/gsl_integration.h), first 60 of 100 sites.

chain_<model>_<case>.npz: a sweep of the unmodified reference routines
driven by oracle/ref_harness.cpp on such a chain (an off-centre band, so the
on-site energies e_N are not zero), in the format of make_golden.py, with
the chain used.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(REPO, "oracle", "_ref", "ref_harness")
sys.path.insert(0, HERE)
from make_golden import parse  # noqa: E402

KEEP = 60
# name: (kind, Lambda, z, DiscScheme, BandOffset, params)
CHAINS = {
    "const": ("const", 2.5, 1.0, 0, 0.0, ()),
    "const_z05": ("const", 2.5, 0.5, 0, 0.0, ()),
    "const_co_L2": ("const", 2.0, 1.0, 1, 0.0, (1.0,)),
    "const_off01": ("const", 2.5, 1.0, 0, 0.1, ()),
    "lorentzian": ("lorentzian", 2.5, 1.0, 0, 0.0, (0.0, 0.05, 0.1, 0.0, 0.3, 0.0)),
    "table": ("table", 2.5, 1.0, 0, 0.0,
              tuple(v for w in np.linspace(-1.0, 1.0, 41) for v in (float(w), float(1.0 - 0.5 * w * w + 0.2 * w)))),
}
# name: (model, nsites, ncutoff, Lambda, U, ed, Gamma1, Gamma2|B, chain)
SWEEPS = {
    "chain_1chQS_off01_n12_k150": ("1chQS", 12, 150, 2.5, 0.5, -0.25, 0.02, 0.0, "const_off01"),
    "chain_1chQSz_off01_n10_k200": ("1chQSz", 10, 200, 2.5, 0.5, -0.25, 0.02, 1.0e-3, "const_off01"),
    "chain_2chQS_lor_n5_k80": ("2chQS", 5, 80, 2.5, 0.3, -0.15, 0.01, 0.01, "lorentzian"),
}


def lanczos(kind, lam, z, disc, off, params, n=100):
    args = [HARNESS, "lanczos", kind, repr(lam), repr(z), str(disc), repr(off), str(n)] + [repr(p) for p in params]
    out = subprocess.run(args, check=True, capture_output=True, text=True,
                         env=dict(os.environ, OPENBLAS_NUM_THREADS="1")).stdout.splitlines()
    c = np.array([[float(x) for x in l.split()[2:4]] for l in out if l.startswith("CHAIN")])
    fsq = [float(l.split()[1]) for l in out if l.startswith("FSQ")][0]
    return c[:, 0], c[:, 1], fsq


def main() -> None:
    if not os.path.exists(HARNESS):
        sys.exit("build the reference first: bash oracle/build_ref.sh")
    out = {}
    full = {}
    for name, (kind, lam, z, disc, off, params) in CHAINS.items():
        chi, en, fsq = lanczos(kind, lam, z, disc, off, params)
        full[name] = (chi, en)
        out[f"{name}_chi"] = chi[:KEEP]
        out[f"{name}_en"] = en[:KEEP]
        out[f"{name}_fsq"] = np.array(fsq)
        out[f"{name}_band"] = np.array([kind, lam, z, disc, off], dtype=object).astype(str)
        out[f"{name}_params"] = np.array(params, dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "chain_lanczos.npz"), **out)
    print("chain_lanczos", len(CHAINS), "chains")
    for name, (model, ns, nc, lam, U, ed, g1, x, ch) in SWEEPS.items():
        chi, en = full[ch]
        with tempfile.NamedTemporaryFile("w", suffix=".dat", delete=False) as f:
            for a, b in zip(chi, en):
                f.write(f"{float(a)!r} {float(b)!r}\n")
            path = f.name
        try:
            args = [HARNESS, model, str(ns), str(nc), repr(lam), repr(U), repr(ed), repr(g1), repr(x), "0.0", path]
            txt = subprocess.run(args, check=True, capture_output=True, text=True,
                                 env=dict(os.environ, OPENBLAS_NUM_THREADS="1")).stdout
        finally:
            os.unlink(path)
        d = parse(txt)
        d["config"] = np.array([model, ns, nc, lam, U, ed, g1, x], dtype=object).astype(str)
        d["chain_chi"] = chi[:KEEP]
        d["chain_en"] = en[:KEEP]
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(name, d["niters"], "iterations")


if __name__ == "__main__":
    main()
