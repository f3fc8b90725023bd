"""Wilson chains of non-flat bands (nrg_chain_lanczos, host code) and the
oracle's sweeps on them, on the CPU, against the reference's own
CNRGchain::SetChainLanczos and NRG routines (tests/golden/chain_*.npz, made by
tests/golden/make_chain_golden.py).

Tolerance: the first 60 hoppings within 1e-12 relative and on-site energies
within 1e-9 absolute of the reference's chain of 100 sites (the Lanczos
recurrence loses digits towards the end of the chain; both implementations
integrate the band exactly to rounding); sweeps as the other oracle fixtures."""
import os

import numpy as np
import pytest

import twochnrg_gb300 as tg
from oracle import oracle as orc

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ["const", "const_z05", "const_co_L2", "const_off01", "lorentzian", "table"]
SWEEPS = ["chain_1chQS_off01_n12_k150", "chain_1chQSz_off01_n10_k200", "chain_2chQS_lor_n5_k80"]


@pytest.fixture(scope="module")
def lib_built():
    from twochnrg_gb300 import build
    build.build()


@pytest.mark.parametrize("name", NAMES)
def test_lanczos_matches_reference(lib_built, name):
    g = np.load(os.path.join(GOLD, "chain_lanczos.npz"))
    kind, lam, z, disc, off = g[f"{name}_band"]
    chi, en, fsq = tg.chain_lanczos(str(kind), 100, float(lam), g[f"{name}_params"], float(z), int(disc), float(off))
    k = len(g[f"{name}_chi"])
    np.testing.assert_allclose(chi[:k], g[f"{name}_chi"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(en[:k], g[f"{name}_en"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(fsq, float(g[f"{name}_fsq"]), rtol=1e-13)


def test_flat_band_lanczos_is_wilsons_chain(lib_built):
    """For the flat band (z = 1) the Lanczos chain is Wilson's closed form
    (CNRGchain::SetChainWilson) away from the truncated end, to the round-off
    the recurrence accumulates (1e-12 by site 40)."""
    lam = 2.5
    chi, en, fsq = tg.chain_lanczos("const", 100, lam)
    n = np.arange(40)
    wilson = (1 - lam ** -(n + 1.0)) / (np.sqrt(1 - lam ** -(2 * n + 1.0)) * np.sqrt(1 - lam ** -(2 * n + 3.0)))
    np.testing.assert_allclose(chi[:10], wilson[:10], rtol=1e-15)
    np.testing.assert_allclose(chi[:40], wilson, rtol=1e-12)
    assert np.abs(en[:40]).max() < 1e-12
    assert abs(fsq - 2.0) < 1e-14


def test_lanczos_arguments(lib_built):
    with pytest.raises(tg.NRGError):
        tg.chain_lanczos("lorentzian", 20, 2.5, (0, 0.05, 0.1, 0, 0.3, 0), disc_scheme=1)  # no Gamma/w form
    with pytest.raises(tg.NRGError):
        tg.chain_lanczos("table", 20, 2.5, (0.0, 1.0, 0.5))  # odd number of table values
    with pytest.raises(tg.NRGError):
        tg.chain_lanczos("const", 20, 1.0)  # Lambda must exceed 1


@pytest.mark.parametrize("name", SWEEPS)
def test_oracle_sweep_on_a_chain(name):
    g = np.load(os.path.join(GOLD, name + ".npz"))
    model, ns, nc, lam, U, ed, g1, x = g["config"]
    s = orc.run(model, int(ns), int(nc), float(lam), float(U), float(ed), float(g1), float(x),
                nthreads=min(8, os.cpu_count() or 1), wilson=(g["chain_chi"], g["chain_en"]))
    assert len(s.iters) == int(g["niters"])
    for n, it in enumerate(s.iters):
        np.testing.assert_array_equal(it.qn, g[f"qn_{n}"])
        np.testing.assert_array_equal(it.bsize, g[f"bsize_{n}"])
        assert it.nkept == int(g[f"nkept_{n}"])
        np.testing.assert_allclose(it.params, g[f"params_{n}"], rtol=0, atol=0)
        np.testing.assert_allclose(it.en, g[f"en_{n}"], rtol=0, atol=1e-11)
        np.testing.assert_allclose(it.thermo, g[f"thermo_{n}"], rtol=1e-11, atol=1e-13)
        np.testing.assert_allclose(it.opavg, g[f"opavg_{n}"], rtol=1e-11, atol=1e-13)
