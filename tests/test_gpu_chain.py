"""Sweeps on a Wilson chain other than the flat band's (nrg_set_chain) on the
GPU, against the reference routines run on the same chain
(tests/golden/chain_*.npz, made by tests/golden/make_chain_golden.py) and the
oracle.  Tolerances as for the flat-band sweeps: block eigenvalues 1e-10
relative to the largest level, thermodynamics and averages 1e-8, block
bookkeeping exact."""
import os

import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SWEEPS = ["chain_1chQS_off01_n12_k150", "chain_1chQSz_off01_n10_k200", "chain_2chQS_lor_n5_k80"]


def _compare(gpu_iters, ref):
    for n, a in enumerate(gpu_iters):
        np.testing.assert_array_equal(a.qn, ref[f"qn_{n}"], err_msg=f"N={n} sectors")
        np.testing.assert_array_equal(a.bsize, ref[f"bsize_{n}"])
        assert a.nkept == int(ref[f"nkept_{n}"]), n
        en = ref[f"en_{n}"]
        scale = max(1.0, float(np.abs(en).max()))
        assert np.abs(a.en - en).max() / scale < 1e-10, n
        np.testing.assert_allclose(a.thermo, ref[f"thermo_{n}"], rtol=1e-8, atol=1e-14)
        np.testing.assert_allclose(a.opavg, ref[f"opavg_{n}"], rtol=1e-8, atol=1e-12)


@pytest.mark.parametrize("name", SWEEPS)
def test_sweep_on_a_chain_matches_reference(engine, name):
    g = np.load(os.path.join(GOLD, name + ".npz"))
    model, ns, nc, lam, U, ed, g1, x = g["config"]
    engine.set_chain(g["chain_chi"], g["chain_en"])
    try:
        r = engine.sweep(str(model), int(ns), int(nc), float(lam), float(U), float(ed), float(g1), float(x))
    finally:
        engine.set_chain()
    assert len(r.iters) == int(g["niters"])
    _compare(r.iters, g)
    # e_N and the hoppings the iterations used
    for n, it in enumerate(r.iters):
        p = g[f"params_{n}"]
        assert it.params[0] == p[0] and it.params[1] == p[1]
        nch = 2 if str(model) == "2chQS" else 1
        assert it.params[3] == p[nch + 1]


def test_free_chain_and_flat_band_reset(engine):
    g = np.load(os.path.join(GOLD, "chain_1chQS_off01_n12_k150.npz"))
    chi, en = g["chain_chi"], g["chain_en"]
    engine.set_chain(chi, en)
    try:
        r = engine.sweep_chain("1chQS", 8, 120, 2.5)
        with pytest.raises(Exception):
            engine.sweep("1chQS", 80, 120, 2.5, 0.5, -0.25, 0.02)  # longer than the chain
    finally:
        engine.set_chain()
    o = orc.run("1chQS", 8, 120, 2.5, 0, 0, 0, chain=True, wilson=(chi, en))
    for a, b in zip(r.iters, o.iters):
        np.testing.assert_allclose(a.thermo, b.thermo, rtol=1e-8, atol=1e-14)
    # back on the flat band
    f = engine.sweep("1chQS", 6, 100, 2.5, 0.5, -0.25, 0.02)
    fo = orc.run("1chQS", 6, 100, 2.5, 0.5, -0.25, 0.02)
    for a, b in zip(f.iters, fo.iters):
        np.testing.assert_allclose(a.thermo, b.thermo, rtol=1e-8, atol=1e-14)
