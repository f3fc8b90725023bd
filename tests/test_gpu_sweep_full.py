"""The headline two-channel workload at its full size -- 3000 kept
multiplets, iterations 0-4 (3 and 4 at about 45 000 states in ~53 blocks of
up to 4344) -- against the reference's own routines
(tests/golden/cfg1_2chQS_n5_k3000.npz, made by oracle/ref_harness from the
reference sources).  Both arithmetic forms: every integer of the block
bookkeeping exact (sectors, sizes, Nkept, kept blocks), E_cut and the block
eigenvalues within 1e-10 (FP64) / 1e-9 (mixed) of the iteration's largest
level, thermodynamics and operator averages within 1e-8 relative.
"""
import os

import numpy as np
import pytest

import twochnrg_gb300 as tg

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "cfg1_2chQS_n5_k3000.npz")


@pytest.mark.parametrize("prec,eig_tol", [(tg.PREC_FP64, 1e-10), (tg.PREC_MIXED, 1e-9)], ids=["fp64", "mixed"])
def test_full_size_iterations_match_reference(engine, prec, eig_tol):
    g = np.load(GOLD)
    model, ns, nc, lam, U, ed, g1, x = g["config"][:8]
    r = engine.sweep(str(model), int(ns), int(nc), float(lam), float(U), float(ed), float(g1), float(x),
                     precision=prec)
    assert len(r.iters) == int(g["niters"])
    for n, a in enumerate(r.iters):
        np.testing.assert_array_equal(a.qn, g[f"qn_{n}"], err_msg=f"N={n} sectors")
        np.testing.assert_array_equal(a.bsize, g[f"bsize_{n}"], err_msg=f"N={n} block sizes")
        assert a.nkept == int(g[f"nkept_{n}"]), f"N={n} Nkept"
        np.testing.assert_array_equal(a.kept_bsize, g[f"kept_bsize_{n}"], err_msg=f"N={n} kept blocks")
        en = g[f"en_{n}"]
        scale = max(1.0, float(np.abs(en).max()))
        assert float(np.abs(a.en - en).max()) / scale < eig_tol, f"N={n} eigenvalues"
        assert abs(a.ecut - float(g[f"ecut_{n}"])) / scale < eig_tol, f"N={n} E_cut"
        np.testing.assert_allclose(a.thermo, g[f"thermo_{n}"], rtol=1e-8, atol=1e-14, err_msg=f"N={n} thermo")
        np.testing.assert_allclose(a.opavg, g[f"opavg_{n}"], rtol=1e-8, atol=1e-12, err_msg=f"N={n} <O>")
    assert max(int(a.bsize.max()) for a in r.iters) > 4000
