"""DM-NRG on the GPU (nrg_sweep_run_dm -> nrg_dm_backprop -> nrg_lehmann)
against the reference DM_NRG's own A(omega) (tests/golden/dm_*.npz, made by
tests/golden/make_dm_golden.py) and against the oracle on other temperatures
and frequency grids.

Tolerance: spectra within 1e-8 relative (the block eigenvectors come from a
different eigensolver than LAPACK's, so agreement is at the eigenvector
round-off, amplified by near-degenerate levels), with an absolute floor of
1e-10 of the spectrum's maximum for the exponentially small tails."""
import os

import numpy as np
import pytest

import twochnrg_gb300 as tg
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ["dm_1chQS_n10_k60_T0", "dm_1chQS_n10_k60_M6", "dm_1chQS_n16_k150_M12"]


def _close(A, ref):
    np.testing.assert_allclose(A, ref, rtol=1e-8, atol=1e-10 * float(np.max(np.abs(ref))))


@pytest.mark.parametrize("name", CASES)
def test_dm_spectral_matches_reference(engine, name):
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    ns, nc, U, G, ed, lam, b, nw, mtemp = g["config"]
    nsh = engine.sweep_dm(int(ns), int(nc), lam, U, ed, G)
    assert nsh == int(ns)
    prm = engine.dm_params(mtemp=int(mtemp), bbroad=b, nw=int(nw))
    tr = engine.dm_backprop(prm)
    assert np.all(np.isfinite(tr))
    om, A = engine.lehmann(prm)
    np.testing.assert_allclose(om, g["omega"], rtol=1e-14)
    _close(A, g["A"])


def test_dm_against_oracle_on_a_log_grid(engine):
    lam, ns = 2.5, 12
    temp = 0.7 * lam ** (-(8 - 1) / 2.0) / 0.727     # T = D_8 / betabar
    om = np.concatenate([-np.logspace(0, -5, 60), np.logspace(-5, 0, 60)])
    o_om, o_A, o_tr = orc.dm_spectral(ns, 80, lam, 0.4, -0.2, 0.015, temp, 0.6, omegas=om)
    engine.sweep_dm(ns, 80, lam, 0.4, -0.2, 0.015)
    prm = engine.dm_params(temp=temp, bbroad=0.6)
    tr = engine.dm_backprop(prm)
    np.testing.assert_allclose(tr, o_tr, rtol=1e-10)
    g_om, A = engine.lehmann(prm, omegas=om)
    np.testing.assert_array_equal(g_om, om)
    _close(A, o_A)
    t = engine.timing()
    assert t["lehmann_pairs"] > 0 and t["lehmann_evals"] > 0


def test_dm_call_order_and_model_errors(engine):
    cfg = tg.SweepConfig(tg.MODEL_2CH_QS, 3, 40, 2.5, 0.3, -0.15, 0.01, 0.01, 0.0, 0)
    import ctypes
    st = engine.L.nrg_sweep_run_dm(engine.h, ctypes.byref(cfg))
    assert st == 1  # DM shells exist for the one-channel |Q S> model only
    engine.sweep_dm(6, 40, 2.5, 0.5, -0.25, 0.02)
    prm = engine.dm_params(nw=2)
    with pytest.raises(tg.NRGError) as e:  # Lehmann sums before the backward sweep
        engine.lehmann(prm)
    assert e.value.status == 8
