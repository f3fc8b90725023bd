"""The oracle's DM-NRG restatement (forward sweep with UpdateBefCut = 1 and
c_d, FDM density-matrix backward sweep, FDM spectral function) against the
reference DM_NRG's own rho_0_0_OmegaRhow.dat on the same inputs
(tests/golden/make_dm_golden.py).  Both use LAPACK dspev, so the match is at
round-off: 1e-12 relative."""
import os

import numpy as np
import pytest

from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ["dm_1chQS_n10_k60_T0", "dm_1chQS_n10_k60_M6", "dm_1chQS_n16_k150_M12"]


@pytest.mark.parametrize("name", CASES)
def test_dm_spectral_matches_reference(name):
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    ns, nc, U, G, ed, lam, b, nw, mtemp = g["config"]
    om, A, tr = orc.dm_spectral(int(ns), int(nc), lam, U, ed, G, 0.0, b, nw=int(nw), mtemp=int(mtemp))
    np.testing.assert_allclose(om, g["omega"], rtol=1e-14)
    np.testing.assert_allclose(A, g["A"], rtol=1e-12, atol=1e-300)
    assert np.all(np.isfinite(tr)) and tr[-1] > 0


def test_dm_trace_is_one_in_the_default_branch():
    # With T below every shell's scale all weight sits in the last shell's
    # ground multiplet and every reduced density matrix has unit trace.
    _, _, tr = orc.dm_spectral(8, 40, 2.5, 0.5, -0.25, 0.02, 0.0, 0.6, nw=2)
    np.testing.assert_allclose(tr, 1.0, rtol=1e-12)
