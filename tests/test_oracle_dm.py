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


def test_two_channel_all_kept_is_one_channel_with_summed_gamma():
    """The two-channel Anderson impurity couples to the even combination of
    two identical Wilson chains only; the odd one is a free chain.  With every
    state kept the FDM sum reduces to the last shell's exact Lehmann sum, so
    A(omega) of 2chQS(Gamma1, Gamma2) equals 1chQS(Gamma1 + Gamma2) to
    round-off.  This pins the two-channel c_d rule (for which the reference
    has none) and the 16-state site's multiplet algebra."""
    om = np.concatenate([-np.logspace(0, -3, 25), np.logspace(-3, 0, 25)])
    T = 1e-3
    _, A2, tr2 = orc.dm_spectral(2, 100000, 2.5, 0.3, -0.15, 0.01, T, 0.6, omegas=om, model="2chQS", gamma2=0.012,
                                 nthreads=min(8, os.cpu_count() or 1))
    _, A1, tr1 = orc.dm_spectral(2, 100000, 2.5, 0.3, -0.15, 0.022, T, 0.6, omegas=om)
    assert np.abs(A2 - A1).max() < 1e-12 * np.abs(A1).max()
    np.testing.assert_allclose(tr2, tr1, rtol=1e-12)


def test_two_channel_trace_is_one_in_the_default_branch():
    """The backward sweep's partial trace over the 16-state site (children
    weighted by the squared Clebsch-Gordan sums of site multiplets of spin 0,
    1/2 and 1) keeps the trace.  Six shells: with an odd number of sites the
    free odd chain has a zero mode, the ground multiplets are degenerate to
    round-off, and SetRhoNmax's beta cap of 1e10 (versus the partition sum's
    exact beta) then counts them in rho but not in Z, in both
    implementations."""
    _, _, tr = orc.dm_spectral(6, 60, 2.5, 0.3, -0.15, 0.01, 0.0, 0.6, nw=2, model="2chQS", gamma2=0.012)
    np.testing.assert_allclose(tr, 1.0, rtol=1e-12)
