"""Derivatives of the DM-NRG spectral function (nrg_grad_forward_dm ->
nrg_dm_backprop with tangents -> nrg_lehmann_grad) against central finite
differences of the GPU DM-NRG itself (nrg_sweep_run_dm -> nrg_dm_backprop ->
nrg_lehmann at p +- h).

Step h = 1e-5 |p|, with the kept-state sets of both displaced sweeps equal to
the undisplaced one's (the derivatives are taken at a fixed kept set).
Tolerance: 1e-6 of the largest |dA/dp| over the frequencies plus 1e-6
relative.  The asymmetric point (eps_d != -U/2) is checked for every
parameter; the particle-hole symmetric one for Gamma, which keeps the
symmetry (eps_d and U break it, and the levels that the symmetry pairs are
split there only by the irrelevant operators, closer than the difference
quotient resolves at this step)."""
import numpy as np
import pytest

import twochnrg_gb300 as tg

pytestmark = pytest.mark.gpu

# (nsites, ncutoff, Lambda, U, eps_d, Gamma, mtemp, parameters checked)
CASES = [
    ("asym_T0", (14, 120, 2.5, 0.4, -0.15, 0.02, -1, (0, 1, 2))),
    ("asym_M10", (14, 120, 2.5, 0.4, -0.15, 0.02, 10, (0, 1, 2))),
    ("sym_M10_gamma", (14, 120, 2.5, 0.4, -0.2, 0.015, 10, (2,))),
]


def _same_kept(a, b):
    return all(x.nkept == y.nkept and np.array_equal(x.kept_bsize, y.kept_bsize) for x, y in zip(a.iters, b.iters))


def _spectrum(engine, case, k=None, delta=0.0):
    ns, nc, lam, U, ed, G, mtemp, _ = case
    p = [ed, U, G]
    if k is not None:
        p[k] += delta
    engine.sweep_dm(ns, nc, lam, p[1], p[0], p[2])
    sweep = engine.fetch()
    prm = engine.dm_params(mtemp=mtemp, bbroad=0.6, nw=4)
    engine.dm_backprop(prm)
    om, A = engine.lehmann(prm)
    return sweep, om, A


@pytest.mark.parametrize("name,case", CASES, ids=[c[0] for c in CASES])
def test_dA_matches_central_differences(engine, name, case):
    ns, nc, lam, U, ed, G, mtemp, check = case
    g = engine.grad_forward_dm(ns, nc, lam, U, ed, G)
    prm = engine.dm_params(mtemp=mtemp, bbroad=0.6, nw=4)
    engine.dm_backprop(prm)
    om, A, dA = engine.lehmann_grad(prm)
    assert dA.shape == (4, len(om))
    assert np.all(np.isfinite(dA))
    assert np.abs(dA[3]).max() == 0.0  # no field in the |Q S> model
    ref_sweep, ref_om, ref_A = _spectrum(engine, case)
    np.testing.assert_array_equal(om, ref_om)
    # the forward pass and the spectrum are the plain DM-NRG's
    np.testing.assert_allclose(A, ref_A, rtol=1e-12, atol=1e-14 * np.abs(ref_A).max())
    assert _same_kept(g.sweep, ref_sweep)
    params = [ed, U, G]
    failures = []
    for k in check:
        h = 1e-5 * abs(params[k])
        sp, _, Ap = _spectrum(engine, case, k, h)
        sm, _, Am = _spectrum(engine, case, k, -h)
        assert _same_kept(sp, ref_sweep) and _same_kept(sm, ref_sweep)
        fd = (Ap - Am) / (2 * h)
        scale = np.abs(fd).max()
        assert scale > 0.0
        err = np.abs(dA[k] - fd)
        bad = err > 1e-6 * scale + 1e-6 * np.abs(fd)
        if bad.any():
            failures.append(f"parameter {k}: max |analytic - fd| {err.max():.3e} at omega {om[np.argmax(err)]:.3e}, "
                            f"max |fd| {scale:.3e}, {int(bad.sum())} of {len(om)} frequencies")
    assert not failures, "; ".join(failures)


def test_dA_backward_is_the_contraction(engine):
    ns, nc, lam, U, ed, G, mtemp, _ = CASES[0][1]
    engine.grad_forward_dm(ns, nc, lam, U, ed, G)
    prm = engine.dm_params(mtemp=mtemp, bbroad=0.6, nw=4)
    engine.dm_backprop(prm)
    om, A, dA = engine.lehmann_grad(prm)
    w = np.random.default_rng(5).standard_normal(len(om))
    np.testing.assert_allclose(engine.lehmann_grad_backward(w), dA @ w, rtol=1e-12, atol=1e-14 * np.abs(dA).sum())
    with pytest.raises(ValueError):
        engine.lehmann_grad_backward(w[:-1])


def test_dA_needs_the_tangent_shells(engine):
    ns, nc, lam, U, ed, G, mtemp, _ = CASES[0][1]
    engine.sweep_dm(ns, nc, lam, U, ed, G)  # shells without tangents
    prm = engine.dm_params(mtemp=mtemp, bbroad=0.6, nw=4)
    engine.dm_backprop(prm)
    with pytest.raises(tg.NRGError) as e:
        engine.lehmann_grad(prm)
    assert e.value.status == 8  # NRG_ERR_STATE
    cfg = tg.SweepConfig(tg.MODELS["2chQS"], ns, nc, lam, U, ed, G, G, 0.0, tg.PREC_FP64, 0.0)
    g = tg._Grad()
    assert engine.L.nrg_grad_forward_dm(engine.h, tg.ctypes.byref(cfg), tg.ctypes.byref(g)) == 1  # NRG_ERR_ARG


def test_dA_matches_differences_of_the_oracle(engine):
    """The same derivatives against central differences of the oracle's
    DM-NRG (the reference's algorithm restated on the CPU), on a log grid at
    T = D_8 / betabar."""
    from oracle import oracle as orc
    ns, nc, lam, U, ed, G = 12, 80, 2.5, 0.4, -0.15, 0.015
    temp = 0.7 * lam ** (-(8 - 1) / 2.0) / 0.727
    om = np.concatenate([-np.logspace(0, -5, 40), np.logspace(-5, 0, 40)])
    engine.grad_forward_dm(ns, nc, lam, U, ed, G)
    prm = engine.dm_params(temp=temp, bbroad=0.6)
    engine.dm_backprop(prm)
    _, A, dA = engine.lehmann_grad(prm, omegas=om)
    params = [ed, U, G]
    failures = []
    for k in range(3):
        h = 1e-5 * abs(params[k])
        out = []
        for sgn in (1, -1):
            p = list(params)
            p[k] += sgn * h
            out.append(orc.dm_spectral(ns, nc, lam, p[1], p[0], p[2], temp, 0.6, omegas=om)[1])
        fd = (out[0] - out[1]) / (2 * h)
        err = np.abs(dA[k] - fd)
        scale = np.abs(fd).max()
        if (err > 1e-6 * scale + 1e-6 * np.abs(fd)).any():
            failures.append(f"parameter {k}: max |analytic - fd| {err.max():.3e}, max |fd| {scale:.3e}")
    assert not failures, "; ".join(failures)
