"""Derivatives of the sweep (nrg_grad_forward / nrg_grad_backward) against
central finite differences of the GPU sweep itself, and the Hellmann-Feynman
identities of the reference's averaged operators.

Finite differences: step h = 1e-5 |p| for eps_d, U and Gamma (1e-6 for the
small field B), with the kept-state sets of both displaced sweeps equal to
the undisplaced one's (the derivatives are taken at a fixed kept set).
Tolerance: 1e-6 relative plus 1e-6 of the largest derivative of that
quantity over the sweep (at least 1e-3: derivatives that vanish by symmetry
leave only the sweep's round-off, ~1e-10, in the difference quotient); 1e-5
for B, whose difference quotient carries the round-off over a smaller step.
"""
import numpy as np
import pytest

import twochnrg_gb300 as tg

pytestmark = pytest.mark.gpu

# an asymmetric (Q,Sz) case with a field, and the symmetric (Q,S) case (where
# the derivatives of T chi with respect to eps_d vanish)
CASES = [("1chQSz", 12, 120, 2.5, 0.4, -0.15, 0.015, 1e-3), ("1chQS", 12, 120, 2.5, 0.4, -0.2, 0.015, 0.0)]


def _sweep(engine, case, k=None, delta=0.0):
    model, ns, nc, lam, U, ed, G, B = case
    p = [ed, U, G, B]
    if k is not None:
        p[k] += delta
    return engine.sweep(model, ns, nc, lam, p[1], p[0], p[2], p[3])


def _same_kept(a, b):
    return all(x.nkept == y.nkept and np.array_equal(x.kept_bsize, y.kept_bsize) for x, y in zip(a.iters, b.iters))


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_grad_matches_central_differences(engine, case):
    g = engine.grad_forward(*case)
    ref = _sweep(engine, case)
    for a, b in zip(g.sweep.iters, ref.iters):  # the forward pass is the plain sweep
        assert a.nkept == b.nkept
        np.testing.assert_allclose(a.en, b.en, rtol=0, atol=1e-12 * max(1.0, np.abs(b.en).max()))
        np.testing.assert_allclose(a.thermo, b.thermo, rtol=1e-12)
    params = [case[5], case[4], case[6], case[7]]
    failures = []
    for k in range(4):
        if k == 3 and case[0] == "1chQS":
            assert np.abs(g.d_thermo[:, 3]).max() == 0.0  # no field in the |Q S> model
            continue
        h = 1e-6 if k == 3 else 1e-5 * abs(params[k])
        plus, minus = _sweep(engine, case, k, h), _sweep(engine, case, k, -h)
        assert _same_kept(plus, ref) and _same_kept(minus, ref)
        fd_t = np.array([(p.thermo[:, 2:] - m.thermo[:, 2:]) / (2 * h) for p, m in zip(plus.iters, minus.iters)])
        fd_o = np.array([(p.opavg - m.opavg) / (2 * h) for p, m in zip(plus.iters, minus.iters)])
        rel = 1e-5 if k == 3 else 1e-6
        for what, fd, an in (("thermo", fd_t, g.d_thermo[:, k, :, 2:]), ("opavg", fd_o, g.d_opavg[:, k])):
            scale = max(np.abs(fd).max(), 1e-3)
            bad = np.abs(an - fd) > rel * np.abs(fd) + rel * scale
            if bad.any():
                failures.append(f"parameter {k} {what}: max |analytic - fd| {np.abs(an - fd).max():.3e}, "
                                f"max |fd| {np.abs(fd).max():.3e}")
    assert not failures, "; ".join(failures)


def test_grad_matches_differences_of_the_oracle(engine):
    """The asymmetric (Q,Sz) case against central differences of the oracle's
    sweep (the reference's algorithm restated on the CPU)."""
    from oracle import oracle as orc
    case = CASES[0]
    model, ns, nc, lam, U, ed, G, B = case
    g = engine.grad_forward(*case)
    params = [ed, U, G, B]
    failures = []
    for k in range(4):
        h = 1e-6 if k == 3 else 1e-5 * abs(params[k])
        runs = []
        for sgn in (1, -1):
            p = list(params)
            p[k] += sgn * h
            runs.append(orc.run(model, ns, nc, lam, p[1], p[0], p[2], p[3]))
        assert all(a.nkept == b.nkept == c.nkept for a, b, c in zip(runs[0].iters, runs[1].iters, g.sweep.iters))
        fd_t = np.array([(a.thermo[:, 2:] - b.thermo[:, 2:]) / (2 * h) for a, b in zip(runs[0].iters, runs[1].iters)])
        fd_o = np.array([(a.opavg - b.opavg) / (2 * h) for a, b in zip(runs[0].iters, runs[1].iters)])
        rel = 1e-5 if k == 3 else 1e-6
        for what, fd, an in (("thermo", fd_t, g.d_thermo[:, k, :, 2:]), ("opavg", fd_o, g.d_opavg[:, k])):
            scale = max(np.abs(fd).max(), 1e-3)
            if (np.abs(an - fd) > rel * np.abs(fd) + rel * scale).any():
                failures.append(f"parameter {k} {what}: max |analytic - fd| {np.abs(an - fd).max():.3e}, "
                                f"max |fd| {np.abs(fd).max():.3e}")
    assert not failures, "; ".join(failures)


def test_backward_is_the_jacobian_contraction(engine):
    case = CASES[0]
    g = engine.grad_forward(*case)
    rng = np.random.default_rng(3)
    n = len(g.sweep.iters)
    gt = rng.standard_normal((n, 16))
    go = rng.standard_normal((n, g.d_opavg.shape[2]))
    ge = rng.standard_normal(n)
    got = engine.grad_backward(gt, go, ge)
    want = (np.einsum("nv,nkv->k", gt, g.d_thermo.reshape(n, 4, 16)) + np.einsum("no,nko->k", go, g.d_opavg)
            + np.einsum("n,nk->k", ge, g.d_egs))
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(engine.grad_backward(g_egs=ge), np.einsum("n,nk->k", ge, g.d_egs), rtol=1e-12)


def test_hellmann_feynman_at_the_last_iteration(engine):
    """d E_gs / d eps_d = <n_d> and d E_gs / dU = <n_up n_dn> + 1/2 =
    (<n_d^2> - <n_d>)/2 + 1/2 (the impurity levels U/2, eps_d + U/2,
    2 eps_d + 3U/2), with the reference's averaged operators n_d and n_d^2
    (CalcOpAvg) at the last iteration, whose temperature (betabar / D_N,
    about 1e-9 here) leaves only the ground state: agreement to the NRG's
    truncation error (1e-4)."""
    g = engine.grad_forward("1chQS", 40, 300, 2.5, 0.4, -0.15, 0.015)
    nd, nd2 = g.sweep.iters[-1].opavg[0], g.sweep.iters[-1].opavg[1]
    assert abs(g.d_egs[-1, 0] - nd) < 1e-4 * max(1.0, abs(nd))
    assert abs(g.d_egs[-1, 1] - (0.5 * (nd2 - nd) + 0.5)) < 1e-4
