"""Per-step drop-ins for the NRG_main call sites against the oracle's inputs
and outputs of one iteration:

  nrg_diag_hn    (DiagHN + SetE0zero)  eigenvalues within 1e-12 of the
                 spectrum's scale; eigenvectors by residual against the
                 oracle's H_N, orthonormality, and against dspev's up to sign
                 where the level is isolated
  nrg_cut_states (SetKept + CutStates) bit-exact: energies after SetDegen,
                 Kept, Nkept, Ecut, AeigCut's BlockBegEnd / BlockBegEndBC /
                 BlockBegEndEigVec / StCameFrom / dEn / dEigVec
  nrg_update_ops (UpdateMatrices)      block-pair lists exact, elements within
                 1e-12 of the operator's largest element
"""
import numpy as np
import pytest

import twochnrg_gb300 as tg
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

# model, nsites, ncutoff, Lambda, U, ed, Gamma1, Gamma2 or B, capture iteration
CASES = [
    ("1chQS", 6, 80, 2.5, 0.5, -0.25, 0.02, 0.0, 4),
    ("1chQSz", 6, 70, 2.5, 0.4, -0.2, 0.015, 1e-3, 3),
    ("2chQS", 4, 60, 2.5, 0.3, -0.15, 0.01, 0.01, 2),
    ("2chQS", 2, 60, 2.5, 0.3, -0.15, 0.01, 0.02, 0),   # first iteration: H_{-1} operators
]


@pytest.fixture(scope="module", params=CASES, ids=[f"{c[0]}-N{c[8]}" for c in CASES])
def step(request):
    model, ns, nc, lam, U, ed, g1, g2, n = request.param
    o = orc.run(model, ns, nc, lam, U, ed, g1, g2, capture_iter=n)
    return model, nc, o.iters[n]


def _ops(cap, pre):
    return [(cap[f"{pre}_map.{o}"], cap[f"{pre}_mbe.{o}"], cap[f"{pre}_el.{o}"]) for o in range(cap["nmats"])]


def _basis(cap):
    return (cap["basis_qn"], cap["basis_bbe"], cap["basis_itype"], cap["basis_stcf"], cap["basis_en"])


def test_diag_hn(engine, step):
    model, _, it = step
    cap = it.cap
    en, vec, emin = engine.diag_hn(model, cap["params"], cap["old_qn"], cap["old_bbe"], _ops(cap, "old"),
                                   *_basis(cap))
    ref = cap["eig_en"]
    scale = max(1.0, float(np.max(np.abs(ref))) + abs(it.emin))
    assert abs(emin - it.emin) < 1e-12 * scale
    assert np.max(np.abs(en - ref)) < 1e-12 * scale
    assert en.min() == 0.0
    bbe = cap["basis_bbe"]
    hpos = vpos = 0
    for b in range(len(bbe) // 2):
        b0, b1 = int(bbe[2 * b]), int(bbe[2 * b + 1])
        n = b1 - b0 + 1
        A = np.zeros((n, n))
        iu = np.triu_indices(n)
        A[iu] = it.H[hpos:hpos + n * (n + 1) // 2]
        A = A + A.T - np.diag(np.diag(A))
        hpos += n * (n + 1) // 2
        Z = vec[vpos:vpos + n * n].reshape(n, n)
        Zr = cap["eig_evec"][vpos:vpos + n * n].reshape(n, n)
        vpos += n * n
        w = en[b0:b1 + 1] + emin
        assert np.all(np.diff(en[b0:b1 + 1]) >= 0)
        assert np.max(np.abs(A @ Z.T - Z.T * w)) < 1e-11 * scale
        assert np.max(np.abs(Z @ Z.T - np.eye(n))) < 1e-11
        wr = ref[b0:b1 + 1]
        gaps = np.diff(wr)
        for k in range(n):
            if (k == 0 or gaps[k - 1] > 1e-6 * scale) and (k == n - 1 or gaps[k] > 1e-6 * scale):
                s = np.sign(Z[k] @ Zr[k])
                assert np.max(np.abs(s * Z[k] - Zr[k])) < 1e-8
    assert vpos == len(vec)


def test_cut_states(engine, step):
    _, nc, it = step
    cap = it.cap
    r = engine.cut_states(cap["basis_qn"], cap["basis_bbe"], cap["eig_en"], cap["eig_evec"], nc)
    np.testing.assert_array_equal(r["en"], cap["kept_en"])
    np.testing.assert_array_equal(r["kept"], cap["kept"])
    assert r["nkept"] == it.nkept
    assert r["ecut"] == it.ecut
    np.testing.assert_array_equal(r["qn"], cap["cut_qn"])
    for k in ("bbe", "bbe_bc", "bbe_eig", "stcf"):
        np.testing.assert_array_equal(r[k], cap["cut_" + k], err_msg=k)
    np.testing.assert_array_equal(r["cut_en"], cap["cut_en"])
    np.testing.assert_array_equal(r["cut_kept"], cap["cut_kept"])
    np.testing.assert_array_equal(r["eigvec"], cap["cut_evec"])


def test_cut_states_keeps_everything_when_ncutoff_covers_all(engine, step):
    _, _, it = step
    cap = it.cap
    ns = len(cap["eig_en"])
    r = engine.cut_states(cap["basis_qn"], cap["basis_bbe"], cap["eig_en"], cap["eig_evec"], ns + 5)
    assert r["nkept"] == ns and np.all(r["kept"] == 1)
    np.testing.assert_array_equal(r["bbe"], cap["basis_bbe"])
    np.testing.assert_array_equal(r["bbe_bc"], cap["basis_bbe"])
    np.testing.assert_array_equal(r["stcf"], np.arange(ns))
    np.testing.assert_array_equal(r["eigvec"], cap["eig_evec"])


def test_update_ops(engine, step):
    model, _, it = step
    cap = it.cap
    new = engine.update_ops(model, cap["old_qn"], cap["old_bbe"], *_basis(cap), cap["cut_qn"], cap["cut_bbe"],
                            cap["cut_bbe_eig"], cap["cut_evec"], _ops(cap, "old"))
    ref = _ops(cap, "new")
    assert len(new) == len(ref)
    for o, ((mp, mbe, el), (mpr, mber, elr)) in enumerate(zip(new, ref)):
        np.testing.assert_array_equal(mp, mpr, err_msg=f"MatBlockMap op {o}")
        np.testing.assert_array_equal(mbe, mber, err_msg=f"MatBlockBegEnd op {o}")
        scale = max(1.0, float(np.max(np.abs(elr)))) if len(elr) else 1.0
        assert len(el) == len(elr)
        assert np.max(np.abs(el - elr), initial=0.0) < 1e-12 * scale, f"MatEl op {o}"


def test_step_argument_errors(engine, step):
    model, nc, it = step
    cap = it.cap
    with pytest.raises(tg.NRGError) as e:  # energies not E_min-shifted
        engine.cut_states(cap["basis_qn"], cap["basis_bbe"], cap["eig_en"] + 1.0, None, nc)
    assert e.value.status == 1
    stcf = cap["basis_stcf"].copy()
    stcf[[0, -1]] = stcf[[-1, 0]]
    if stcf[0] != cap["basis_stcf"][0]:
        with pytest.raises(tg.NRGError) as e:  # a basis BuildBasis would not make
            engine.diag_hn(model, cap["params"], cap["old_qn"], cap["old_bbe"], _ops(cap, "old"),
                           cap["basis_qn"], cap["basis_bbe"], cap["basis_itype"], stcf, cap["basis_en"])
        assert e.value.status == 6
    with pytest.raises(tg.NRGError) as e:  # superconducting leads
        p = np.append(cap["params"][:-1], 0.1)
        engine.diag_hn(model, p, cap["old_qn"], cap["old_bbe"], _ops(cap, "old"), *_basis(cap))
    assert e.value.status == 1
