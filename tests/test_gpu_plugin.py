"""Models supplied through the plug-in boundary (nrg_sweep_run_model): the
built-in one-channel models restated in Python (plugin_models.py) must pass
the same parity tests as the built-in ones -- the reference's golden
fixtures with the tolerances of test_gpu_sweep.py -- and give the built-in
sweep's results bit for bit (their tables are identical)."""
import os

import numpy as np
import pytest

import plugin_models as pm
import twochnrg_gb300 as tg
from test_gpu_sweep import GOLD, compare

pytestmark = pytest.mark.gpu


def _fixture(name):
    g = np.load(os.path.join(GOLD, name + ".npz"))

    class Ref:
        iters = []

    for n in range(int(g["niters"])):
        class It:
            pass
        it = It()
        it.qn, it.bsize, it.en = g[f"qn_{n}"], g[f"bsize_{n}"], g[f"en_{n}"]
        it.nkept, it.ecut = int(g[f"nkept_{n}"]), float(g[f"ecut_{n}"])
        it.kept_bsize, it.thermo, it.opavg = g[f"kept_bsize_{n}"], g[f"thermo_{n}"], g[f"opavg_{n}"]
        Ref.iters.append(it)
    return g["config"], Ref


def _same(a, b):
    assert len(a.iters) == len(b.iters)
    for x, y in zip(a.iters, b.iters):
        np.testing.assert_array_equal(x.qn, y.qn)
        np.testing.assert_array_equal(x.bsize, y.bsize)
        np.testing.assert_array_equal(x.en, y.en)
        np.testing.assert_array_equal(x.kept_bsize, y.kept_bsize)
        np.testing.assert_array_equal(x.thermo, y.thermo)
        np.testing.assert_array_equal(x.opavg, y.opavg)
        assert x.nkept == y.nkept and x.ecut == y.ecut and x.emin == y.emin


def test_plugin_qs_matches_reference_fixture(engine):
    cfg, ref = _fixture("cfg0_1chQS_n40_k500")
    model, ns, nc, lam, U, ed, g1, _ = cfg[:8]
    assert str(model) == "1chQS"
    plug = pm.one_channel_qs(float(U), float(ed), float(lam))
    r = engine.sweep_model(plug, int(ns), int(nc), float(lam), float(g1))
    compare(r, ref, "1chQS")
    b = engine.sweep("1chQS", int(ns), int(nc), float(lam), float(U), float(ed), float(g1))
    _same(r, b)


def test_plugin_qsz_matches_reference_fixture(engine):
    cfg, ref = _fixture("qsz_1chQSz_n14_k300")
    model, ns, nc, lam, U, ed, g1, B = cfg[:8]
    assert str(model) == "1chQSz"
    plug = pm.one_channel_qsz(float(U), float(ed), float(B), float(lam))
    r = engine.sweep_model(plug, int(ns), int(nc), float(lam), float(g1))
    compare(r, ref, "1chQSz")
    b = engine.sweep("1chQSz", int(ns), int(nc), float(lam), float(U), float(ed), float(g1), float(B))
    _same(r, b)


def test_plugin_two_channel_matches_reference_fixture(engine):
    cfg, ref = _fixture("cfg1_2chQS_n8_k300")
    model, ns, nc, lam, U, ed, g1, g2 = cfg[:8]
    assert str(model) == "2chQS"
    plug = pm.two_channel_qs(float(U), float(ed), float(lam))
    r = engine.sweep_model(plug, int(ns), int(nc), float(lam), float(g1), float(g2))
    compare(r, ref, "2chQS")
    b = engine.sweep("2chQS", int(ns), int(nc), float(lam), float(U), float(ed), float(g1), float(g2))
    _same(r, b)


def test_plugin_q_matches_reference_fixture(engine):
    cfg, ref = _fixture("q_1chQ_n12_k200")
    model, ns, nc, lam, U, ed, g1, _ = cfg[:8]
    assert str(model) == "1chQ"
    plug = pm.one_channel_q(float(U), float(ed), float(lam))
    r = engine.sweep_model(plug, int(ns), int(nc), float(lam), float(g1))
    compare(r, ref, "1chQ")
    b = engine.sweep("1chQ", int(ns), int(nc), float(lam), float(U), float(ed), float(g1))
    _same(r, b)


def test_plugin_mixed_precision(engine, monkeypatch):
    """The plug-in model through the mixed form (large-block thresholds
    lowered so the blocked reduction runs) against the FP64 built-in."""
    monkeypatch.setenv("NRG_BIG_N", "48")
    monkeypatch.setenv("NRG_MIXED_N", "48")
    plug = pm.one_channel_qs(0.5, -0.25, 2.5)
    r = engine.sweep_model(plug, 12, 300, 2.5, 0.02, precision=tg.PREC_MIXED)
    b = engine.sweep("1chQS", 12, 300, 2.5, 0.5, -0.25, 0.02)
    for x, y in zip(r.iters, b.iters):
        np.testing.assert_array_equal(x.bsize, y.bsize)
        assert x.nkept == y.nkept
        assert np.max(np.abs(x.en - y.en)) < 1e-9 * max(1.0, float(np.max(np.abs(y.en))))


def test_plugin_errors(engine):
    plug = pm.one_channel_qs(0.5, -0.25, 2.5)
    bad = pm.one_channel_qs(0.5, -0.25, 2.5)
    bad.hn_form = 7
    with pytest.raises(tg.NRGError):
        engine.sweep_model(bad, 4, 50, 2.5, 0.02)

    def boom(*a):
        raise ValueError("rule failed")
    bad = pm.one_channel_qs(0.5, -0.25, 2.5)
    bad.hn_coef = boom
    with pytest.raises(ValueError, match="rule failed"):
        engine.sweep_model(bad, 4, 50, 2.5, 0.02)
    # the context stays usable
    r = engine.sweep_model(plug, 4, 50, 2.5, 0.02)
    assert len(r.iters) == 4


# The per-call-site drop-ins (DiagHN and UpdateMatrices, where the reference
# calls CalcHNMatEl / CalcMatEl / CheckForMatEl) with the plug-in models: the
# results equal the built-in models' bit for bit on the oracle's captured
# iteration inputs.
STEP_CASES = [
    ("1chQS", 6, 80, 2.5, 0.5, -0.25, 0.02, 0.0, 4),
    ("1chQSz", 6, 70, 2.5, 0.4, -0.2, 0.015, 1e-3, 3),
    ("2chQS", 4, 60, 2.5, 0.3, -0.15, 0.01, 0.01, 2),
]


def _plugin_for(model, U, ed, x, lam):
    if model == "1chQS":
        return pm.one_channel_qs(U, ed, lam)
    if model == "1chQSz":
        return pm.one_channel_qsz(U, ed, x, lam)
    return pm.two_channel_qs(U, ed, lam)


@pytest.mark.parametrize("case", STEP_CASES, ids=[f"{c[0]}-N{c[8]}" for c in STEP_CASES])
def test_plugin_per_call_site(engine, case):
    from oracle import oracle as orc
    model, ns, nc, lam, U, ed, g1, x, n = case
    it = orc.run(model, ns, nc, lam, U, ed, g1, x, capture_iter=n).iters[n]
    cap = it.cap
    plug = _plugin_for(model, U, ed, x, lam)
    ops = [(cap[f"old_map.{o}"], cap[f"old_mbe.{o}"], cap[f"old_el.{o}"]) for o in range(cap["nmats"])]
    basis = (cap["basis_qn"], cap["basis_bbe"], cap["basis_itype"], cap["basis_stcf"], cap["basis_en"])
    a = engine.diag_hn(model, cap["params"], cap["old_qn"], cap["old_bbe"], ops, *basis)
    b = engine.diag_hn(plug, cap["params"], cap["old_qn"], cap["old_bbe"], ops, *basis)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    assert a[2] == b[2]
    args = (cap["old_qn"], cap["old_bbe"], *basis, cap["cut_qn"], cap["cut_bbe"], cap["cut_bbe_eig"],
            cap["cut_evec"], ops)
    na, nb = engine.update_ops(model, *args), engine.update_ops(plug, *args)
    assert len(na) == len(nb)
    for (m1, e1, v1), (m2, e2, v2) in zip(na, nb):
        np.testing.assert_array_equal(m1, m2)
        np.testing.assert_array_equal(e1, e2)
        np.testing.assert_array_equal(v1, v2)
