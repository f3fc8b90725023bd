"""The plug-in boundary's host tables (no device): the built-in one-channel
models restated as plug-ins (plugin_models.py) give the built-in models'
H_N coefficient tables, operator site factors and selection rules bit for
bit, and malformed descriptions are refused."""
import numpy as np
import pytest

import plugin_models as pm
import twochnrg_gb300 as tg

CASES = [("1chQS", lambda: pm.one_channel_qs(0.5, -0.25, 2.5), 4, 4),
         ("1chQSz", lambda: pm.one_channel_qsz(0.5, -0.25, 1e-3, 2.5), 4, 4),
         ("2chQS", lambda: pm.two_channel_qs(0.3, -0.15, 2.5), 16, 5),
         ("1chQ", lambda: pm.one_channel_q(0.4, -0.2, 2.5), 4, 4)]
QN = [(-1.0, 0.0), (0.0, 0.5), (1.0, 0.0), (0.0, -0.5), (2.0, 0.5), (1.0, 1.0), (-2.0, 1.5)]


@pytest.mark.parametrize("name,make,ntypes,nops", CASES, ids=[c[0] for c in CASES])
def test_tables_equal_builtin(name, make, ntypes, nops):
    a, b = tg.ModelTables(name), tg.ModelTables(make())
    for S in np.arange(0.0, 8.5, 0.5):
        ta, tb = a.hn_table(S), b.hn_table(S)
        per_pair = {"1chQS": 2, "1chQSz": 4, "2chQS": 8, "1chQ": 4}[name]  # 2 nchan nsigma
        assert ta.shape == tb.shape and ta.size == ntypes * ntypes * per_pair
        np.testing.assert_array_equal(ta, tb)
    for o in range(nops):
        for Si in np.arange(0.0, 3.0 if ntypes > 4 else 4.0, 0.5):
            for Sj in np.arange(0.0, 3.0 if ntypes > 4 else 4.0, 0.5):
                for ti in range(ntypes):
                    for tj in range(ntypes):
                        assert a.op_factor(o, Si, Sj, ti, tj) == b.op_factor(o, Si, Sj, ti, tj)
        for qi in QN:
            for qj in QN:
                assert a.op_check(o, qi, qj) == b.op_check(o, qi, qj)


def test_malformed_descriptions_refused():
    good = pm.one_channel_qs(0.5, -0.25, 2.5)
    tg.ModelTables(good).hn_table(0.5)
    for field, value in [("hn_form", 9), ("op_class", [tg.OP_SITE, 7, 2, 2]), ("site_bsize", [1, 0, 1, 1]),
                         ("op_class", [])]:
        bad = pm.one_channel_qs(0.5, -0.25, 2.5)
        setattr(bad, field, value)
        with pytest.raises(tg.NRGError):
            tg.ModelTables(bad).hn_table(0.5)


def test_callback_error_surfaces():
    bad = pm.one_channel_qs(0.5, -0.25, 2.5)

    def boom(*a):
        raise KeyError("no rule")
    bad.hn_coef = boom
    with pytest.raises(KeyError):
        tg.ModelTables(bad).hn_table(0.5)
    bad = pm.one_channel_qs(0.5, -0.25, 2.5)
    bad.hn_coef = lambda *a: float("inf")
    with pytest.raises(tg.NRGError):
        tg.ModelTables(bad).hn_table(0.5)
