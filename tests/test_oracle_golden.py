"""The CPU oracle against the reference's golden data (no GPU).

run1_log.npz  : eigenvalue lines of the reference's own log Runs/run1 (6 digits)
<case>.npz    : full-precision output of the unmodified reference routines
                (tests/golden/make_golden.py).
"""
import os

import numpy as np
import pytest

from oracle import oracle as orc

GOLD = os.path.join(os.path.dirname(__file__), "golden")
CASES = ["run1_1chQS", "small_2chQS_n5_k60", "qsz_1chQSz_n14_k300", "cfg1_2chQS_n8_k300",
         "cfg0_1chQS_n40_k500", "q_1chQ_n12_k200", "s_1chS_n12_k200", "sz_1chSz_n12_k200"]


def _run(name, **kw):
    g = np.load(os.path.join(GOLD, name + ".npz"))
    model, ns, nc, lam, U, ed, g1, x = g["config"][:8]
    delta = float(g["config"][8]) if len(g["config"]) > 8 else 0.0  # superconducting leads' gap
    s = orc.run(model, int(ns), int(nc), float(lam), float(U), float(ed), float(g1), float(x),
                nthreads=min(8, os.cpu_count() or 1), delta_sc=delta, **kw)
    return g, s


def test_run1_log_reproduced():
    """All rescaled levels of Runs/run1/output_NRG_test.txt, to the 6 digits printed."""
    log = np.load(os.path.join(GOLD, "run1_log.npz"))
    s = orc.run("1chQS", 4, 1000, 2.5, 0.5, -0.25, 0.026444289241359498)
    ours_e, ours_q, ours_s = [], [], []
    for it in s.iters:
        q = np.repeat(it.qn[:, 0], it.bsize)
        ss = np.repeat(it.qn[:, 1], it.bsize)
        ours_e += list(it.en); ours_q += list(q); ours_s += list(ss)
    gold_e = log["en"][3:]  # the first three lines are H_{-1}
    assert len(gold_e) == len(ours_e)
    assert np.array_equal(log["q"][3:], np.array(ours_q))
    assert np.array_equal(log["s"][3:], np.array(ours_s))
    printed = np.array([float("%.6g" % x) for x in ours_e])
    assert np.array_equal(printed, gold_e)
    assert [it.nkept for it in s.iters] == list(log["nkept"][-4:])


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name):
    g, s = _run(name)
    assert len(s.iters) == int(g["niters"])
    np.testing.assert_array_equal(s.opavg_m1, g["opavg_m1"])
    for n, it in enumerate(s.iters):
        np.testing.assert_array_equal(it.qn, g[f"qn_{n}"])
        np.testing.assert_array_equal(it.bsize, g[f"bsize_{n}"])
        np.testing.assert_array_equal(it.kept_bsize, g[f"kept_bsize_{n}"])
        assert it.nkept == int(g[f"nkept_{n}"])
        # same arithmetic as the reference: equal up to the LAPACK build
        np.testing.assert_allclose(it.en, g[f"en_{n}"], rtol=0, atol=1e-11)
        np.testing.assert_allclose(it.thermo, g[f"thermo_{n}"], rtol=1e-11, atol=1e-13)
        np.testing.assert_allclose(it.opavg, g[f"opavg_{n}"], rtol=1e-11, atol=1e-13)
        np.testing.assert_allclose(it.ecut, float(g[f"ecut_{n}"]), rtol=0, atol=1e-11)


def test_clebsch_gordan_known_values():
    cg = orc.lib().oracle_cgordan
    assert abs(cg(0.5, 0.5, 0.5, -0.5, 0.0, 0.0) - np.sqrt(0.5)) < 1e-15
    assert abs(cg(0.5, -0.5, 0.5, 0.5, 0.0, 0.0) + np.sqrt(0.5)) < 1e-15
    assert abs(cg(1.0, 1.0, 0.5, -0.5, 0.5, 0.5) - np.sqrt(2.0 / 3.0)) < 1e-15
    assert cg(1.0, 1.0, 1.0, 1.0, 1.0, 1.0) == 0.0


def test_oracle_matches_reference_full_size_start():
    """The headline workload (two channels, 3000 kept): the oracle's first
    three iterations against the reference's own (fixture made by the
    reference routines; iterations 3-4 at full size are checked on the GPU
    and by the bench's CPU sample, minutes each on one core)."""
    g = np.load(os.path.join(GOLD, "cfg1_2chQS_n5_k3000.npz"))
    o = orc.run("2chQS", 3, 3000, 2.5, 0.3, -0.15, 0.01, 0.01, nthreads=min(8, os.cpu_count() or 1))
    for n, it in enumerate(o.iters):
        np.testing.assert_array_equal(it.bsize, g[f"bsize_{n}"])
        assert it.nkept == int(g[f"nkept_{n}"])
        np.testing.assert_array_equal(it.kept_bsize, g[f"kept_bsize_{n}"])
        np.testing.assert_allclose(it.en, g[f"en_{n}"], rtol=0, atol=1e-12 * max(1.0, np.abs(it.en).max()))
        np.testing.assert_allclose(it.thermo, g[f"thermo_{n}"], rtol=1e-12)
        np.testing.assert_allclose(it.opavg, g[f"opavg_{n}"], rtol=1e-12, atol=1e-14)
