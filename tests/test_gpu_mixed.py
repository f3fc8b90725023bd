"""The mixed-precision form (NRG_PREC_MIXED): large blocks reduced by the
blocked Householder panels with their trailing updates as split-BF16
products on the tensor cores.

The thresholds of the large-block paths are lowered through NRG_BIG_N and
NRG_MIXED_N so that these small workloads run through the blocked path.  Tolerances of the mixed form, as the
metric states them: block eigenvalues 1e-9 relative to the largest level of
the iteration; thermodynamics and operator averages 1e-8 relative; every
integer of the block bookkeeping exact.  Observed errors are ~1e-13.
"""
import os

import numpy as np
import pytest

import twochnrg_gb300 as tg
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
EIG_TOL = 1e-9
OBS_TOL = 1e-8


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
    return g, Ref


def compare(gpu, ref):
    assert len(gpu.iters) == len(ref.iters)
    worst = 0.0
    for n, (a, b) in enumerate(zip(gpu.iters, ref.iters)):
        np.testing.assert_array_equal(a.bsize, b.bsize, err_msg=f"N={n} block sizes")
        assert a.nkept == b.nkept, f"N={n} Nkept {a.nkept} != {b.nkept}"
        np.testing.assert_array_equal(a.kept_bsize, b.kept_bsize, err_msg=f"N={n} kept blocks")
        scale = max(1.0, float(np.max(np.abs(b.en))))
        err = float(np.max(np.abs(a.en - b.en))) / scale
        worst = max(worst, err)
        assert err < EIG_TOL, f"N={n} eigenvalue error {err:.3e}"
        np.testing.assert_allclose(a.thermo, b.thermo, rtol=OBS_TOL, atol=1e-14, err_msg=f"N={n} thermo")
        np.testing.assert_allclose(a.opavg, b.opavg, rtol=OBS_TOL, atol=1e-12, err_msg=f"N={n} <O>")
    return worst


@pytest.fixture
def blocked_everywhere(monkeypatch):
    # every block from 48 states on is a "large" block, and takes the blocked path
    monkeypatch.setenv("NRG_BIG_N", "48")
    monkeypatch.setenv("NRG_MIXED_N", "48")


@pytest.mark.parametrize("name", ["cfg1_2chQS_n8_k300", "cfg0_1chQS_n40_k500", "qsz_1chQSz_n14_k300"])
def test_mixed_matches_reference_fixture(engine, blocked_everywhere, name):
    g, ref = _fixture(name)
    model, ns, nc, lam, U, ed, g1, x = g["config"][:8]
    r = engine.sweep(str(model), int(ns), int(nc), float(lam), float(U), float(ed), float(g1), float(x),
                     precision=tg.PREC_MIXED)
    compare(r, ref)


@pytest.mark.parametrize("split", ["1", "4"])
def test_mixed_matches_oracle_two_channel(engine, blocked_everywhere, monkeypatch, split):
    # one grid, and four concurrent grids of a quarter of the SMs each
    monkeypatch.setenv("NRG_GRID_SPLIT", split)
    case = ("2chQS", 5, 200, 2.5, 0.3, -0.15, 0.01, 0.01)
    r = engine.sweep(*case, precision=tg.PREC_MIXED)
    o = orc.run(*case, nthreads=min(8, os.cpu_count() or 1))
    compare(r, o)


def test_mixed_default_threshold_agrees_with_fp64(engine):
    # the default threshold on a sweep whose largest blocks pass it
    case = ("2chQS", 4, 3000, 2.5, 0.3, -0.15, 0.01, 0.01)
    a = engine.sweep(*case)
    b = engine.sweep(*case, precision=tg.PREC_MIXED)
    assert max(int(it.bsize.max()) for it in a.iters) >= 4200
    compare(b, a)
