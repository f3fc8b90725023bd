"""Parity of the GB300 sweep (C ABI, device kernels) against the CPU oracle
and the reference's golden fixtures.

Tolerances: block eigenvalues 1e-10 relative to the largest level of the
iteration; thermodynamics and operator averages 1e-8 relative (averages with
an absolute floor of 1e-12); every integer
of the block bookkeeping (sectors, sizes, kept counts, kept blocks) exact.
"""
import os

import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
EIG_TOL = 1e-10
OBS_TOL = 1e-8


def compare(gpu, ref, model=""):
    assert len(gpu.iters) == len(ref.iters)
    for n, (a, b) in enumerate(zip(gpu.iters, ref.iters)):
        # one-quantum-number blocks: the engine reports |Q> as (Q, 0) and |S>,
        # |Sz> as (0, S), (0, Sz), the reference the one number
        nq = b.qn.shape[1]
        qa = a.qn[:, ::-1] if model in ("1chS", "1chSz") else a.qn
        np.testing.assert_array_equal(qa[:, :nq], b.qn, err_msg=f"N={n} sectors")
        assert not qa[:, nq:].any()
        np.testing.assert_array_equal(a.bsize, b.bsize, err_msg=f"N={n} block sizes")
        assert a.nkept == b.nkept, f"N={n} Nkept {a.nkept} != {b.nkept}"
        np.testing.assert_array_equal(a.kept_bsize, b.kept_bsize, err_msg=f"N={n} kept blocks")
        scale = max(1.0, float(np.max(np.abs(b.en))))
        err = float(np.max(np.abs(a.en - b.en))) / scale
        assert err < EIG_TOL, f"N={n} eigenvalue error {err:.3e}"
        assert abs(a.ecut - b.ecut) / scale < EIG_TOL
        np.testing.assert_allclose(a.thermo, b.thermo, rtol=OBS_TOL, atol=1e-14, err_msg=f"N={n} thermo")
        # absolute floor 1e-12: <S_z> in the |Q> basis vanishes by symmetry and
        # is round-off (~1e-14) in both implementations
        np.testing.assert_allclose(a.opavg, b.opavg, rtol=OBS_TOL, atol=1e-12, err_msg=f"N={n} <O>")


CASES = [
    ("1chQS", 12, 150, 2.5, 0.5, -0.25, 0.02, 0.0),
    ("1chQSz", 10, 200, 2.5, 0.5, -0.25, 0.02, 1e-3),
    ("2chQS", 5, 80, 2.5, 0.3, -0.15, 0.01, 0.01),
    ("2chQS", 4, 40, 2.5, 0.3, -0.15, 0.01, 0.02),
    ("1chQ", 12, 150, 2.5, 0.4, -0.2, 0.015, 0.0),
    ("1chS", 12, 150, 2.5, 0.4, -0.2, 0.015, 0.0, 0.02),
    ("1chSz", 10, 200, 2.5, 0.4, -0.2, 0.015, 1e-4, 0.02),
]


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-n{c[1]}-k{c[2]}" for c in CASES])
def test_sweep_matches_oracle(engine, case):
    delta = case[8] if len(case) > 8 else 0.0  # superconducting leads' gap
    g = engine.sweep(*case[:8], delta_sc=delta)
    o = orc.run(*case[:8], nthreads=min(8, os.cpu_count() or 1), delta_sc=delta)
    compare(g, o, case[0])
    np.testing.assert_allclose(g.opavg_m1, o.opavg_m1, rtol=1e-15)


@pytest.mark.parametrize("name", ["cfg0_1chQS_n40_k500", "qsz_1chQSz_n14_k300", "cfg1_2chQS_n8_k300",
                                  "q_1chQ_n12_k200", "s_1chS_n12_k200", "sz_1chSz_n12_k200"])
def test_sweep_matches_reference_fixture(engine, name):
    g = np.load(os.path.join(GOLD, name + ".npz"))
    model, ns, nc, lam, U, ed, g1, x = g["config"][:8]
    delta = float(g["config"][8]) if len(g["config"]) > 8 else 0.0
    r = engine.sweep(model, int(ns), int(nc), float(lam), float(U), float(ed), float(g1), float(x), delta_sc=delta)

    class Ref:  # fixture in the oracle's shape
        iters = []

    for n in range(int(g["niters"])):
        class It:
            pass
        it = It()
        it.qn, it.bsize, it.en = g[f"qn_{n}"], g[f"bsize_{n}"], g[f"en_{n}"]
        it.nkept, it.ecut = int(g[f"nkept_{n}"]), float(g[f"ecut_{n}"])
        it.kept_bsize, it.thermo, it.opavg = g[f"kept_bsize_{n}"], g[f"thermo_{n}"], g[f"opavg_{n}"]
        Ref.iters.append(it)
    compare(r, Ref, str(model))


def test_kernels_launched(engine):
    before = engine.kernel_count
    engine.sweep("1chQS", 3, 50, 2.5, 0.5, -0.25, 0.02)
    assert engine.kernel_count > before
