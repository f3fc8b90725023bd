"""Host logic of bench.py that needs no device: the sweep estimate, the
parity summaries, the fixture loader and the traffic scaling."""
import copy

import numpy as np

import bench


def test_sweep_estimate():
    # measured iterations, then every later one at the last measured time
    assert bench.sweep_estimate([0.5, 1.0, 2.0, 10.0], 50) == 3.5 + 47 * 10.0
    assert bench.sweep_estimate([4.0], 1) == 4.0


def test_fixture_and_parity_summaries():
    ref = bench.load_fixture(bench.REF_FIXTURE)
    assert len(ref) == 5
    assert all(it.seconds is not None for it in ref)
    same = bench.sweep_errors(ref, ref)
    assert same["bookkeeping_exact"] and same["iterations"] == 5
    assert same["eigenvalues_rel_max"] == 0.0 and same["thermo_rel_max"] == 0.0
    moved = copy.deepcopy(ref)
    scale = max(1.0, float(np.abs(ref[3].en).max()))
    moved[3].en = ref[3].en + 1e-11 * scale
    moved[2].thermo = ref[2].thermo * (1.0 + 2e-9)
    e = bench.sweep_errors(moved, ref)
    assert abs(e["eigenvalues_rel_max"] - 1e-11) < 1e-13
    assert abs(e["thermo_rel_max"] - 2e-9) < 1e-12
    assert e["bookkeeping_exact"]
    moved[4].nkept += 1
    assert not bench.sweep_errors(moved, ref)["bookkeeping_exact"]


def test_traffic_scaling():
    # lower triangle read once (n^2/2 doubles) plus the measured writes
    assert abs(bench.TRIDIAG_DRAM_BYTES_PER_ELEMENT - 4.0 * (1.0 + 4.4 / 23.3)) < 1e-12

    class It:
        bsize = np.array([3, 4])

    class R:
        iters = [It(), It()]

    assert bench.sum_n2(R) == 2 * (9 + 16)
    assert bench.sum_n3(R) == 2 * (27 + 64)


def test_fd_error():
    an = np.array([1.0, 2.0, -3.0])
    fd = np.array([1.0, 2.0, -3.0 + 3e-6])
    assert abs(bench.fd_error(an, fd) - 1e-6) < 1e-12
    # derivatives that vanish: the error is taken against the floor
    assert abs(bench.fd_error(np.zeros(2), np.array([1e-9, -2e-9])) - 2e-6) < 1e-18
    assert bench.fd_error(np.zeros(2), np.array([1e-9, -2e-9]), 0.0) == 1.0


def test_tchi_on_a_temperature_grid():
    import twochnrg_gb300 as tg
    lam, betabar, n = 2.5, 0.727, 6
    its = []
    for N in range(n):
        DN = 0.5 * (1 + 1 / lam) * lam ** (-(N - 1) / 2.0)
        betas = betabar * lam ** ((np.arange(1, 5) - 4) / 8.0)
        th = np.zeros((4, 4))
        th[:, 0], th[:, 1] = betas, DN / betas
        th[:, 2] = 0.25 + 0.1 * np.log(th[:, 1])  # linear in ln T: interpolated exactly
        its.append(tg.Iteration(params=np.zeros(4), qn=np.zeros((0, 2)), bsize=np.zeros(0, np.int64),
                                en=np.zeros(0), emin=0.0, ecut=0.0, nkept=0, thermo=th, opavg=np.zeros(0),
                                kept_bsize=np.zeros(0, np.int64)))
    dth = np.zeros((n, 4, 4, 4))
    for k in range(4):
        dth[:, k, :, 2] = np.array([it.thermo[:, 2] for it in its]) * (k + 1)
    g = tg.GradResult(tg.SweepResult(iters=its), dth, np.zeros((n, 4, 0)), np.zeros((n, 4)), np.zeros(n),
                      np.zeros((n, 4)))
    T = np.array([it.thermo[:, 1] for it in its]).ravel()
    temps = np.array([T.min() / 2, T.min() * 1.3, np.sqrt(T.min() * T.max()), T.max() / 1.1, T.max() * 2])
    tchi, dt = g.tchi_on(temps)
    want = 0.25 + 0.1 * np.log(temps)
    assert np.isnan(tchi[0]) and np.isnan(tchi[-1]) and np.isnan(dt[:, 0]).all()
    np.testing.assert_allclose(tchi[1:-1], want[1:-1], rtol=1e-12)
    for k in range(4):
        np.testing.assert_allclose(dt[k, 1:-1], (k + 1) * want[1:-1], rtol=1e-12)
