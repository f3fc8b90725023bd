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
