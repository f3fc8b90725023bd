"""Drop-in DiagBlock replacement (nrg_diag_blocks) against LAPACK dspev as the
reference calls it, on random blocks and on real NRG blocks.

Tolerances: eigenvalues 1e-12 relative to the block norm; eigenvectors by
residual and orthogonality (1e-12), and against dspev's up to sign where the
level is isolated.
"""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _check_block(A, w, Z, wr, Zr):
    nrm = max(1.0, float(np.max(np.abs(wr))))
    assert np.max(np.abs(w - wr)) / nrm < 1e-12
    n = A.shape[0]
    R = A @ Z.T - Z.T * w
    assert np.max(np.abs(R)) / nrm < 1e-12
    assert np.max(np.abs(Z @ Z.T - np.eye(n))) < 1e-12
    gaps = np.diff(wr)
    for k in range(n):
        iso = (k == 0 or gaps[k - 1] > 1e-6 * nrm) and (k == n - 1 or gaps[k] > 1e-6 * nrm)
        if iso:
            s = np.sign(Z[k] @ Zr[k])
            assert np.max(np.abs(s * Z[k] - Zr[k])) < 1e-9


def test_random_blocks(engine):
    rng = np.random.default_rng(7)
    sizes = [1, 2, 3, 17, 64, 130, 333]
    mats = []
    for n in sizes:
        X = rng.standard_normal((n, n))
        A = 0.5 * (X + X.T)
        if n > 20:  # planted exact degeneracy
            A[:3, :] = 0.0; A[:, :3] = 0.0
            A[0, 0] = A[1, 1] = A[2, 2] = 0.25
        mats.append(A)
    packed = np.concatenate([orc.pack_upper(A) for A in mats])
    ws, Zs = engine.diag_blocks(sizes, packed)
    for A, w, Z in zip(mats, ws, Zs):
        wr, Zr = orc.diag_block(orc.pack_upper(A), A.shape[0])
        _check_block(A, w, Z, wr, Zr)


def test_zero_and_diagonal_blocks(engine):
    """Blocks whose tridiagonal splits everywhere: the zero matrix (all
    levels 0, eigenvectors the identity, as dspev returns them) and a diagonal
    one with a repeated level."""
    Z0 = np.zeros((6, 6))
    D = np.diag([0.5, -1.0, 0.5, 2.0, 0.5])
    ws, Zs = engine.diag_blocks([6, 5], np.concatenate([orc.pack_upper(Z0), orc.pack_upper(D)]))
    assert not ws[0].any()
    np.testing.assert_array_equal(Zs[0], np.eye(6))
    wr, Zr = orc.diag_block(orc.pack_upper(D), 5)
    _check_block(D, ws[1], Zs[1], wr, Zr)


def test_large_block_whole_gpu_path(engine, monkeypatch):
    rng = np.random.default_rng(11)
    n = 1300
    monkeypatch.setenv("NRG_BIG_N", "1000")  # route the block to the cooperative-grid kernel
    X = rng.standard_normal((n, n))
    A = (X + X.T) / np.sqrt(n)
    ws, Zs = engine.diag_blocks([n], orc.pack_upper(A))
    wr, Zr = orc.diag_block(orc.pack_upper(A), n)
    _check_block(A, ws[0], Zs[0], wr, Zr)


@pytest.mark.parametrize("path", ["grid", "cluster256"])
def test_lower_triangle_kernels_on_ragged_sizes(engine, monkeypatch, path):
    """Both Householder kernels work on the lower triangle in tiles of 8 rows
    by 32 columns: sizes around the tile edges (2 and 3: no full step; 8, 9,
    31 to 34, 65) through the whole-grid kernel (threshold lowered to 2) and
    through the cluster kernel's 256-thread form."""
    rng = np.random.default_rng(21)
    if path == "grid":
        monkeypatch.setenv("NRG_BIG_N", "2")
    else:
        monkeypatch.setenv("NRG_CLUSTER_THREADS", path[len("cluster"):])
        monkeypatch.setenv("NRG_CLUSTER", "4")
    sizes = [2, 3, 8, 9, 31, 32, 33, 34, 65, 257]
    mats = []
    for n in sizes:
        X = rng.standard_normal((n, n))
        mats.append((X + X.T) / np.sqrt(n))
    ws, Zs = engine.diag_blocks(sizes, np.concatenate([orc.pack_upper(A) for A in mats]))
    for A, w, Z in zip(mats, ws, Zs):
        wr, Zr = orc.diag_block(orc.pack_upper(A), A.shape[0])
        _check_block(A, w, Z, wr, Zr)


@pytest.mark.parametrize("split", ["1", "2", "3"])
def test_concurrent_grids_path(engine, monkeypatch, split):
    """Several large blocks dealt to concurrent cooperative grids, next to
    small blocks on the cluster kernel."""
    rng = np.random.default_rng(12)
    monkeypatch.setenv("NRG_BIG_N", "1000")
    monkeypatch.setenv("NRG_GRID_SPLIT", split)
    sizes = [1100, 300, 1250, 1020, 64]
    mats = []
    for n in sizes:
        X = rng.standard_normal((n, n))
        mats.append((X + X.T) / np.sqrt(n))
    ws, Zs = engine.diag_blocks(sizes, np.concatenate([orc.pack_upper(A) for A in mats]))
    for A, w, Z in zip(mats, ws, Zs):
        wr, Zr = orc.diag_block(orc.pack_upper(A), A.shape[0])
        _check_block(A, w, Z, wr, Zr)


def test_nrg_blocks_from_a_real_iteration(engine):
    """The H_N blocks the reference assembles (two-channel, N=2) diagonalized
    through the drop-in must give the oracle's levels (before SetE0zero)."""
    s = orc.run("2chQS", 3, 120, 2.5, 0.3, -0.15, 0.01, 0.01, capture_iter=2)
    it = s.iters[2]
    ws, _ = engine.diag_blocks(it.bsize, it.H)
    w = np.concatenate(ws) - it.emin
    # the oracle's levels went through SetDegen (MyEPS = 1e-18): compare to 1e-12
    assert np.max(np.abs(w - it.en)) < 1e-12 * max(1.0, float(np.max(np.abs(it.en))))
