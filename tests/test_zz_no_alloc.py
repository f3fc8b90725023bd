"""nrg_diag_block_noalloc: the block eigensolver for callers that cannot
allocate device memory when they need a block diagonalized.

The test allocates the caller's device buffers itself (through the CUDA
runtime the library links), calls the no-allocation entry point twice in a
row through the C ABI and checks each result against the allocating drop-in
nrg_diag_blocks on the same matrix, with the tolerances of the other
eigensolver tests: eigenvalues 1e-12 relative to the block norm; eigenvectors
by residual and orthogonality (1e-12) and, for isolated levels, against the
allocating entry point's vectors up to sign (1e-9).  This file is collected
last so that a failure here leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

import twochnrg_gb300 as tg
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

NRG_OK, NRG_ERR_SIZE = 0, 5
MAX_N = 256  # NRG_NOALLOC_MAX_N


def _runtime():
    L = tg.load_library()
    L.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
    L.cudaFree.argtypes = [ctypes.c_void_p]
    L.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    L.cudaDeviceSynchronize.argtypes = []
    L.nrg_diag_block_noalloc.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p]
    return L


def _dmalloc(L, nbytes):
    p = ctypes.c_void_p()
    assert L.cudaMalloc(ctypes.byref(p), nbytes) == 0
    return p


def _matrix(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, n))
    A = 0.5 * (X + X.T)
    if n >= 8:  # an exactly degenerate pair, as SU(2)-related levels give
        A[:2, :] = 0.0
        A[:, :2] = 0.0
        A[0, 0] = A[1, 1] = 0.3
    return A


def _check(A, w, Z, wr, Zr):
    n = A.shape[0]
    nrm = max(1.0, float(np.max(np.abs(wr))))
    assert np.max(np.abs(w - wr)) / nrm < 1e-12
    assert np.max(np.abs(A @ Z.T - Z.T * w)) / nrm < 1e-12
    assert np.max(np.abs(Z @ Z.T - np.eye(n))) < 1e-12
    gaps = np.diff(wr)
    for k in range(n):
        if (k == 0 or gaps[k - 1] > 1e-6 * nrm) and (k == n - 1 or gaps[k] > 1e-6 * nrm):
            s = np.sign(Z[k] @ Zr[k])
            assert np.max(np.abs(s * Z[k] - Zr[k])) < 1e-9


@pytest.mark.parametrize("n", [1, 37, 200, MAX_N])
def test_noalloc_matches_allocating_entry_point(engine, n):
    L = _runtime()
    A = np.ascontiguousarray(_matrix(n, 100 + n))
    ws, Zs = engine.diag_blocks([n], orc.pack_upper(A))
    dA = _dmalloc(L, A.nbytes)
    dW = _dmalloc(L, 8 * n)
    dZ = _dmalloc(L, 8 * n * n)
    try:
        assert L.cudaMemcpy(dA, A.ctypes.data, A.nbytes, 1) == 0  # host -> device
        for _ in range(2):  # the second call reuses the scratch the first one left behind
            st = L.nrg_diag_block_noalloc(n, dA, dW, dZ, None)
            assert st == NRG_OK, f"status {st}"
            w = np.empty(n)
            Z = np.empty((n, n))
            assert L.cudaMemcpy(w.ctypes.data, dW, 8 * n, 2) == 0  # device -> host
            assert L.cudaMemcpy(Z.ctypes.data, dZ, 8 * n * n, 2) == 0
            _check(A, w, Z, ws[0], Zs[0])
        back = np.empty_like(A)
        assert L.cudaMemcpy(back.ctypes.data, dA, A.nbytes, 2) == 0
        assert np.array_equal(back, A)  # the input is left untouched
    finally:
        for p in (dA, dW, dZ):
            L.cudaFree(p)


def test_noalloc_rejects_blocks_above_the_limit():
    L = _runtime()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    assert L.nrg_diag_block_noalloc(MAX_N + 1, dummy, dummy, dummy, None) == NRG_ERR_SIZE
