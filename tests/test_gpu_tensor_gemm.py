"""The FP64-accurate tensor-core product (nrg_gemm_f64_tensor), the building
block of the mixed-precision form, against numpy's FP64 product.

Error model, relative to |A_i| |B_j| (|A_i| the largest magnitude in row
i): the slice pairs past level S-1 are dropped (S - 1 pairs of terms below
2^-8S each) and the fourth accumulator (levels 3 and up) rounds in FP32 at
about 2^-39 per addition; both add up over k terms with random signs, to
about 2^-35 sqrt(k/64) for 5 slices and 2^-36 for 6.  The tests check
2^-32 sqrt(k/64) (5 slices) and 2^-34 sqrt(k/64) (6 slices) plus FP64
rounding of the result.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bound(A, B, S):
    k = A.shape[1]
    ra = np.abs(A).max(axis=1)
    rb = np.abs(B).max(axis=1)
    return np.outer(ra, rb) * 2.0 ** (-32 if S == 5 else -34) * np.sqrt(max(k, 64) / 64)


@pytest.mark.parametrize("m,n,k", [(128, 128, 64), (200, 77, 100), (300, 300, 16), (1, 5, 3), (257, 129, 256)])
def test_products(engine, m, n, k):
    rng = np.random.default_rng(m * 1000 + n + k)
    # rows of very different magnitudes, as Householder vectors and w have
    A = rng.standard_normal((m, k)) * np.exp(rng.uniform(-20, 5, size=(m, 1)))
    B = rng.standard_normal((n, k)) * np.exp(rng.uniform(-20, 5, size=(n, 1)))
    C = rng.standard_normal((m, n))
    for S in (5, 6):
        out = engine.gemm_f64_tensor(A, B, C, alpha=-1.0, slices=S)
        ref = C - A @ B.T
        err = np.abs(out - ref)
        assert np.all(err <= _bound(A, B, S) + 4 * np.finfo(float).eps * np.abs(ref)), (S, err.max())


def test_zero_rows_and_exact_integers(engine):
    # integer operands below 2^7 are exact in the first slice: the result is exact
    rng = np.random.default_rng(7)
    A = rng.integers(-100, 100, size=(150, 64)).astype(float)
    B = rng.integers(-100, 100, size=(140, 64)).astype(float)
    A[3] = 0.0
    B[10] = 0.0
    out = engine.gemm_f64_tensor(A, B, np.zeros((150, 140)), alpha=1.0, slices=5)
    assert np.array_equal(out, A @ B.T)


def test_two_calls_in_a_row_agree(engine):
    rng = np.random.default_rng(11)
    A = rng.standard_normal((384, 128))
    B = rng.standard_normal((256, 128))
    C = rng.standard_normal((384, 256))
    a = engine.gemm_f64_tensor(A, B, C, alpha=0.5)
    b = engine.gemm_f64_tensor(A, B, C, alpha=0.5)
    assert np.array_equal(a, b)
