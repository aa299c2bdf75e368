"""FP64-accurate tensor-core GEMM (nrg_dgemm_tc) against numpy's FP64 GEMM."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1, 1), (7, 13, 5), (64, 64, 64), (65, 63, 31), (200, 150, 400), (70, 90, 1100)]


def _mat(rng, r, c, kind):
    a = rng.standard_normal((r, c))
    if kind == "edge":  # maxima just below a power of two: top digit +64
        a = a / np.abs(a).max() * (2.0 - 1e-3)
    elif kind == "wide":  # entries spanning many binades
        a = a * np.exp2(rng.integers(-30, 3, size=(r, c)))
    elif kind == "sparse":
        a[rng.random((r, c)) < 0.7] = 0.0
    return a


@pytest.mark.parametrize("kind", ["normal", "edge", "wide", "sparse"])
@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True), (True, True)])
def test_dgemm_tc_matches_fp64(gpu_engine, kind, ta, tb):
    rng = np.random.default_rng(11)
    for M, N, K in SHAPES:
        A = _mat(rng, K if ta else M, M if ta else K, kind)
        B = _mat(rng, N if tb else K, K if tb else N, kind)
        C = gpu_engine.dgemm_tc(A, B, ta, tb)
        ref = (A.T if ta else A) @ (B.T if tb else B)
        tol = K * 2.0 ** -52 * max(np.abs(A).max(), 1e-300) * max(np.abs(B).max(), 1e-300)
        assert np.abs(C - ref).max() <= tol, (kind, ta, tb, M, N, K, np.abs(C - ref).max(), tol)


@pytest.mark.parametrize("alpha", [-1.0, -0.75, 3.0])
def test_dgemm_tc_alpha(gpu_engine, alpha):
    """Scaled and negated products (a negative alpha flips the sign bits of
    the A digit planes inside the kernel)."""
    rng = np.random.default_rng(5)
    for M, N, K in SHAPES:
        A = _mat(rng, M, K, "normal")
        B = _mat(rng, K, N, "wide")
        C = gpu_engine.dgemm_tc(A, B, False, False, alpha)
        ref = alpha * (A @ B)
        tol = abs(alpha) * K * 2.0 ** -52 * np.abs(A).max() * np.abs(B).max()
        assert np.abs(C - ref).max() <= tol, (alpha, M, N, K, np.abs(C - ref).max(), tol)
