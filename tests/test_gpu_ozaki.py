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


def _split_model(A):
    """The value the digit split keeps of A: with e = ilogb(max|A|) + 1,
    rint(A 2^(55-e)) 2^(e-55), ties to even (numpy's rint)."""
    mx = np.abs(A).max()
    e = 0 if mx == 0 else int(np.frexp(mx)[1])
    return np.ldexp(np.rint(np.ldexp(A, 55 - e)), e - 55)


def test_split_rounding_is_exact(gpu_engine):
    """A @ (2^s I) keeps every digit of A (B's only digit is its top one), so
    the product shows the split of A bit for bit: ties to even, negative
    ties, entries below half a unit, and subnormal entries of a subnormal
    block (B scaled so that the product is a normal number)."""
    rng = np.random.default_rng(3)
    n = 24
    ulp = 2.0 ** -55  # half a unit of A 2^54 (max 1.5, so e = 1)
    A = rng.uniform(-1.0, 1.0, (n, n))
    A[0, 0] = 1.5
    A[0, 1:9] = np.array([3, 5, -3, -5, 7, 1, -1, 9]) * ulp  # exact ties
    A[1, 1:5] = [ulp * 0.5, -ulp * 0.49, ulp * 1.0000001, 2.0 ** -1074]
    A[2, :] = 0.0
    for a, s in [(A, 0), (A * 2.0 ** -1062, 1000), (rng.standard_normal((n, n)) * 2.0 ** -1070, 1000)]:
        B = np.eye(n) * 2.0 ** s
        C = gpu_engine.dgemm_tc(a, B, False, False)
        want = _split_model(a) * 2.0 ** s
        assert np.array_equal(C, want), np.abs(C - want).max()


def test_split_non_finite_block_poisons_the_product(gpu_engine):
    """An Inf or NaN operand makes the whole product non-finite (the
    refinement's convergence check then hands the block to FP64)."""
    rng = np.random.default_rng(4)
    for bad in (np.inf, -np.inf, np.nan):
        A = rng.standard_normal((40, 30))
        A[7, 3] = bad
        C = gpu_engine.dgemm_tc(A, rng.standard_normal((30, 20)), False, False)
        assert not np.isfinite(C).any()
