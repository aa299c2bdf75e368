"""The block eigensolver through nrg_eigh_batched, both precision paths:
random, exactly degenerate and near-degenerate symmetric blocks across the
shared-memory and global-memory size ranges, against numpy's LAPACK syevd."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 3, 17, 64, 150, 233, 240, 300, 420]


def _blocks(seed=7):
    rng = np.random.default_rng(seed)
    mats = []
    for n in SIZES:
        a = rng.standard_normal((n, n))
        mats.append((a + a.T) * 0.5)
    # exact degeneracies: a 3-fold repeated spectrum in a random basis
    b = rng.standard_normal((40, 40))
    b = b + b.T
    q, _ = np.linalg.qr(rng.standard_normal((120, 120)))
    mats.append(q @ np.kron(np.eye(3), b) @ q.T)
    # near-degenerate pairs split by 1e-9 .. 1e-5
    d = np.sort(rng.uniform(-3, 3, 60))
    d = np.concatenate([d, d + np.logspace(-9, -5, 60)])
    q, _ = np.linalg.qr(rng.standard_normal((120, 120)))
    mats.append((q * d) @ q.T)
    return [0.5 * (m + m.T) for m in mats]


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_eigh_batched(gpu_engine, mixed_engine, mode):
    eng = gpu_engine if mode == "fp64" else mixed_engine
    mats = _blocks()
    out = eng.eigh_batched(mats)
    for h, (w, U) in zip(mats, out):
        n = h.shape[0]
        scale = max(1.0, np.abs(h).max())
        wr = np.linalg.eigvalsh(h)
        assert np.abs(w - wr).max() <= 1e-12 * scale * max(1, n) ** 0.5, (mode, n)
        assert np.all(np.diff(w) >= 0)
        assert np.abs(U.T @ U - np.eye(n)).max() <= 1e-12 * max(1, n) ** 0.5, (mode, n)
        assert np.abs(h @ U - U * w).max() <= 1e-11 * scale * max(1, n) ** 0.5, (mode, n)
