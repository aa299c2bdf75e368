"""The block eigensolver through nrg_eigh_batched, both precision paths:
random, exactly degenerate and near-degenerate symmetric blocks across the
shared-memory and global-memory size ranges, against numpy's LAPACK syevd."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 3, 17, 64, 150, 233, 240, 300, 420, 706, 1000]


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
    # a large block with a 2-fold degenerate spectrum and near-degenerate pairs
    d = np.sort(rng.uniform(-4, 4, 160))
    d = np.concatenate([d, d, d + np.logspace(-10, -4, 160)])
    q, _ = np.linalg.qr(rng.standard_normal((480, 480)))
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


@pytest.mark.parametrize("mode,n", [("fp64", 1500), ("mixed", 1500), ("mixed", 4300), ("fp64", 4300)])
def test_eigh_large_blocks(gpu_engine, mixed_engine, mode, n):
    """Blocks of the two-channel workload's size (up to ~4300 rows): the
    one-CTA reflector solver streaming the matrix from global memory, with
    its bisection and inverse iteration, in FP64 (no refinement) and FP32
    followed by the FP64-accurate refinement (one or two extra Newton steps
    above 1536 / 3072 rows, no FP64 re-solve); at 4300 rows the FP64
    back-transform runs on 4-column tiles."""
    eng = gpu_engine if mode == "fp64" else mixed_engine
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n))
    h = 0.5 * (a + a.T)
    # an NRG-like spectrum: a dense low part and exact pairs
    d = np.sort(rng.uniform(-2, 6, n // 2))
    d = np.concatenate([d, d[: n - n // 2]])
    q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    g = (q * d) @ q.T
    g = 0.5 * (g + g.T)
    before = eng.fallback_count()
    for m in (h, g):
        (w, U), = eng.eigh_batched([m])
        scale = max(1.0, np.abs(m).max())
        wr = np.linalg.eigvalsh(m)
        assert np.abs(w - wr).max() <= 1e-12 * scale * n ** 0.5, (mode, n)
        assert np.abs(U.T @ U - np.eye(n)).max() <= 1e-12 * n ** 0.5, (mode, n)
        assert np.abs(m @ U - U * w).max() <= 1e-11 * scale * n ** 0.5, (mode, n)
    # the mixed path refined these blocks itself (no FP64 re-solve)
    assert eng.fallback_count() == before, (mode, n)


@pytest.mark.parametrize("chain", [100, 300])
def test_long_near_degenerate_chain(mixed_engine, chain):
    """A chain of `chain` levels 1e-7 |H| apart (consecutive gaps inside the
    refinement's cluster threshold, far above its 64-level in-kernel limit)
    among well-separated levels: the long-cluster Rayleigh-Ritz pass
    diagonalises it in FP64, with no FP64 re-solve of the block."""
    rng = np.random.default_rng(chain)
    n = 600
    d = np.sort(rng.uniform(-5, 5, n - chain))
    d = np.concatenate([d, 1.234 + 1e-6 * np.arange(chain)])
    q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    m = (q * d) @ q.T
    m = 0.5 * (m + m.T)
    before = mixed_engine.fallback_count()
    (w, U), = mixed_engine.eigh_batched([m])
    wr = np.linalg.eigvalsh(m)
    scale = np.abs(m).max()
    assert np.abs(w - wr).max() <= 1e-12 * scale * n ** 0.5
    assert np.abs(U.T @ U - np.eye(n)).max() <= 1e-12 * n ** 0.5
    assert np.abs(m @ U - U * w).max() <= 1e-11 * scale * n ** 0.5
    assert mixed_engine.fallback_count() == before


@pytest.mark.parametrize("sizes", [[240, 300, 420], [480, 640], [706]])
def test_cluster_and_one_cta_solvers_agree(monkeypatch, sizes):
    """The thread-block-cluster solver (blocks above one SM's shared memory;
    8-CTA clusters below ~660 rows, 16 above) and the one-CTA solver give the
    same refined eigenpairs, launch after launch of different sizes."""
    from nrgplusplus_gb300 import api
    rng = np.random.default_rng(len(sizes))
    mats = []
    for n in sizes:
        a = rng.standard_normal((n, n))
        mats.append((a + a.T) * 0.5)
    out = {}
    for flag in ("2", "1", "0"):
        monkeypatch.setenv("NRG_EIG_CLUSTER", flag)
        eng = api.Engine(api.PREC_MIXED)
        eng.eigh_batched(mats)        # the largest launch first,
        eng.eigh_batched(mats[:1])    # a smaller one,
        out[flag] = eng.eigh_batched(mats)  # and the largest again
        eng.close()
    for h, (w2, U2), (w1, U1), (w0, U0) in zip(mats, out["2"], out["1"], out["0"]):
        n = h.shape[0]
        scale = max(1.0, np.abs(h).max())
        for w, U in ((w2, U2), (w1, U1)):
            assert np.abs(w - w0).max() <= 1e-12 * scale * n ** 0.5
            assert np.abs(h @ U - U * w).max() <= 1e-11 * scale * n ** 0.5


def test_autotuned_back_transform_is_bit_identical():
    """The autotuner times every reflector tile width on the first launch of
    a block-size histogram; whichever it keeps, the eigenpairs are the same
    bit for bit as with the autotuner off."""
    from nrgplusplus_gb300 import api
    mats = _blocks(5)[6:12]
    out = {}
    for on in (True, False):
        eng = api.Engine(api.PREC_MIXED)
        eng.set_autotune(on)
        out[on] = [eng.eigh_batched(mats), eng.eigh_batched(mats)]
        rep = eng.autotune_report()
        eng.close()
        if on:
            assert rep and "tw=" in rep[0]
        else:
            assert rep == []
    for a, b in zip(out[True][0] + out[True][1], out[False][0] + out[False][1]):
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
