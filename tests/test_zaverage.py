"""The z-averaged / arbitrary-DOS Wilson-chain coefficient generator
(nrgplusplus_gb300.zaverage) against the coefficients the reference ships
(independFiles/zAverage/hoppingElementsL3.h5 and pseudoGap3.h5)."""
import numpy as np
import pytest

from conftest import golden

mpmath = pytest.importorskip("mpmath")
from nrgplusplus_gb300 import zaverage  # noqa: E402


def test_flat_band_against_reference():
    fx = golden("shipped_zaverage")
    tn = np.array(zaverage.flat_band_tn(1.0, 3.0))
    ref = fx["flat_tn_z1_L3"]
    assert tn.shape == ref.shape == (81,)
    # the 21 coefficients inside the 22-level Krylov space
    assert np.abs(tn[:21] - ref[:21]).max() < 1e-13
    # past it the recursion is the reference's own, value for value
    assert np.allclose(tn[21:], ref[21:], rtol=1e-6)


@pytest.mark.parametrize("r,key", [(1.0, "Pseudo"), (0.5, "Pseudo2")])
def test_pseudogap_against_reference(r, key):
    fx = golden("shipped_zaverage")
    tn, en = zaverage.dos_tn(zaverage.pseudogap_dos(r), 1.0, 3.0)
    assert np.abs(np.array(tn) - fx["tn" + key]).max() < 1e-13
    assert np.abs(np.array(en) - fx["en" + key]).max() < 1e-13


def test_flat_dos_limit_of_the_general_generator():
    """A flat density of states (1/2 on [-1, 1]) through the arbitrary-DOS
    generator: particle-hole symmetric (site energies 0), and the rescaled
    hoppings settle to a constant along the chain (the logarithmic mesh is
    self-similar), approached geometrically."""
    tn, en = zaverage.dos_tn(lambda x: mpmath.mpf(0.5) if abs(x) < 1 else mpmath.mpf(0), 1.0, 3.0, nitr=30)
    assert np.abs(en).max() < 1e-12
    d = np.abs(np.diff(tn))
    assert d[-1] < 1e-11 and d[-1] < d[-10] < d[-20]
